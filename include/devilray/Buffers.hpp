// Buffers.hpp -- accumulation buffers of a Renderer (include/Buffers.hpp of the
// reference): per pixel the colour sum with the sample count in w, and the
// path-ray casts.
#pragma once

#include "device/Array.hpp"
#include "Utils.hpp"

#include <cstdint>

struct Buffers
{
    explicit Buffers(Size2i resolution);

    // Zeroes host and device copies (the device side with one asynchronous fill).
    void reset();
    void ensureDeviceAllocation();

    // Sum of the host copy of `casts` (call casts.updateHostData() first).
    uint64_t totalCasts() const;

    static constexpr int maxPathLength = 10;

    DeviceArray<Vec4> color;
    mutable DeviceArray<uint32_t> casts;
};
