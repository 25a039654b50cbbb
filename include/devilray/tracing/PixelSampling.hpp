#pragma once

// Sub-pixel position of a camera ray (include/tracing/PixelSampling.hpp);
// values equal dr_pixel_sampling.
enum class PixelSampling : int {
    Center = 0,
    UniformRandom = 1,
};
