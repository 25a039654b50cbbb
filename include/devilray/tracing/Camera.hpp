#pragma once

#include "Utils.hpp"
#include "models/Matrix.hpp"

struct Intrinsics
{
    float focal_length;
    Vec2f center;
};

// Pinhole camera (include/tracing/Camera.hpp): camera-to-world transform,
// intrinsics in sensor units, resolution and physical pixel size.
struct Camera
{
    mutable Matrix4x4f transform;

    Intrinsics intrinsics;
    Size2i resolution;
    Size2f physical_pixel_size;
};
