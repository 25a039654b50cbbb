// Transform.hpp -- scale then translate (include/Transform.hpp of the reference).
// The library traces world-space triangles, so a transform is applied to the
// mesh's points when a Renderer takes the scene.
#pragma once

#include "Utils.hpp"

struct Transform
{
    Vec3 s = Vec3{1, 1, 1};
    Vec3 p = Vec3{0, 0, 0};

    constexpr Ray applyInverse(const Ray &ray_in_world) const
    {
        const Vec3 inv_s = s.inv();
        return Ray{(ray_in_world.p - p) * inv_s, ray_in_world.v * inv_s};
    }
    constexpr Vec3 applyToPoint(const Vec3 &point) const { return point * s + p; }
};
