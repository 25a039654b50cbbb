// TriangleMesh.hpp -- a placed view of a GpuTris (include/tracing/TriangleMesh.hpp
// of the reference). The pointers name the GpuTris' HOST arrays: a Renderer
// flattens the views of its scene into one world-space triangle soup for the
// device when it takes the scene.
#pragma once

#include "models/BBH.hpp"
#include "models/Mesh.hpp"
#include "tracing/DistributionSamplers.hpp"
#include "Transform.hpp"
#include "Utils.hpp"

struct TriangleMesh
{
    Vec3 *points;
    Vec3 *normals;
    Triangle *triangles;
    int triangle_count;

    Transform model_to_world;
    int material;

    AliasEntry *triangle_sampler;
    float surface_area;
    float base_surface_area;

    BBHGpuView bbh;

    void setPosition(const Vec3 &pos) { model_to_world.p = pos; }
    // Scales the light-power area by (sx sy sz)^(2/3).
    void setScale(const Vec3 &scale)
    {
        model_to_world.s = scale;
        const float vol = scale.x * scale.y * scale.z;
        surface_area = base_surface_area * std::cbrt(vol * vol);
    }
};
