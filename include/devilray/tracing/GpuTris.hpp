// GpuTris.hpp -- mesh storage of a scene (include/tracing/GpuTris.hpp of the
// reference). Unlike the reference, convertMeshToTris leaves the mesh's
// triangle order unchanged (the library's hierarchy is built per scene), so the
// triangle sampler pairs with the stored triangles as built.
#pragma once

#include "device/Vector.hpp"
#include "models/BBH.hpp"
#include "models/Mesh.hpp"
#include "tracing/DistributionSamplers.hpp"
#include "tracing/Material.hpp"
#include "tracing/TriangleMesh.hpp"
#include "Utils.hpp"

struct GpuTris
{
    DeviceVector<Vec3> points;
    DeviceVector<Vec3> normals;
    DeviceVector<Triangle> triangles;

    AliasTable triangle_sampler;

    BBH bbh;
};

// Copies the mesh; the triangle sampler is the alias table of the triangle
// areas (when requested); bbh holds the mesh's root box.
GpuTris convertMeshToTris(Mesh &mesh, bool generateTriangleSampler = true);
// Square of side `size` centred at `center`, facing `normal`, `right` along
// one edge; two triangles (0, 2, 1), (0, 3, 2).
GpuTris createQuadMesh(Vec3 center, Vec3 normal, Vec3 right, float size);
// A view with an identity transform, material 0 and the mesh's total area.
TriangleMesh viewGpuTris(GpuTris &tris);
