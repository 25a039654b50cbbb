// GpuTris.cpp -- mesh storage and views (src/GpuTris.cpp of the reference).
#include "tracing/GpuTris.hpp"

#include <vector>

namespace {

float totalSurfaceArea(const GpuTris &tris)
{
    double total = 0;  // float areas summed in double, as the reference
    const Vec3 *p = tris.points.hostPtr();
    for (size_t i = 0; i < tris.triangles.size(); ++i) {
        const Triangle &t = tris.triangles[i];
        total += triangleArea(p[t.a.pi], p[t.b.pi], p[t.c.pi]);
    }
    return static_cast<float>(total);
}

BBH rootBox(const Mesh &mesh)
{
    AABB box = AABB::empty();
    for (const Vec3 &q : mesh.points) box = box.extend(q);
    std::vector<BBHNode> nodes;
    BBHNode root{};
    root.box = box;
    root.tris_begin = 0;
    root.tris_end = (int)mesh.triangles.size();
    nodes.push_back(root);
    return BBH{0, DeviceVector<BBHNode>(std::move(nodes))};
}

}  // namespace

GpuTris convertMeshToTris(Mesh &mesh, bool generateTriangleSampler)
{
    AliasTable sampler;
    if (generateTriangleSampler) {
        std::vector<float> areas;
        areas.reserve(mesh.triangles.size());
        for (const Triangle &t : mesh.triangles)
            areas.push_back(triangleArea(mesh.points[t.a.pi], mesh.points[t.b.pi], mesh.points[t.c.pi]));
        sampler = generateAliasTable(areas);
    }
    BBH bbh = rootBox(mesh);
    return GpuTris{DeviceVector<Vec3>(mesh.points), DeviceVector<Vec3>(mesh.normals),
                   DeviceVector<Triangle>(mesh.triangles), std::move(sampler), std::move(bbh)};
}

TriangleMesh viewGpuTris(GpuTris &tris)
{
    TriangleMesh obj{};
    obj.points = tris.points.hostPtr();
    obj.normals = tris.normals.hostPtr();
    obj.triangles = tris.triangles.hostPtr();
    obj.triangle_sampler = tris.triangle_sampler.entries.hostPtr();
    obj.bbh = createBBHGpuView(tris.bbh);
    obj.triangle_count = (int)tris.triangles.size();
    obj.model_to_world = Transform{};
    obj.material = 0;
    obj.base_surface_area = totalSurfaceArea(tris);
    obj.surface_area = obj.base_surface_area;
    return obj;
}

GpuTris createQuadMesh(Vec3 center, Vec3 normal, Vec3 right, float size)
{
    const Vec3 up = right.cross(normal);
    const float half = size / 2.0f;
    Mesh mesh;
    mesh.name = "quad";
    mesh.points = {
        center + right * (-half) + up * (-half),
        center + right * (half) + up * (-half),
        center + right * (half) + up * (half),
        center + right * (-half) + up * (half),
    };
    mesh.normals = {normal};
    mesh.triangles = {
        Triangle{{0, 0}, {2, 0}, {1, 0}},
        Triangle{{0, 0}, {3, 0}, {2, 0}},
    };
    return convertMeshToTris(mesh);
}
