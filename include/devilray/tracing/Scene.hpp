// Scene.hpp -- objects, materials and mesh storage (include/tracing/Scene.hpp of
// the reference). A value type moved into a Renderer; `mesh_storage` keeps the
// GpuTris the object views point into.
#pragma once

#include "device/Vector.hpp"
#include "tracing/GpuTris.hpp"
#include "tracing/Material.hpp"
#include "tracing/TriangleMesh.hpp"

#include <list>

struct ObjectsInfo
{
    float total_radiant_power;
};

struct Scene
{
    // The device form of a scene is the dr_scene a Renderer builds from it;
    // these keep the reference's calls and only manage the host vectors'
    // device copies.
    void deleteDeviceMemory()
    {
        materials.deleteDeviceMemory();
        objects.deleteDeviceMemory();
    }
    void ensureDeviceAllocation() {}

    ObjectsInfo info{};

    DeviceVector<TriangleMesh> objects{{}};
    DeviceVector<Material> materials{{}};

    std::list<GpuTris> mesh_storage;
};
