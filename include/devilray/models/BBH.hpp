// BBH.hpp -- bounding-box hierarchy types of the reference
// (include/models/BBH.hpp). The traversal hierarchy of this library is built by
// dr_scene_create over the whole scene (binned SAH, 2- or 8-wide, on the
// library's own layout); the per-mesh BBH of a GpuTris holds the mesh's root
// box only, one leaf over all its triangles.
#pragma once

#include "device/Vector.hpp"
#include "models/Mesh.hpp"
#include "Utils.hpp"

#include <span>

struct BBHNode
{
    AABB box;
    int left_child = -1;
    int right_child = -1;
    int parent_index = -1;

    int tris_begin;
    int tris_end;

    constexpr bool isLeaf() const { return left_child == -1 && right_child == -1; }
};

struct BBH
{
    int depth;
    DeviceVector<BBHNode> nodes;
};

struct BBHGpuView
{
    std::span<const BBHNode> nodes;

    constexpr bool isEmpty() const { return nodes.size() == 0; }
};

inline BBHGpuView createBBHGpuView(BBH &bbh) { return BBHGpuView{std::span<const BBHNode>{bbh.nodes.hostPtr(), bbh.nodes.size()}}; }
