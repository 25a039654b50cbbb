// oracle_scene.hpp -- the oracle's flattened scene (TEST INFRASTRUCTURE):
// shared by the FP32 integrator (oracle_render.cpp) and its FP64 restatement
// (oracle_render_f64.cpp).
#pragma once

#include "oracle.h"

#include <memory>
#include <vector>

namespace oracle {

struct V4 {
    float x, y, z, w;
};

struct Mat {
    int kind;
    float ior;
    V4 emission, albedo, debug;
};

struct BbhDel {
    void operator()(or_bbh *p) const { or_bbh_destroy(p); }
};
using BbhPtr = std::unique_ptr<or_bbh, BbhDel>;

}  // namespace oracle

struct or_scene {
    std::vector<float> pos;                 // 9 floats per triangle
    std::vector<or_object> objects;
    std::vector<int32_t> tri_object;        // triangle -> object
    std::vector<oracle::Mat> mats;
    std::vector<int32_t> tri_material;      // triangle -> material (object's unless overridden)
    // light sampling
    std::vector<or_alias_entry> light_table;
    float total_power = 0.0f;
    // per-object triangle tables, two index orders
    std::vector<or_alias_entry> tri_table[2];
    std::vector<int32_t> tri_table_map[2];  // [order][tri_begin + i] -> soup triangle
    // closest hit structures
    oracle::BbhPtr soup_bbh;
    std::vector<oracle::BbhPtr> obj_bbh;
    std::vector<std::vector<int32_t>> obj_order;  // per object: sorted position -> soup triangle
    float slack = 0.0f;
};
