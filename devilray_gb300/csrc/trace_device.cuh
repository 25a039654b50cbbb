// trace_device.cuh -- per-ray closest-hit and any-hit traversal (device
// functions shared by the public trace kernels and the renderer's wavefront).
//
// Stack traversal of the two-box BVH: nearer child first, conservative culling
// (widened boxes, enter <= best), leaf scan with the reference or watertight
// triangle test; a candidate wins on smaller t, or equal t with a smaller
// original triangle index, so the result equals a brute-force scan.
#pragma once

#include "trace_kernels.cuh"
#include "tri_device.cuh"
#include "trace_wide.cuh"

#include <climits>

namespace dr {

struct TraceStats {
    unsigned long long nodes = 0, boxes = 0, tris = 0;
};

template <int MODE, bool COUNT>
__device__ __forceinline__ void closest_hit(const TraceArgs &a, const DevRay &r, uint32_t root, float &best_t,
                                            int32_t &best_prim, TraceStats &st)
{
    best_t = r.tmax;
    best_prim = INT_MAX;
    if (root == kNoRoot) return;
    WtSetup w;
    if (MODE == 1) w = wt_setup(r.v);
    int32_t stack[kStackSize];
    int sp = 0;
    int32_t cur = (int32_t)root;
    while (true) {
        if (cur >= 0) {
            const float4 *np = reinterpret_cast<const float4 *>(a.nodes + cur);
            const float4 c0xy = __ldg(np), c1xy = __ldg(np + 1), cz = __ldg(np + 2);
            const int4 link = __ldg(reinterpret_cast<const int4 *>(np + 3));
            float t0, t1;
            bool h0, h1;
            intersect_children(c0xy, c1xy, cz, r, best_t, t0, t1, h0, h1);
            if (COUNT) {
                ++st.nodes;
                st.boxes += 2;
            }
            if (h0 && h1) {
                const bool swap = t1 < t0;
                if (sp >= kStackSize) {
                    atomicOr(a.error, ERR_STACK_OVERFLOW);
                    return;
                }
                stack[sp++] = swap ? link.x : link.y;
                cur = swap ? link.y : link.x;
            } else if (h0) {
                cur = link.x;
            } else if (h1) {
                cur = link.y;
            } else {
                if (sp == 0) return;
                cur = stack[--sp];
            }
        } else {
            const uint32_t code = ~(uint32_t)cur;
            const uint32_t first = code >> kLeafCountBits, count = code & kMaxLeafSize;
            for (uint32_t k = first; k < first + count; ++k) {
                if (COUNT) ++st.tris;
                float t;
                const bool ok = MODE == 1 ? tri_test_wt(a.tri_wt, k, r, w, best_t, t)
                                          : tri_test_ref(a.tri_ref, k, r, best_t, t);
                if (ok) {
                    const int32_t prim = __ldg(a.prim + k);
                    if (t < best_t || prim < best_prim) {
                        best_t = t;
                        best_prim = prim;
                    }
                }
            }
            if (sp == 0) return;
            cur = stack[--sp];
        }
    }
}

// Any hit with t <= tmax.
template <int MODE>
__device__ __forceinline__ bool any_hit(const TraceArgs &a, const DevRay &r, uint32_t root)
{
    if (root == kNoRoot) return false;
    WtSetup w;
    if (MODE == 1) w = wt_setup(r.v);
    int32_t stack[kStackSize];
    int sp = 0;
    int32_t cur = (int32_t)root;
    const float tmax = r.tmax;
    while (true) {
        if (cur >= 0) {
            const float4 *np = reinterpret_cast<const float4 *>(a.nodes + cur);
            const float4 c0xy = __ldg(np), c1xy = __ldg(np + 1), cz = __ldg(np + 2);
            const int4 link = __ldg(reinterpret_cast<const int4 *>(np + 3));
            float t0, t1;
            bool h0, h1;
            intersect_children(c0xy, c1xy, cz, r, tmax, t0, t1, h0, h1);
            if (h0 && h1) {
                if (sp >= kStackSize) {
                    atomicOr(a.error, ERR_STACK_OVERFLOW);
                    return false;
                }
                const bool swap = t1 < t0;
                stack[sp++] = swap ? link.x : link.y;
                cur = swap ? link.y : link.x;
            } else if (h0) {
                cur = link.x;
            } else if (h1) {
                cur = link.y;
            } else {
                if (sp == 0) return false;
                cur = stack[--sp];
            }
        } else {
            const uint32_t code = ~(uint32_t)cur;
            const uint32_t first = code >> kLeafCountBits, count = code & kMaxLeafSize;
            for (uint32_t k = first; k < first + count; ++k) {
                float t;
                const bool ok = MODE == 1 ? tri_test_wt(a.tri_wt, k, r, w, tmax, t)
                                          : tri_test_ref(a.tri_ref, k, r, tmax, t);
                if (ok) return true;
            }
            if (sp == 0) return false;
            cur = stack[--sp];
        }
    }
}

// Closest / any hit in the scene's layout.
template <int MODE, bool COUNT, int LAYOUT>
__device__ __forceinline__ void scene_closest(const TraceArgs &a, const DevRay &r, uint32_t root, float &best_t,
                                              int32_t &best_prim, TraceStats &st)
{
    if (LAYOUT == 8) {
        const Wide8Args w{a.nodes8, a.tri_ref, a.tri_wt, a.prim, a.num_nodes, a.error, a.stack_limit};
        if (COUNT) wide_traverse<MODE, false>(w, r, root, best_t, best_prim, &st.nodes, &st.boxes, &st.tris);
        else wide_traverse<MODE, false>(w, r, root, best_t, best_prim, nullptr, nullptr, nullptr);
    } else {
        closest_hit<MODE, COUNT>(a, r, root, best_t, best_prim, st);
    }
}

template <int MODE, int LAYOUT>
__device__ __forceinline__ bool scene_any(const TraceArgs &a, const DevRay &r, uint32_t root)
{
    if (LAYOUT == 8) {
        const Wide8Args w{a.nodes8, a.tri_ref, a.tri_wt, a.prim, a.num_nodes, a.error, a.stack_limit};
        float t;
        int32_t prim;
        return wide_traverse<MODE, true>(w, r, root, t, prim, nullptr, nullptr, nullptr);
    }
    return any_hit<MODE>(a, r, root);
}

// Root of a single-scene hierarchy.
__host__ __device__ __forceinline__ uint32_t scene_root(uint32_t num_nodes) { return num_nodes ? 0u : kNoRoot; }

}  // namespace dr
