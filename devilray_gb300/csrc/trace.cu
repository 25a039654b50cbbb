// trace.cu -- closest-hit and any-hit BVH traversal on sm_103a.
//
// Replaces the reference's per-object stackless descent with parent pointers
// (DevilRay include/tracing/IntersectionTestsImpl.hpp:141-251) by a stack
// traversal of a binned-SAH two-box BVH. Culling is conservative (widened
// boxes, enter <= best), and a candidate wins when its t is smaller, or equal
// with a smaller original triangle index, so the result equals a brute-force
// scan of the reference triangle test over the whole soup.

#include "dr_internal.h"
#include "tri_device.cuh"
#include "trace_kernels.cuh"

#include <climits>

namespace dr {

// Counters are reduced per warp and added once per warp.
__device__ __forceinline__ void add_counters(unsigned long long *c, unsigned long long nodes,
                                             unsigned long long boxes, unsigned long long tris,
                                             unsigned long long hits)
{
    for (int off = 16; off > 0; off >>= 1) {
        nodes += __shfl_down_sync(0xffffffffu, nodes, off);
        boxes += __shfl_down_sync(0xffffffffu, boxes, off);
        tris += __shfl_down_sync(0xffffffffu, tris, off);
        hits += __shfl_down_sync(0xffffffffu, hits, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(c + 0, nodes);
        atomicAdd(c + 1, boxes);
        atomicAdd(c + 2, tris);
        atomicAdd(c + 3, hits);
    }
}

template <int MODE, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_closest(TraceArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long n_nodes = 0, n_boxes = 0, n_tris = 0, n_hits = 0;
    if (i < a.n) {
        DevRay r;
        const bool valid = load_ray(a.rays, i, r);
        float best_t = r.tmax;
        int32_t best_prim = INT_MAX;
        if (valid && a.num_nodes > 0) {
            WtSetup w;
            if (MODE == 1) w = wt_setup(r.v);
            int32_t stack[kStackSize];
            int sp = 0;
            int32_t cur = 0;
            while (true) {
                if (cur >= 0) {
                    const float4 *np = reinterpret_cast<const float4 *>(a.nodes + cur);
                    const float4 c0xy = __ldg(np), c1xy = __ldg(np + 1), cz = __ldg(np + 2);
                    const int4 link = __ldg(reinterpret_cast<const int4 *>(np + 3));
                    float t0, t1;
                    bool h0, h1;
                    intersect_children(c0xy, c1xy, cz, r, best_t, t0, t1, h0, h1);
                    if (COUNT) {
                        ++n_nodes;
                        n_boxes += 2;
                    }
                    if (h0 && h1) {
                        const bool swap = t1 < t0;
                        if (sp >= kStackSize) {
                            atomicOr(a.error, ERR_STACK_OVERFLOW);
                            break;
                        }
                        stack[sp++] = swap ? link.x : link.y;
                        cur = swap ? link.y : link.x;
                    } else if (h0) {
                        cur = link.x;
                    } else if (h1) {
                        cur = link.y;
                    } else {
                        if (sp == 0) break;
                        cur = stack[--sp];
                    }
                } else {
                    const uint32_t code = ~(uint32_t)cur;
                    const uint32_t first = code >> kLeafCountBits, count = code & kMaxLeafSize;
                    for (uint32_t k = first; k < first + count; ++k) {
                        if (COUNT) ++n_tris;
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
                    if (sp == 0) break;
                    cur = stack[--sp];
                }
            }
        }
        dr_hit h;
        if (best_prim != INT_MAX) {
            h.t = best_t;
            h.prim = best_prim;
            n_hits = 1;
        } else {
            h.t = __int_as_float(0x7f800000);
            h.prim = -1;
        }
        reinterpret_cast<float2 *>(a.hits)[i] = make_float2(h.t, __int_as_float(h.prim));
    }
    if (COUNT) add_counters(a.counters, n_nodes, n_boxes, n_tris, n_hits);
}

template <int MODE>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_any(TraceArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    DevRay r;
    const bool valid = load_ray(a.rays, i, r);
    uint8_t hit = 0;
    if (valid && a.num_nodes > 0) {
        WtSetup w;
        if (MODE == 1) w = wt_setup(r.v);
        int32_t stack[kStackSize];
        int sp = 0;
        int32_t cur = 0;
        const float tmax = r.tmax;
        while (!hit) {
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
                        break;
                    }
                    const bool swap = t1 < t0;
                    stack[sp++] = swap ? link.x : link.y;
                    cur = swap ? link.y : link.x;
                } else if (h0) {
                    cur = link.x;
                } else if (h1) {
                    cur = link.y;
                } else {
                    if (sp == 0) break;
                    cur = stack[--sp];
                }
            } else {
                const uint32_t code = ~(uint32_t)cur;
                const uint32_t first = code >> kLeafCountBits, count = code & kMaxLeafSize;
                for (uint32_t k = first; k < first + count; ++k) {
                    float t;
                    const bool ok = MODE == 1 ? tri_test_wt(a.tri_wt, k, r, w, tmax, t)
                                              : tri_test_ref(a.tri_ref, k, r, tmax, t);
                    if (ok) {
                        hit = 1;
                        break;
                    }
                }
                if (hit || sp == 0) break;
                cur = stack[--sp];
            }
        }
    }
    a.occluded[i] = hit;
}

cudaError_t launch_trace_closest(const TraceArgs &a, int mode, bool count, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    const uint64_t blocks = (a.n + kTraceBlock - 1) / kTraceBlock;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)blocks), block(kTraceBlock);
    if (mode == 1) {
        if (count) k_trace_closest<1, true><<<grid, block, 0, s>>>(a);
        else k_trace_closest<1, false><<<grid, block, 0, s>>>(a);
    } else {
        if (count) k_trace_closest<0, true><<<grid, block, 0, s>>>(a);
        else k_trace_closest<0, false><<<grid, block, 0, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_any(const TraceArgs &a, int mode, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    const uint64_t blocks = (a.n + kTraceBlock - 1) / kTraceBlock;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)blocks), block(kTraceBlock);
    if (mode == 1) k_trace_any<1><<<grid, block, 0, s>>>(a);
    else k_trace_any<0><<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace dr
