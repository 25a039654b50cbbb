// trace.cu -- public closest-hit and any-hit kernels on sm_103a.
//
// Replaces the reference's per-object stackless descent with parent pointers
// (DevilRay include/tracing/IntersectionTestsImpl.hpp:141-251) by the stack
// traversal of trace_device.cuh over a binned-SAH two-box BVH. One thread per
// ray; the result equals a brute-force scan of the reference triangle test
// over the whole soup (smallest t, ties to the smaller triangle index).

// The public 8-wide kernels run the slab FMAs of slots j and j + 4 as packed
// FP32 pairs and are compiled for 7 resident blocks per SM (73 registers).
// Measured on the incoherent workload (2^20 triangles, 16.8 M rays, closest
// hit): scalar at 8 blocks 3.383 ms, packed at 7 blocks 3.336-3.339 ms,
// packed at 6 blocks 3.534 ms, scalar at 7 blocks 3.409 ms; hits identical.
#ifndef DR_PACKED_SLAB
#define DR_PACKED_SLAB 1
#endif
#ifndef DR_P8_MIN_BLOCKS
#define DR_P8_MIN_BLOCKS 7
#endif

#include "dr_internal.h"
#include "trace_device.cuh"
#include "persistent.cuh"

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

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

template <int MODE, bool COUNT, int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_closest(TraceArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TraceStats st;
    unsigned long long n_hits = 0;
    if (i < a.n) {
        DevRay r;
        const bool valid = load_ray(a.rays, i, r);
        float best_t = r.tmax;
        int32_t best_prim = INT_MAX;
        if (valid) scene_closest<MODE, COUNT, LAYOUT>(a, r, scene_root(a.num_nodes), best_t, best_prim, st);
        float2 out;
        if (best_prim != INT_MAX) {
            out = make_float2(best_t, __int_as_float(best_prim));
            n_hits = 1;
        } else {
            out = make_float2(__int_as_float(0x7f800000), __int_as_float(-1));
        }
        reinterpret_cast<float2 *>(a.hits)[i] = out;
    }
    if (COUNT) add_counters(a.counters, st.nodes, st.boxes, st.tris, n_hits);
}

template <int MODE, int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_any(TraceArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    DevRay r;
    const bool valid = load_ray(a.rays, i, r);
    a.occluded[i] = (valid && scene_any<MODE, LAYOUT>(a, r, scene_root(a.num_nodes))) ? 1 : 0;
}

// Persistent kernels for the compressed 8-wide layout.
template <int MODE, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock, kP8MinBlocks) k_trace_closest_p8(TraceArgs a)
{
    const Wide8Args w{a.nodes8, a.tri_ref, a.tri_wt, a.prim, a.num_nodes, a.error, a.stack_limit};
    const DirectSource src{a.rays, a.hits, nullptr, scene_root(a.num_nodes)};
    unsigned long long nn = 0, nb = 0, nt = 0, nh = 0;
    persistent_wide<MODE, false, COUNT, DR_TRI_BATCH_CLOSEST != 0>(w, src, a.n, a.work, nn, nb, nt, nh);
    if (COUNT) add_counters(a.counters, nn, nb, nt, nh);
}

template <int MODE>
__global__ void __launch_bounds__(kTraceBlock, kP8MinBlocks) k_trace_any_p8(TraceArgs a)
{
    const Wide8Args w{a.nodes8, a.tri_ref, a.tri_wt, a.prim, a.num_nodes, a.error, a.stack_limit};
    const DirectSource src{a.rays, nullptr, a.occluded, scene_root(a.num_nodes)};
    unsigned long long nn = 0, nb = 0, nt = 0, nh = 0;
    persistent_wide<MODE, true, false, DR_TRI_BATCH_ANY != 0>(w, src, a.n, a.work, nn, nb, nt, nh);
}

int resident_blocks(const void *kernel, int block_threads)
{
    // one entry per kernel: kernels of the same signature differ in registers
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> cache;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &e : cache)
        if (e.first == kernel) return e.second;
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, block_threads, 0) != cudaSuccess || b <= 0) {
        cudaGetLastError();
        b = 4;
    }
    cache.emplace_back(kernel, b);
    return b;
}

template <typename K>
unsigned persistent_grid(K kernel, int num_sms, uint64_t n)
{
    const int per_sm = resident_blocks((const void *)kernel, kTraceBlock);
    const uint64_t need = (n + kTraceBlock - 1) / kTraceBlock;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)num_sms * per_sm));
}

cudaError_t launch_trace_closest(const TraceArgs &a, int mode, bool count, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    const uint64_t blocks = (a.n + kTraceBlock - 1) / kTraceBlock;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)blocks), block(kTraceBlock);
    if (a.layout == 8) {
        cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) return e;
        if (mode == 1) {
            if (count) k_trace_closest_p8<1, true><<<persistent_grid(k_trace_closest_p8<1, true>, a.num_sms, a.n), block, 0, s>>>(a);
            else k_trace_closest_p8<1, false><<<persistent_grid(k_trace_closest_p8<1, false>, a.num_sms, a.n), block, 0, s>>>(a);
        } else {
            if (count) k_trace_closest_p8<0, true><<<persistent_grid(k_trace_closest_p8<0, true>, a.num_sms, a.n), block, 0, s>>>(a);
            else k_trace_closest_p8<0, false><<<persistent_grid(k_trace_closest_p8<0, false>, a.num_sms, a.n), block, 0, s>>>(a);
        }
    } else {
        if (mode == 1) {
            if (count) k_trace_closest<1, true, 2><<<grid, block, 0, s>>>(a);
            else k_trace_closest<1, false, 2><<<grid, block, 0, s>>>(a);
        } else {
            if (count) k_trace_closest<0, true, 2><<<grid, block, 0, s>>>(a);
            else k_trace_closest<0, false, 2><<<grid, block, 0, s>>>(a);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_any(const TraceArgs &a, int mode, cudaStream_t s)
{
    if (a.n == 0) return cudaSuccess;
    const uint64_t blocks = (a.n + kTraceBlock - 1) / kTraceBlock;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)blocks), block(kTraceBlock);
    if (a.layout == 8) {
        cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) return e;
        if (mode == 1) k_trace_any_p8<1><<<persistent_grid(k_trace_any_p8<1>, a.num_sms, a.n), block, 0, s>>>(a);
        else k_trace_any_p8<0><<<persistent_grid(k_trace_any_p8<0>, a.num_sms, a.n), block, 0, s>>>(a);
    } else {
        if (mode == 1) k_trace_any<1, 2><<<grid, block, 0, s>>>(a);
        else k_trace_any<0, 2><<<grid, block, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace dr
