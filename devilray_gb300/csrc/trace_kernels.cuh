// trace_kernels.cuh -- launch interface of the traversal kernels.
#pragma once

#include "dr_internal.h"

namespace dr {

constexpr int kTraceBlock = 128;

struct TraceArgs {
    const Bvh2Node *nodes;
    const Bvh8Node *nodes8;   // compressed 8-wide layout (used when layout == 8)
    int layout;
    const float4 *tri_ref;
    const float4 *tri_wt;
    const int32_t *prim;
    uint32_t num_nodes;
    const dr_ray *rays;
    uint64_t n;
    dr_hit *hits;          // closest hit
    uint8_t *occluded;     // any hit
    unsigned long long *counters;
    uint32_t *error;
    unsigned long long *work;  // persistent-kernel ray counter (zeroed before each launch)
    int num_sms;
    uint32_t stack_limit;      // 8-wide traversal stack entries (<= kWideStack)
};

// Launch helpers dispatch on a.layout (2 or 8) and the triangle mode.
// Resident blocks per SM of `kernel` at `block_threads` threads (cached per kernel).
int resident_blocks(const void *kernel, int block_threads);
cudaError_t launch_trace_closest(const TraceArgs &a, int mode, bool count, cudaStream_t s);
cudaError_t launch_trace_any(const TraceArgs &a, int mode, cudaStream_t s);

}  // namespace dr
