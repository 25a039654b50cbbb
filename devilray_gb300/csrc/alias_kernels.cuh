// alias_kernels.cuh -- alias-table build / sampling interface.
#pragma once

#include "dr_internal.h"

namespace dr {

constexpr int kSweepBlock = 512;

// sample() of include/tracing/DistributionSamplers.hpp:64-88 (DevilRay) for
// given uniforms u0 (slot) and u1 (A or B); FP32 as the reference.
__device__ __forceinline__ void alias_sample(const dr_alias_entry *__restrict__ table, uint32_t n, float u0,
                                             float u1, int32_t &index, float &pdf)
{
    float findex = u0 * (float)n;
    if (findex == (float)n) findex = (float)n - 1;
    const int idx = static_cast<int>(findex);
    // 20-byte entries are only 4-byte aligned: scalar loads.
    const float *e = reinterpret_cast<const float *>(table + idx);
    const float p_A = __ldg(e);
    if (u1 <= p_A) {
        index = __ldg(reinterpret_cast<const int32_t *>(e) + 3);
        pdf = __ldg(e + 1);
    } else {
        index = __ldg(reinterpret_cast<const int32_t *>(e) + 4);
        pdf = __ldg(e + 2);
    }
}

size_t alias_scratch_bytes(uint32_t n, int mode);
cudaError_t launch_alias_build(const float *w, uint32_t n, dr_alias_entry *out, int mode, void *scratch,
                               size_t scratch_bytes, int num_sms, cudaStream_t st);
// Reference-mode builds of many small tables (one device thread per table).
cudaError_t launch_alias_ref_segments(const float *w, uint32_t total_n, const uint32_t *begin, const uint32_t *count,
                                     uint32_t nseg, dr_alias_entry *out, void *scratch, size_t scratch_bytes,
                                     cudaStream_t st);
// Sweep-mode builds of many tables, one device thread per table (any size;
// the table equals launch_alias_build's DR_ALIAS_SWEEP table of the segment).
constexpr uint32_t kSweepThreadMax = 1u << 16;  // larger tables: the parallel build
cudaError_t launch_alias_sweep_segments(const float *w, const uint32_t *begin, const uint32_t *count, uint32_t nseg,
                                       dr_alias_entry *out, cudaStream_t st);
cudaError_t launch_alias_sample(const dr_alias_entry *table, uint32_t n, const float *u, uint64_t draws,
                                int32_t *index, float *pdf, cudaStream_t st);

}  // namespace dr
