// diag.cu -- diagnostics without a counterpart in the reference:
//  * the read-bandwidth probe: the roofline denominator of the traversal
//    kernels (streaming reads of a buffer that fits in L2 give the L2 read
//    bandwidth, a buffer larger than L2 the HBM read bandwidth);
//  * the failure paths' test hooks: a bounded mbarrier wait made to give up,
//    a lower cap on the traversal stack, and failed device allocations. None
//    of them faults, traps or hangs a GPU: each makes the library take the
//    same error path that a real timeout, overflow or out-of-memory takes.

#include "dr_internal.h"
#include "mbarrier.cuh"

namespace dr {
namespace {

__global__ void __launch_bounds__(256) k_read_stream(const float4 *__restrict__ buf, uint64_t n4, uint32_t reps,
                                                     float *__restrict__ sink)
{
    float acc = 0.0f;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint32_t r = 0; r < reps; ++r) {
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
            float4 v;
            // ld.global.cg: cached in L2 only, so L1 hits do not inflate the figure
            asm volatile("ld.global.cg.v4.f32 {%0,%1,%2,%3}, [%4];"
                         : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                         : "l"(buf + i));
            acc += v.x + v.y + v.z + v.w;
        }
    }
    if (acc == 1234.5678f) sink[0] = acc;  // keeps the loads alive
}

// One warp waits on phase 0 of an mbarrier that expects one arrival and gets
// none, with at most `polls` polls of the same bounded wait the product
// kernels use; when it gives up it reports the timeout as they do. No copy and
// no MMA is in flight on the barrier.
__global__ void k_expire_wait(uint32_t polls, uint32_t *error)
{
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(b, 0, polls));
    if (!ok && threadIdx.x == 0) atomicOr(error, ERR_TIMEOUT);
}

}  // namespace
}  // namespace dr

using namespace dr;

extern "C" dr_status dr_debug_expire_wait(dr_context *ctx, uint32_t polls, void *stream)
{
    DR_CHECK_ARG(ctx, "dr_debug_expire_wait: NULL context");
    DR_CUDA(cudaSetDevice(ctx->device));
    k_expire_wait<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(polls, ctx->d_error);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

extern "C" dr_status dr_debug_stack_limit(dr_context *ctx, uint32_t entries)
{
    DR_CHECK_ARG(ctx, "dr_debug_stack_limit: NULL context");
    DR_CHECK_ARG(entries <= 64, "dr_debug_stack_limit: at most 64 entries");
    ctx->stack_limit = entries ? entries : 64;
    return DR_OK;
}

extern "C" dr_status dr_probe_read_bandwidth(dr_context *ctx, const void *buf_dev, uint64_t bytes, uint32_t reps,
                                             double *gbs_out, void *stream)
{
    DR_CHECK_ARG(ctx && buf_dev && gbs_out && bytes >= 16 && reps > 0, "dr_probe_read_bandwidth: bad argument");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(buf_dev) & 15) == 0, "dr_probe_read_bandwidth: buffer not 16-byte aligned");
    DR_CUDA(cudaSetDevice(ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    const uint64_t n4 = bytes / 16;
    const int blocks = ctx->num_sms * 8;
    // a word of the context's status block that nothing else uses
    float *sink = reinterpret_cast<float *>(reinterpret_cast<char *>(ctx->d_error) + 128);
    k_read_stream<<<blocks, 256, 0, st>>>(static_cast<const float4 *>(buf_dev), n4, 1, sink);  // warm
    cudaEvent_t a, b;
    DR_CUDA(cudaEventCreate(&a));
    DR_CUDA(cudaEventCreate(&b));
    DR_CUDA(cudaEventRecord(a, st));
    k_read_stream<<<blocks, 256, 0, st>>>(static_cast<const float4 *>(buf_dev), n4, reps, sink);
    DR_CUDA(cudaGetLastError());
    DR_CUDA(cudaEventRecord(b, st));
    DR_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    DR_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *gbs_out = (double)n4 * 16.0 * reps / (ms * 1e-3) / 1e9;
    return DR_OK;
}
