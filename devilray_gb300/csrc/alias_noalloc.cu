// alias_noalloc.cu -- alias-table build that allocates no device memory.
//
// dr_alias_build() keeps its scratch in the context and grows it with
// cudaMalloc. Some callers cannot allow that: a host application that owns
// every device allocation and hands a plugin only pre-allocated buffers, or a
// frame loop in which cudaMalloc's implicit device synchronisation would
// stall the GPU. For them dr_alias_build_noalloc() runs the same sweep-mode
// kernels with their scratch in the file-scope array below, which every GPU
// that loads this library holds until the process exits.
//
//  * Limit: n <= kNoAllocMaxEntries (65,536 weights, about 2.6 MB of scratch).
//    Larger n is rejected with DR_ERR_TOO_LARGE.
//  * Set-up: the first call on a device looks up the device address of the
//    array (cudaGetSymbolAddress, with that device current) and caches it;
//    make that first call before any stream capture. The cache lives as long
//    as the process: a device reset (cudaDeviceReset) after the first call is
//    not supported, because the array's address may change with the new
//    context while the cached one would not.
//  * Sharing: every call uses the same array and the array keeps the last
//    call's contents. The build's first kernel re-initialises the running
//    totals it reads, so stale contents never leak into a result, but calls
//    whose work overlaps on the GPU (different streams without ordering) race
//    on the array.

#include "dr_internal.h"
#include "alias_kernels.cuh"

#include <mutex>

namespace dr {
namespace {

constexpr uint32_t kNoAllocMaxEntries = 65536;
// alias_scratch_bytes(65536, sweep) = 512 + 128 tiles x 48 + 65536 x 40 + 256
constexpr size_t kNoAllocScratchBytes = 512 + ((kNoAllocMaxEntries + kSweepBlock - 1) / kSweepBlock) * 48 +
                                        (size_t)kNoAllocMaxEntries * 40 + 256 + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Per-device set-up: the host-side name of the array is not a device address,
// so the kernel gets the address cudaGetSymbolAddress returns for the current
// device.
dr_status noalloc_setup(int device, void **ptr, int *num_sms)
{
    if (device < 0 || device >= kMaxDevices) return fail(DR_ERR_UNSUPPORTED, "dr_alias_build_noalloc: device %d", device);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int sms = 0;
        const cudaError_t e2 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaDeviceGetAttribute(multiProcessorCount)");
        g_num_sms[device] = sms;
        g_scratch_ptr[device] = p;
    }
    *ptr = g_scratch_ptr[device];
    *num_sms = g_num_sms[device];
    return DR_OK;
}

}  // namespace
}  // namespace dr

using namespace dr;

extern "C" dr_status dr_alias_build_noalloc(const float *weights_dev, uint32_t n, dr_alias_entry *table_dev,
                                            void *stream)
{
    DR_CHECK_ARG(n == 0 || (weights_dev && table_dev), "dr_alias_build_noalloc: NULL buffer");
    if (n > kNoAllocMaxEntries)
        return fail(DR_ERR_TOO_LARGE, "dr_alias_build_noalloc: n = %u exceeds the fixed scratch limit of %u weights",
                    n, kNoAllocMaxEntries);
    if (n == 0) return DR_OK;
    int device = 0;
    DR_CUDA(cudaGetDevice(&device));
    void *scratch = nullptr;
    int num_sms = 0;
    const dr_status s = noalloc_setup(device, &scratch, &num_sms);
    if (s != DR_OK) return s;
    DR_CUDA(launch_alias_build(weights_dev, n, table_dev, DR_ALIAS_SWEEP, scratch, kNoAllocScratchBytes, num_sms,
                               static_cast<cudaStream_t>(stream)));
    return DR_OK;
}
