// ref_shim.cpp -- the one host function the reference's DeviceMemory.cu needs
// from DevUtils.cu (which also holds a cuRAND kernel and so cannot be built
// as plain C++). Same contract as src/device/DevUtils.cu:12-22 (DevilRay):
// report a pending CUDA error; the harness never launches device work.
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

void cudaCheckLastError(const char *file, int line, bool abort)
{
    const auto code = cudaPeekAtLastError();
    if (code != cudaSuccess) {
        std::fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
        if (abort) std::exit(code);
    }
}
