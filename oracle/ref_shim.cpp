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

// checkerPattern lives in src/device/implementation.cu beside the render
// kernel (a CUDA translation unit the harness does not build). Contract of
// include/tracing/PathGeneration.hpp:24-29: checker cell parity of uv scaled by
// checker_count on each axis, XOR-ed; 1 selects `bright`, 0 selects `dark`.
#include "Utils.hpp"

HD Vec4 checkerPattern(const Vec2f &uv, const int checker_count, const Vec4 dark, const Vec4 bright)
{
    const int cell = (int(uv.x * checker_count) % 2) ^ (int(uv.y * checker_count) % 2);
    const float f = (float)cell;
    return bright * f + dark * (1 - f);
}
