// framebuffer.cu -- accumulation buffers of a progressive render and their
// display conversion on the device (Renderer::createPixels of the reference,
// src/Renderer.cpp:51-90, which copies the whole buffer to the host each frame).

#include "dr_internal.h"
#include "alias_kernels.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

struct dr_framebuffer {
    dr_context *ctx = nullptr;
    int32_t width = 0, height = 0;
    float4 *accum = nullptr;
    uint32_t *casts = nullptr;
    uint32_t *pixels = nullptr;
};

namespace dr {
namespace {

// toSRGB of createPixels: linear passes through; otherwise clamp to [0, 1],
// 12.92 r below 0.0031308, else 1.055 r^(1/2.4) - 0.055 (evaluated in double
// after the FP32 power, as the reference's mixed float/double expression).
__device__ __forceinline__ float to_srgb(float linear, bool gamma)
{
    if (!gamma) return linear;
    const float r = fminf(fmaxf(linear, 0.f), 1.f);
    if (r < 0.0031308) return (float)((double)r * 12.92);
    // the float power rounded from a double power: the correctly rounded powf
    const float p = (float)pow((double)r, (double)(1 / 2.4f));
    return (float)((double)p * 1.055 - 0.055f);
}

__device__ __forceinline__ uint32_t to_u32(float f) { return (uint32_t)roundf(f); }

__global__ void k_tonemap(const float4 *__restrict__ accum, int32_t w, int32_t h, int gamma, uint32_t *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const float4 p = accum[x + (size_t)y * w];
    float r = 0.f, g = 0.f, b = 0.f;
    if (p.w != 0.f) {
        r = p.x / p.w;
        g = p.y / p.w;
        b = p.z / p.w;
    }
    const uint32_t v = (to_u32(to_srgb(r, gamma) * 255)) | (to_u32(to_srgb(g, gamma) * 255) << 8) |
                       (to_u32(to_srgb(b, gamma) * 255) << 16) | (to_u32(1.0f * 255) << 24);
    out[x + (size_t)(h - y - 1) * w] = v;
}

__global__ void k_resolve(const float4 *__restrict__ accum, uint64_t n, float *__restrict__ rgb)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = accum[i];
    const bool any = p.w != 0.f;
    rgb[3 * i] = any ? p.x / p.w : 0.0f;
    rgb[3 * i + 1] = any ? p.y / p.w : 0.0f;
    rgb[3 * i + 2] = any ? p.z / p.w : 0.0f;
}

}  // namespace
}  // namespace dr

using namespace dr;

extern "C" {

dr_status dr_framebuffer_create(dr_context *ctx, int32_t width, int32_t height, dr_framebuffer **out)
{
    DR_CHECK_ARG(ctx && out && width > 0 && height > 0, "dr_framebuffer_create: bad argument");
    DR_CHECK_ARG(height <= 65535 && (uint64_t)width * (uint64_t)height < (1ull << 31),
                 "dr_framebuffer_create: image too large");
    *out = nullptr;
    DR_CUDA(cudaSetDevice(ctx->device));
    auto *fb = new (std::nothrow) dr_framebuffer;
    if (!fb) return fail(DR_ERR_OUT_OF_MEMORY, "host allocation failed");
    fb->ctx = ctx;
    fb->width = width;
    fb->height = height;
    const size_t n = (size_t)width * height;
    cudaError_t e;
    if ((e = dev_malloc(&fb->accum, n * sizeof(float4))) != cudaSuccess ||
        (e = dev_malloc(&fb->casts, n * sizeof(uint32_t))) != cudaSuccess ||
        (e = dev_malloc(&fb->pixels, n * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMemset(fb->accum, 0, n * sizeof(float4))) != cudaSuccess ||
        (e = cudaMemset(fb->casts, 0, n * sizeof(uint32_t))) != cudaSuccess) {
        dr_framebuffer_destroy(fb);
        return cuda_fail(e, "dr_framebuffer_create");
    }
    *out = fb;
    return DR_OK;
}

dr_status dr_framebuffer_destroy(dr_framebuffer *fb)
{
    if (!fb) return DR_OK;
    cudaSetDevice(fb->ctx->device);
    cudaFree(fb->accum);
    cudaFree(fb->casts);
    cudaFree(fb->pixels);
    delete fb;
    return DR_OK;
}

dr_status dr_framebuffer_clear(dr_framebuffer *fb, void *stream)
{
    DR_CHECK_ARG(fb != nullptr, "dr_framebuffer_clear: NULL");
    DR_CUDA(cudaSetDevice(fb->ctx->device));
    const size_t n = (size_t)fb->width * fb->height;
    auto st = static_cast<cudaStream_t>(stream);
    DR_CUDA(cudaMemsetAsync(fb->accum, 0, n * sizeof(float4), st));
    DR_CUDA(cudaMemsetAsync(fb->casts, 0, n * sizeof(uint32_t), st));
    return DR_OK;
}

dr_status dr_framebuffer_device_buffers(dr_framebuffer *fb, float **accum_dev, uint32_t **casts_dev)
{
    DR_CHECK_ARG(fb != nullptr, "dr_framebuffer_device_buffers: NULL");
    if (accum_dev) *accum_dev = reinterpret_cast<float *>(fb->accum);
    if (casts_dev) *casts_dev = fb->casts;
    return DR_OK;
}

dr_status dr_framebuffer_read(dr_framebuffer *fb, float *accum_host, uint32_t *casts_host, uint64_t *total_casts)
{
    DR_CHECK_ARG(fb != nullptr, "dr_framebuffer_read: NULL");
    DR_CUDA(cudaSetDevice(fb->ctx->device));
    const size_t n = (size_t)fb->width * fb->height;
    DR_CUDA(cudaDeviceSynchronize());
    if (accum_host) DR_CUDA(cudaMemcpy(accum_host, fb->accum, n * sizeof(float4), cudaMemcpyDeviceToHost));
    if (casts_host || total_casts) {
        std::vector<uint32_t> tmp;
        uint32_t *dst = casts_host;
        if (!dst) {
            tmp.resize(n);
            dst = tmp.data();
        }
        DR_CUDA(cudaMemcpy(dst, fb->casts, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (total_casts) {
            uint64_t t = 0;
            for (size_t i = 0; i < n; ++i) t += dst[i];
            *total_casts = t;
        }
    }
    return DR_OK;
}

dr_status dr_tonemap(const float *accum_dev, int32_t width, int32_t height, int32_t gamma_corrected,
                     uint32_t *rgba_dev, void *stream)
{
    DR_CHECK_ARG(accum_dev && rgba_dev && width > 0 && height > 0, "dr_tonemap: bad argument");
    DR_CHECK_ARG(height <= 65535 && (uint64_t)width * (uint64_t)height < (1ull << 31), "dr_tonemap: image too large");
    DR_CHECK_ARG(((uintptr_t)accum_dev & 15) == 0, "dr_tonemap: accum_dev must be 16-byte aligned");
    const dim3 grid((width + 127) / 128, height);
    k_tonemap<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(reinterpret_cast<const float4 *>(accum_dev), width,
                                                                 height, gamma_corrected ? 1 : 0, rgba_dev);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_resolve(const float *accum_dev, int32_t width, int32_t height, float *rgb_dev, void *stream)
{
    DR_CHECK_ARG(accum_dev && rgb_dev && width > 0 && height > 0, "dr_resolve: bad argument");
    DR_CHECK_ARG(((uintptr_t)accum_dev & 15) == 0, "dr_resolve: accum_dev must be 16-byte aligned");
    const uint64_t n = (uint64_t)width * (uint64_t)height;
    k_resolve<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4 *>(accum_dev), n, rgb_dev);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_framebuffer_write_pfm(dr_framebuffer *fb, const char *path)
{
    DR_CHECK_ARG(fb && path, "dr_framebuffer_write_pfm: NULL");
    DR_CUDA(cudaSetDevice(fb->ctx->device));
    const size_t n = (size_t)fb->width * fb->height;
    float *rgb = nullptr;
    DR_CUDA(dev_malloc(&rgb, n * 3 * sizeof(float)));
    std::vector<float> host(n * 3);
    dr_status st = dr_resolve(reinterpret_cast<const float *>(fb->accum), fb->width, fb->height, rgb, nullptr);
    cudaError_t e = st == DR_OK ? cudaMemcpy(host.data(), rgb, n * 3 * sizeof(float), cudaMemcpyDeviceToHost)
                                : cudaSuccess;
    cudaFree(rgb);
    if (st != DR_OK) return st;
    if (e != cudaSuccess) return cuda_fail(e, "dr_framebuffer_write_pfm");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(DR_ERR_INVALID_ARGUMENT, "dr_framebuffer_write_pfm: cannot open %s", path);
    // PFM header: colour, width height, negative scale = little-endian samples
    const int hdr = fprintf(f, "PF\n%d %d\n-1.0\n", fb->width, fb->height);
    uint32_t probe = 1;
    const bool little = *reinterpret_cast<unsigned char *>(&probe) == 1;
    bool ok = hdr > 0;
    if (ok && little) {
        ok = fwrite(host.data(), sizeof(float), host.size(), f) == host.size();
    } else if (ok) {
        for (size_t i = 0; ok && i < host.size(); ++i) {
            uint32_t b;
            memcpy(&b, &host[i], 4);
            const unsigned char le[4] = {(unsigned char)b, (unsigned char)(b >> 8), (unsigned char)(b >> 16),
                                         (unsigned char)(b >> 24)};
            ok = fwrite(le, 1, 4, f) == 4;
        }
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) return fail(DR_ERR_INVALID_ARGUMENT, "dr_framebuffer_write_pfm: writing %s failed", path);
    return DR_OK;
}

dr_status dr_framebuffer_tonemap(dr_framebuffer *fb, int32_t gamma_corrected, uint32_t *rgba_host)
{
    DR_CHECK_ARG(fb && rgba_host, "dr_framebuffer_tonemap: NULL");
    DR_CUDA(cudaSetDevice(fb->ctx->device));
    const dr_status st = dr_tonemap(reinterpret_cast<const float *>(fb->accum), fb->width, fb->height,
                                    gamma_corrected, fb->pixels, nullptr);
    if (st != DR_OK) return st;
    DR_CUDA(cudaMemcpy(rgba_host, fb->pixels, (size_t)fb->width * fb->height * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_alias_build_host(dr_context *ctx, const float *w, uint32_t n, dr_alias_entry *out, int32_t mode)
{
    DR_CHECK_ARG(ctx != nullptr, "dr_alias_build_host: ctx is NULL");
    DR_CHECK_ARG(n == 0 || (w && out), "dr_alias_build_host: NULL buffer");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    float *dw = nullptr;
    dr_alias_entry *dt = nullptr;
    DR_CUDA(dev_malloc(&dw, (size_t)n * sizeof(float)));
    cudaError_t e = dev_malloc(&dt, (size_t)n * sizeof(dr_alias_entry));
    if (e == cudaSuccess) e = cudaMemcpy(dw, w, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    dr_status st = DR_OK;
    if (e == cudaSuccess) {
        st = dr_alias_build(ctx, dw, n, dt, mode, nullptr);
        if (st == DR_OK) e = cudaMemcpy(out, dt, (size_t)n * sizeof(dr_alias_entry), cudaMemcpyDeviceToHost);
    }
    cudaFree(dw);
    cudaFree(dt);
    if (e != cudaSuccess) return cuda_fail(e, "dr_alias_build_host");
    return st;
}

}  // extern "C"
