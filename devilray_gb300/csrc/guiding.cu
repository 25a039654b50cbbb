// guiding.cu -- the path-guiding network on tensor cores: inference, one
// training step (forward, loss gradient, backward, weight gradients) and Adam.
//
// Network: 80 inputs (12-frequency encoding of the normalised position, a
// direction, zero padding) -> 4 hidden layers of 64 (ReLU) -> 48 outputs (40
// used: the 8-lobe vMF mixture of guide_math.cuh). Weights and layer inputs
// are BF16, every product accumulates in FP32 (mma.sync m16n8k16 on the
// tensor cores); master weights and Adam moments are FP32.
//
// A warp carries 16 rows through all layers in registers: the FP32
// accumulator fragment of one layer is, pair by pair, the BF16 A fragment of
// the next (m16n8 C layout = m16k16 A layout of two adjacent column tiles).
// Backward products use the transposed weights, staged in shared memory; the
// deltas enter the tensor cores as a BF16 high part plus a BF16 remainder so
// the propagated gradient keeps about 16 bits. Weight gradients are
// delta^T x activations over the batch (K = rows), split over row chunks and
// summed with atomics.

#include "dr_internal.h"
#include "mbarrier.cuh"
#include "guide_math.cuh"
#include "guide_internal.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

namespace dr {
namespace {

constexpr int kIn = 80, kHid = 64, kOut = 48, kLayers = 5;

// CTAs per SM of the tcgen05 inference launch (at most 3 fit: 62.7 KB of
// shared memory each).
#ifndef DR_INFER_CTAS_PER_SM
#define DR_INFER_CTAS_PER_SM 3
#endif
__host__ __device__ constexpr int fan_in(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int fan_out(int l) { return l == kLayers - 1 ? kOut : kHid; }

__host__ __device__ constexpr int w_off(int l)
{
    int o = 0;
    for (int i = 0; i < l; ++i) o += fan_out(i) * fan_in(i) + fan_out(i);
    return o;
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + fan_out(l) * fan_in(l); }
constexpr int kNumParams = w_off(kLayers);
// BF16 weights (no biases) in the same order, for the kernels
__host__ __device__ constexpr int wb_off(int l)
{
    int o = 0;
    for (int i = 0; i < l; ++i) o += fan_out(i) * fan_in(i);
    return o;
}
constexpr int kNumWeights = wb_off(kLayers);

// shared-memory strides (bf16 elements), padded so the 8 rows of a fragment
// load fall in distinct banks
constexpr int kStrideIn = kIn + 8;    // 88
constexpr int kStrideHid = kHid + 8;  // 72
constexpr int kStrideOutT = kOut + 8; // 56: transposed last layer [64][48]

struct GuideParams {
    float center[3];
    float half;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Encoded input pair (columns c, c + 1; c even) of a row.
__device__ __forceinline__ void encode_pair(const float p[3], const float d[3], int c, float &v0, float &v1)
{
    if (c < 72) {
        const int a = c / 24, k = (c % 24) >> 1;
        const float x = ldexpf(p[a], k);  // exact: scaling by a power of two
        sincospif(x, &v0, &v1);
    } else if (c == 72) {
        v0 = d[0];
        v1 = d[1];
    } else if (c == 74) {
        v0 = d[2];
        v1 = 0.0f;
    } else {
        v0 = v1 = 0.0f;
    }
}

// Shared-memory image of the weights: forward W_l [out][in] and, for the
// backward pass, W_l^T [in][out] of layers 1..4.
struct SmemWeights {
    __nv_bfloat16 w0[kHid * kStrideIn];
    __nv_bfloat16 w[3][kHid * kStrideHid];     // layers 1..3
    __nv_bfloat16 w4[kOut * kStrideHid];
    float bias[4 * kHid + kOut];
};
struct SmemWeightsT {
    __nv_bfloat16 t[3][kHid * kStrideHid];     // W_l^T, l = 1..3: [in 64][out 64]
    __nv_bfloat16 t4[kHid * kStrideOutT];      // W_4^T: [in 64][out 48]
};

__device__ void load_weights(SmemWeights &s, const __nv_bfloat16 *wb, const float *params)
{
    for (int i = threadIdx.x; i < kHid * kIn; i += blockDim.x) s.w0[(i / kIn) * kStrideIn + i % kIn] = wb[i];
    for (int l = 1; l <= 3; ++l)
        for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x)
            s.w[l - 1][(i / kHid) * kStrideHid + i % kHid] = wb[wb_off(l) + i];
    for (int i = threadIdx.x; i < kOut * kHid; i += blockDim.x) s.w4[(i / kHid) * kStrideHid + i % kHid] = wb[wb_off(4) + i];
    for (int l = 0; l < kLayers; ++l)
        for (int i = threadIdx.x; i < fan_out(l); i += blockDim.x) s.bias[l * kHid + i] = params[b_off(l) + i];
}

__device__ void load_weights_t(SmemWeightsT &s, const __nv_bfloat16 *wb)
{
    for (int l = 1; l <= 3; ++l)
        for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) {
            const int o = i / kHid, in = i % kHid;
            s.t[l - 1][in * kStrideHid + o] = wb[wb_off(l) + i];
        }
    for (int i = threadIdx.x; i < kOut * kHid; i += blockDim.x) {
        const int o = i / kHid, in = i % kHid;
        s.t4[in * kStrideOutT + o] = wb[wb_off(4) + i];
    }
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// acc[nt] += A (16 x 16 ks-slices) x B where B[k][n] = W[n][k], W row-major with
// `stride`; NT column tiles of 8, KS k-steps of 16.
template <int NT, int KS>
__device__ __forceinline__ void layer_mma(float (&acc)[NT][4], const uint32_t (&a)[KS][4], const __nv_bfloat16 *W,
                                          int stride)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __nv_bfloat16 *row = W + (8 * nt + g) * stride + 16 * ks + 2 * tig;
            mma_bf16(acc[nt], a[ks], ld_pair(row), ld_pair(row + 8));
        }
}

template <int NT>
__device__ __forceinline__ void init_bias(float (&acc)[NT][4], const float *bias)
{
    const int tig = threadIdx.x & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float b0 = bias[8 * nt + 2 * tig], b1 = bias[8 * nt + 2 * tig + 1];
        acc[nt][0] = b0, acc[nt][1] = b1, acc[nt][2] = b0, acc[nt][3] = b1;
    }
}

// ReLU of a 64-wide accumulator, as the A fragments of the next layer.
__device__ __forceinline__ void relu_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4])
{
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        const float *l = acc[2 * ks], *h = acc[2 * ks + 1];
        a[ks][0] = pack_bf16(fmaxf(l[0], 0.0f), fmaxf(l[1], 0.0f));
        a[ks][1] = pack_bf16(fmaxf(l[2], 0.0f), fmaxf(l[3], 0.0f));
        a[ks][2] = pack_bf16(fmaxf(h[0], 0.0f), fmaxf(h[1], 0.0f));
        a[ks][3] = pack_bf16(fmaxf(h[2], 0.0f), fmaxf(h[3], 0.0f));
    }
}

// Input fragments of 16 rows (5 k-steps of 16 encoded columns).
__device__ __forceinline__ void input_frags(const float p_g[3], const float d_g[3], const float p_h[3],
                                            const float d_h[3], uint32_t (&a)[5][4])
{
    const int tig = threadIdx.x & 3;
#pragma unroll
    for (int ks = 0; ks < 5; ++ks) {
        float v0, v1;
        const int c0 = 16 * ks + 2 * tig, c1 = c0 + 8;
        encode_pair(p_g, d_g, c0, v0, v1);
        a[ks][0] = pack_bf16(v0, v1);
        encode_pair(p_h, d_h, c0, v0, v1);
        a[ks][1] = pack_bf16(v0, v1);
        encode_pair(p_g, d_g, c1, v0, v1);
        a[ks][2] = pack_bf16(v0, v1);
        encode_pair(p_h, d_h, c1, v0, v1);
        a[ks][3] = pack_bf16(v0, v1);
    }
}

__device__ __forceinline__ void load_row(const float *pos, const float *dir, const uint32_t *list, uint32_t n, uint32_t r,
                                         const GuideParams &gp, float p[3], float d[3], uint32_t &slot)
{
    slot = r < n ? (list ? list[r] : r) : 0xffffffffu;
    if (r >= n) {
        p[0] = p[1] = p[2] = d[0] = d[1] = d[2] = 0.0f;
        return;
    }
    for (int a = 0; a < 3; ++a) {
        const float x = (pos[3 * (size_t)slot + a] - gp.center[a]) / gp.half;
        p[a] = fminf(1.0f, fmaxf(-1.0f, x));
        d[a] = dir[3 * (size_t)slot + a];
    }
}

// Forward pass of 16 rows per warp; y[slot][40] for rows r < n (slot = list[r]
// or r). Grid-stride over 16-row tiles.
__global__ void __launch_bounds__(128) k_guide_infer(const __nv_bfloat16 *wb, const float *params, GuideParams gp,
                                                     const float *pos, const float *dir, const uint32_t *list,
                                                     const uint32_t *count, uint32_t n_fixed, float *y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    SmemWeights &s = *reinterpret_cast<SmemWeights *>(smem);
    load_weights(s, wb, params);
    __syncthreads();
    const uint32_t n = count ? *count : n_fixed;
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); 16ull * tile < n; tile += warps) {
        const uint32_t r0 = 16 * tile;
        float pg[3], dg[3], ph[3], dh[3];
        uint32_t sg, sh;
        load_row(pos, dir, list, n, r0 + g, gp, pg, dg, sg);
        load_row(pos, dir, list, n, r0 + g + 8, gp, ph, dh, sh);
        uint32_t a0[5][4];
        input_frags(pg, dg, ph, dh, a0);
        float acc[8][4];
        uint32_t a[4][4];
        init_bias(acc, s.bias);
        layer_mma<8, 5>(acc, a0, s.w0, kStrideIn);
        relu_to_a(acc, a);
#pragma unroll
        for (int l = 1; l <= 3; ++l) {
            init_bias(acc, s.bias + l * kHid);
            layer_mma<8, 4>(acc, a, s.w[l - 1], kStrideHid);
            relu_to_a(acc, a);
        }
        float out[6][4];
        init_bias(out, s.bias + 4 * kHid);
        layer_mma<6, 4>(out, a, s.w4, kStrideHid);
#pragma unroll
        for (int nt = 0; nt < 5; ++nt) {
            const int c = 8 * nt + 2 * tig;
            if (sg != 0xffffffffu)
                *reinterpret_cast<float2 *>(y + (size_t)sg * kGuideOut + c) = make_float2(out[nt][0], out[nt][1]);
            if (sh != 0xffffffffu)
                *reinterpret_cast<float2 *>(y + (size_t)sh * kGuideOut + c) = make_float2(out[nt][2], out[nt][3]);
        }
    }
}


// ---- inference on the 5th-generation tensor cores (tcgen05) -------------------
//
// One CTA of 128 threads carries tiles of 128 rows (the M of one tcgen05.mma)
// through the network: layer inputs and weights sit in shared memory in the
// canonical K-major layout without swizzle, the one elected thread issues the
// K/16 MMAs of a layer into a 128 x N FP32 accumulator in tensor memory and
// commits them to an mbarrier, and each warp reads its 32 rows back with
// tcgen05.ld for the bias / ReLU / BF16 epilogue, which writes the next
// layer's input. Same arithmetic as k_guide_infer (BF16 products, FP32 sums).

constexpr int kTcRows = 128;

// Byte offset of element (r, c) of an R x K BF16 matrix in the canonical
// K-major layout: core matrices of 8 rows x 8 columns (8 rows of 16 bytes);
// column chunk j (columns 8j..8j+7) of all R rows is contiguous.
__device__ __forceinline__ uint32_t canon_off(int r, int c, int R) { return (uint32_t)((c >> 3) * R * 16 + r * 16 + (c & 7) * 2); }

// Shared-memory matrix descriptor: start address, leading byte offset (between
// core matrices adjacent along K) and stride byte offset (between core
// matrices adjacent along M or N), all >> 4; version 1 (bits 46-47); no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounded wait on an mbarrier phase; false after the iteration limit.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase)
{
    return mbar_wait_bounded(mbar, phase, kMbarWaitPolls);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared memory of k_guide_infer_tc (byte offsets).
constexpr uint32_t kTcW0 = 0;                        // 64 x 80
constexpr uint32_t kTcW1 = kTcW0 + 64 * 80 * 2;      // 3 x 64 x 64
constexpr uint32_t kTcW4 = kTcW1 + 3 * 64 * 64 * 2;  // 48 x 64
constexpr uint32_t kTcA = kTcW4 + 48 * 64 * 2 + 1024;  // 128 x 80 input / 128 x 64 hidden
constexpr uint32_t kTcBias = kTcA + kTcRows * kIn * 2;
constexpr uint32_t kTcBar = kTcBias + (4 * kHid + kOut) * 4;  // MMA mbarrier, TMEM address, copy mbarrier
constexpr uint32_t kTcSmem = kTcBar + 24;

// The weights as the tcgen05 kernels hold them in shared memory, kept in
// global memory beside the BF16 copy so a CTA fetches them with one bulk
// asynchronous copy: [0, 40960) the forward operands (kTcW0..kTcW4: W_l as
// N = out, K = in, canonical K-major), [40960, 71680) the backward operands of
// layers 1..4 (W_l as N = in 64, K = out).
constexpr uint32_t kImgFwdBytes = 40960;
constexpr uint32_t kImgBytes = kImgFwdBytes + 3 * kHid * kHid * 2 + kHid * kOut * 2;

__device__ __forceinline__ void store_weight(__nv_bfloat16 *wb, unsigned char *img, int l, int idx, float p)
{
    const __nv_bfloat16 b = __float2bfloat16_rn(p);
    wb[wb_off(l) + idx] = b;
    const int o = idx / fan_in(l), in = idx % fan_in(l);
    const uint32_t fwd = l == 0 ? kTcW0 : l == 4 ? kTcW4 : kTcW1 + (uint32_t)(l - 1) * kHid * kHid * 2;
    *reinterpret_cast<__nv_bfloat16 *>(img + fwd + canon_off(o, in, fan_out(l))) = b;
    if (l > 0) {
        const uint32_t bwd = kImgFwdBytes + (uint32_t)(l - 1) * kHid * kHid * 2;
        *reinterpret_cast<__nv_bfloat16 *>(img + bwd + canon_off(in, o, kHid)) = b;
    }
}

// One bulk asynchronous copy of `bytes` of the weight image into shared
// memory, completing on the mbarrier `cbar` (issued by one thread).
__device__ __forceinline__ void fetch_weight_image(uint32_t dst, const unsigned char *img, uint32_t bytes, uint32_t cbar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(cbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(cbar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(img), "r"(bytes), "r"(cbar)
                 : "memory");
}

__global__ void __launch_bounds__(128) k_guide_infer_tc(const unsigned char *img, const float *params, GuideParams gp,
                                                        const float *pos, const float *dir, const uint32_t *list,
                                                        const uint32_t *count, uint32_t n_fixed, float *y,
                                                        uint32_t *error, bool decoded)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights in the canonical layout (B operands: N = outputs, K = inputs):
    // the forward part of the weight image, one bulk copy
    const uint32_t cbar = smem_u32(smem + kTcBar + 16);
    if (tid == 0) fetch_weight_image(smem_u32(smem + kTcW0), img, kImgFwdBytes, cbar);
    float *bias = reinterpret_cast<float *>(smem + kTcBias);
    for (int l = 0; l < kLayers; ++l)
        for (int i = tid; i < fan_out(l); i += 128) bias[l * kHid + i] = params[b_off(l) + i];
    const uint32_t mbar = smem_u32(smem + kTcBar);
    const uint32_t tslot = smem_u32(smem + kTcBar + 8);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;\n" ::"r"(tslot) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *reinterpret_cast<volatile uint32_t *>(smem + kTcBar + 8);
    const uint32_t a_base = smem_u32(smem + kTcA);
    const uint32_t w_base[kLayers] = {smem_u32(smem + kTcW0), smem_u32(smem + kTcW1), smem_u32(smem + kTcW1 + 8192),
                                      smem_u32(smem + kTcW1 + 16384), smem_u32(smem + kTcW4)};
    const uint32_t n = count ? *count : n_fixed;
    uint32_t phase = 0;
    // the weights have landed (bounded wait, one decision for the block)
    bool ok = __syncthreads_and(mbar_wait(cbar, 0) ? 1 : 0) != 0;
    if (!ok && tid == 0) atomicOr(error, ERR_TIMEOUT);
    for (uint32_t tile = blockIdx.x; ok && (uint64_t)tile * kTcRows < n; tile += gridDim.x) {
        const uint32_t r = tile * kTcRows + tid;
        float p[3], d[3];
        uint32_t slot;
        load_row(pos, dir, list, n, r, gp, p, d, slot);
        // input row: 10 chunks of 8 encoded columns
#pragma unroll
        for (int j = 0; j < kIn / 8; ++j) {
            uint32_t q[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float v0, v1;
                encode_pair(p, d, 8 * j + 2 * k, v0, v1);
                q[k] = pack_bf16(v0, v1);
            }
            *reinterpret_cast<uint4 *>(smem + kTcA + canon_off(tid, 8 * j, kTcRows)) = make_uint4(q[0], q[1], q[2], q[3]);
        }
        for (int l = 0; l < kLayers; ++l) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
            const int K = fan_in(l), N = fan_out(l);
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t idesc = idesc_bf16(kTcRows, N);
                for (int s2 = 0; s2 < K / 16; ++s2) {
                    const uint64_t ad = smem_desc(a_base + (uint32_t)s2 * 2 * kTcRows * 16, kTcRows * 16, 128);
                    const uint64_t bd = smem_desc(w_base[l] + (uint32_t)s2 * 2 * N * 16, (uint32_t)N * 16, 128);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(s2));
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                             : "memory");
            }
            // one decision for the whole block: every thread waited (bounded) on the same phase
            if (!__syncthreads_and(mbar_wait(mbar, phase) ? 1 : 0)) {
                if (tid == 0) atomicOr(error, ERR_TIMEOUT);
                ok = false;
                break;
            }
            phase ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
            float v[64];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float t[16];
                tmem_ld16(lane_addr + 16 * c, t);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[16 * c + i] = t[i];
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const float *b = bias + l * kHid;
            if (l < kLayers - 1) {
#pragma unroll
                for (int j = 0; j < kHid / 8; ++j) {
                    uint32_t q[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        q[k] = pack_bf16(fmaxf(v[8 * j + 2 * k] + b[8 * j + 2 * k], 0.0f),
                                         fmaxf(v[8 * j + 2 * k + 1] + b[8 * j + 2 * k + 1], 0.0f));
                    *reinterpret_cast<uint4 *>(smem + kTcA + canon_off(tid, 8 * j, kTcRows)) =
                        make_uint4(q[0], q[1], q[2], q[3]);
                }
            } else if (slot != 0xffffffffu && decoded) {
                float o[kGuideOut];
#pragma unroll
                for (int i = 0; i < kGuideOut; ++i) o[i] = v[i] + b[i];
                guide_store_decoded(y + (size_t)slot * kGuideOut, guide_mix_values(o));
            } else if (slot != 0xffffffffu) {
                float4 *dst = reinterpret_cast<float4 *>(y + (size_t)slot * kGuideOut);
#pragma unroll
                for (int j = 0; j < kGuideOut / 4; ++j)
                    dst[j] = make_float4(v[4 * j] + b[4 * j], v[4 * j + 1] + b[4 * j + 1], v[4 * j + 2] + b[4 * j + 2],
                                         v[4 * j + 3] + b[4 * j + 3]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (!ok) {
        // MMAs or the weight copy still in flight: wait again (bounded) before freeing their memory
        mbar_wait(mbar, phase);
        mbar_wait(cbar, 0);
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;\n" ::"r"(taddr) : "memory");
}

// ---- training -----------------------------------------------------------------

struct TrainBuffers {
    // per layer l (0..4): delta of the layer output, transposed [out][rows] (FP32),
    // and the layer input, transposed [in][rows] (BF16)
    float *deltaT[kLayers];
    __nv_bfloat16 *actT[kLayers];
    uint32_t rows;  // row stride of the transposed arrays (batch capacity)
};

// Writes a 16 x (8 NT) FP32 accumulator transposed: dst[col][row0 + row].
template <int NT>
__device__ __forceinline__ void store_t(float *dst, uint32_t stride, uint32_t row0, const float (&acc)[NT][4], uint32_t n,
                                        int ncols)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int c = 8 * nt + 2 * tig;
        if (c >= ncols) continue;
        if (row0 + g < n) {
            dst[(size_t)c * stride + row0 + g] = acc[nt][0];
            dst[(size_t)(c + 1) * stride + row0 + g] = acc[nt][1];
        }
        if (row0 + g + 8 < n) {
            dst[(size_t)c * stride + row0 + g + 8] = acc[nt][2];
            dst[(size_t)(c + 1) * stride + row0 + g + 8] = acc[nt][3];
        }
    }
}

// Writes BF16 A fragments (KS k-steps) transposed: dst[col][row0 + row].
template <int KS>
__device__ __forceinline__ void store_a_t(__nv_bfloat16 *dst, uint32_t stride, uint32_t row0, const uint32_t (&a)[KS][4],
                                          uint32_t n)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int row = g + ((q & 1) ? 8 : 0);
            const int c = 16 * ks + 2 * tig + ((q & 2) ? 8 : 0);
            if (row0 + row >= n) continue;
            const uint32_t v = a[ks][q];
            __nv_bfloat16 lo, hi;
            const uint16_t lb = (uint16_t)(v & 0xffffu), hb = (uint16_t)(v >> 16);
            memcpy(&lo, &lb, 2);
            memcpy(&hi, &hb, 2);
            dst[(size_t)c * stride + row0 + row] = lo;
            dst[(size_t)(c + 1) * stride + row0 + row] = hi;
        }
}

// Splits FP32 accumulators of 64 (or 48) columns into BF16 high and low A
// fragments (KS k-steps), after masking by the ReLU of `act` (the layer's
// output fragments) when MASK.
template <int KS, bool MASK>
__device__ __forceinline__ void delta_frags(float (&acc)[2 * KS][4], const uint32_t (&act)[4][4], uint32_t (&hi)[KS][4],
                                            uint32_t (&lo)[KS][4])
{
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            // q: 0 (rows g, tile 2ks) 1 (rows g+8, tile 2ks) 2 (rows g, tile 2ks+1) 3 (rows g+8, tile 2ks+1)
            float *c = acc[2 * ks + (q >> 1)] + ((q & 1) ? 2 : 0);
            if (MASK) {
                const uint32_t m = act[ks][q];
                if ((m & 0x7fffu) == 0) c[0] = 0.0f;
                if ((m & 0x7fff0000u) == 0) c[1] = 0.0f;
            }
            const __nv_bfloat162 h = __floats2bfloat162_rn(c[0], c[1]);
            const float2 hf = __bfloat1622float2(h);
            hi[ks][q] = *reinterpret_cast<const uint32_t *>(&h);
            lo[ks][q] = pack_bf16(c[0] - hf.x, c[1] - hf.y);
        }
    }
}

// One block = 4 warps = 64 rows. Forward with stored activations, loss
// gradient, backward deltas; writes deltaT / actT of every layer and adds the
// batch loss. weight_sum: sum of the batch's sample weights (device scalar).
__global__ void __launch_bounds__(128) k_guide_train_fb(const __nv_bfloat16 *wb, const float *params, GuideParams gp,
                                                        const float *pos, const float *dir, const float *sdir,
                                                        const float *weight, uint32_t n, const float *weight_sum,
                                                        TrainBuffers tb, float *loss)
{
    extern __shared__ __align__(16) unsigned char smem[];
    SmemWeights &s = *reinterpret_cast<SmemWeights *>(smem);
    SmemWeightsT &t = *reinterpret_cast<SmemWeightsT *>(smem + sizeof(SmemWeights));
    float *ybuf = reinterpret_cast<float *>(smem + sizeof(SmemWeights) + sizeof(SmemWeightsT));  // [4 warps][16][48]
    load_weights(s, wb, params);
    load_weights_t(t, wb);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    float *yw = ybuf + warp * 16 * kOut;
    const uint32_t r0 = 64 * blockIdx.x + 16 * warp;
    if (r0 >= n) return;  // no block-wide barrier follows
    float pg[3], dg[3], ph[3], dh[3];
    uint32_t sg, sh;
    load_row(pos, dir, nullptr, n, r0 + g, gp, pg, dg, sg);
    load_row(pos, dir, nullptr, n, r0 + g + 8, gp, ph, dh, sh);
    uint32_t a0[5][4], h[4][4][4];  // inputs; outputs of layers 0..3 (post-ReLU)
    input_frags(pg, dg, ph, dh, a0);
    float acc[8][4];
    init_bias(acc, s.bias);
    layer_mma<8, 5>(acc, a0, s.w0, kStrideIn);
    relu_to_a(acc, h[0]);
#pragma unroll
    for (int l = 1; l <= 3; ++l) {
        init_bias(acc, s.bias + l * kHid);
        layer_mma<8, 4>(acc, h[l - 1], s.w[l - 1], kStrideHid);
        relu_to_a(acc, h[l]);
    }
    float out[6][4];
    init_bias(out, s.bias + 4 * kHid);
    layer_mma<6, 4>(out, h[3], s.w4, kStrideHid);
    // layer inputs, transposed
    store_a_t<5>(tb.actT[0], tb.rows, r0, a0, n);
#pragma unroll
    for (int l = 1; l < kLayers; ++l) store_a_t<4>(tb.actT[l], tb.rows, r0, h[l - 1], n);
    // loss gradient, one row per lane
#pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
        const int c = 8 * nt + 2 * tig;
        yw[g * kOut + c] = out[nt][0];
        yw[g * kOut + c + 1] = out[nt][1];
        yw[(g + 8) * kOut + c] = out[nt][2];
        yw[(g + 8) * kOut + c + 1] = out[nt][3];
    }
    __syncwarp();
    float dyrow[kGuideOut];
    if (lane < 16) {
        const uint32_t r = r0 + lane;
        float lq = 0.0f;
        if (r < n) {
            const float wm = *weight_sum / (float)n;
            const float c = wm > 0.0f ? weight[r] / wm : 0.0f;
            lq = guide_loss_grad(yw + lane * kOut, sdir[3 * (size_t)r], sdir[3 * (size_t)r + 1], sdir[3 * (size_t)r + 2],
                                 c / (float)n, dyrow);
            atomicAdd(loss, -c * lq / (float)n);
        } else {
            for (int i = 0; i < kGuideOut; ++i) dyrow[i] = 0.0f;
        }
    }
    __syncwarp();
    if (lane < 16) {
        for (int i = 0; i < kGuideOut; ++i) yw[lane * kOut + i] = dyrow[i];
        for (int i = kGuideOut; i < kOut; ++i) yw[lane * kOut + i] = 0.0f;
    }
    __syncwarp();
    float dy[6][4];
#pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
        const int c = 8 * nt + 2 * tig;
        dy[nt][0] = yw[g * kOut + c];
        dy[nt][1] = yw[g * kOut + c + 1];
        dy[nt][2] = yw[(g + 8) * kOut + c];
        dy[nt][3] = yw[(g + 8) * kOut + c + 1];
    }
    store_t<6>(tb.deltaT[4], tb.rows, r0, dy, n, kOut);
    // delta of h4 = (dy W4) * relu'(h4): A = dy (K = 48), B[k][n] = W4[k][n] = W4T[n][k]
    uint32_t dhi3[3][4], dlo3[3][4];
    {
        uint32_t dummy[4][4] = {};
        delta_frags<3, false>(dy, dummy, dhi3, dlo3);
    }
    float dacc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) dacc[nt][0] = dacc[nt][1] = dacc[nt][2] = dacc[nt][3] = 0.0f;
    layer_mma<8, 3>(dacc, dhi3, t.t4, kStrideOutT);
    layer_mma<8, 3>(dacc, dlo3, t.t4, kStrideOutT);
    uint32_t dhi[4][4], dlo[4][4];
#pragma unroll
    for (int l = 3; l >= 1; --l) {
        delta_frags<4, true>(dacc, h[l], dhi, dlo);  // masks dacc in place by relu'(h_l)
        store_t<8>(tb.deltaT[l], tb.rows, r0, dacc, n, kHid);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) dacc[nt][0] = dacc[nt][1] = dacc[nt][2] = dacc[nt][3] = 0.0f;
        layer_mma<8, 4>(dacc, dhi, t.t[l - 1], kStrideHid);
        layer_mma<8, 4>(dacc, dlo, t.t[l - 1], kStrideHid);
    }
    delta_frags<4, true>(dacc, h[0], dhi, dlo);
    store_t<8>(tb.deltaT[0], tb.rows, r0, dacc, n, kHid);
}

// Issues the K/16 MMAs of one product into the accumulator at taddr
// (accumulating from the first when `acc`).
__device__ __forceinline__ void tc_mma_chain(uint32_t taddr, uint32_t a_base, uint32_t b_base, int M, int N, int K,
                                             bool acc)
{
    const uint32_t idesc = idesc_bf16(M, N);
    for (int s2 = 0; s2 < K / 16; ++s2) {
        const uint64_t ad = smem_desc(a_base + (uint32_t)s2 * 2 * M * 16, (uint32_t)M * 16, 128);
        const uint64_t bd = smem_desc(b_base + (uint32_t)s2 * 2 * N * 16, (uint32_t)N * 16, 128);
        const uint32_t en = (acc || s2 > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
            "l"(ad), "l"(bd), "r"(idesc), "r"(en));
    }
}

// ---- training on the 5th-generation tensor cores (tcgen05) ----------------------
//
// One CTA of 128 threads carries 128-row tiles through the forward pass, the
// loss gradient, the backward deltas and the weight gradients, with the same
// arithmetic as k_guide_train_fb + k_guide_wgrad (BF16 operands, FP32 sums;
// deltas enter the tensor cores as a BF16 high part plus a BF16 remainder):
// thread t owns row t of the tile. Forward layer l: D[128 x out] = x_l W_l^T
// as in k_guide_infer_tc. Backward layer l: D[128 x in] = delta_hi W_l +
// delta_lo W_l, with W_l staged as the N = in, K = out operand. Every layer
// input x_l stays in shared memory for the whole tile, and the delta tile
// holds [delta_hi | delta_lo] as one 128 x 128 matrix. Both serve twice, through two
// descriptors of the same bytes: K-major (the forward product over inputs,
// the backward product over outputs) and MN-major (the weight-gradient
// product over rows): dW_l[128 x (in + 16)] += [delta_hi | delta_lo]^T x_l,
// whose rows 0-63 and 64-127 are the high and low parts of dW_l. The 16 extra
// columns of x_l hold 1.0, so column `in` of the product is the bias
// gradient. The per-layer sums stay in tensor memory across the CTA's tiles
// and are added to the gradient once, at the end. Measured per Adam step:
// 16,384 rows 0.108 ms, 65,536 rows 0.166 ms (mma.sync forward/backward plus
// weight-gradient kernel: 0.180 and 0.545 ms).

// Shared memory of k_guide_train_fused (byte offsets).
constexpr uint32_t kTfX0 = 0;                                  // x_0: 128 x (80 + 16)
constexpr uint32_t kTfX1 = kTfX0 + 12 * 2048;                  // x_1..x_4: 128 x (64 + 16) each
constexpr uint32_t kTfD = kTfX1 + 4 * 10 * 2048;               // [delta_hi | delta_lo]: 128 x 128
constexpr uint32_t kTfW = kTfD + 16 * 2048;                    // forward weights, as kTcW0..kTcW4
constexpr uint32_t kTfWT1 = kTfW + 40960;                      // W_l as [in 64][out 64], l = 1..3
constexpr uint32_t kTfWT4 = kTfWT1 + 3 * kHid * kHid * 2;      // W_4 as [in 64][out 48]
constexpr uint32_t kTfBias = kTfWT4 + kHid * kOut * 2;
constexpr uint32_t kTfBar = kTfBias + (4 * kHid + kOut) * 4;  // MMA mbarrier, TMEM address, copy mbarrier
constexpr uint32_t kTfSmem = kTfBar + 24;
static_assert(kTfWT1 == kTfW + kImgFwdBytes && kTfBias == kTfW + kImgBytes, "the weight image is one copy");
// tensor-memory columns: [0, 64) the forward / backward product, then dW_l
__host__ __device__ constexpr uint32_t tf_dcol(int l) { return l == 0 ? 64u : 160u + 80u * (uint32_t)(l - 1); }

// Instruction descriptor of kind::f16 with both operands MN-major (bits 15, 16).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N) { return idesc_bf16(M, N) | (1u << 15) | (1u << 16); }

__global__ void __launch_bounds__(128) k_guide_train_fused(const unsigned char *img, const float *params,
                                                           GuideParams gp, const float *pos, const float *dir,
                                                           const float *sdir, const float *weight, uint32_t n,
                                                           const float *weight_sum, float *grad, float *loss,
                                                           uint32_t *error)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // forward (N = out, K = in) and backward (N = in, K = out) weights: the
    // weight image, one bulk copy
    const uint32_t cbar = smem_u32(smem + kTfBar + 16);
    if (tid == 0) fetch_weight_image(smem_u32(smem + kTfW), img, kImgBytes, cbar);
    float *bias = reinterpret_cast<float *>(smem + kTfBias);
    for (int l = 0; l < kLayers; ++l)
        for (int i = tid; i < fan_out(l); i += 128) bias[l * kHid + i] = params[b_off(l) + i];
    const uint32_t xoff[kLayers] = {kTfX0, kTfX1, kTfX1 + 20480, kTfX1 + 40960, kTfX1 + 61440};
    // the columns of ones (in .. in + 15) of every x_l
    {
        const uint32_t one2 = 0x3f803f80u;
#pragma unroll
        for (int l = 0; l < kLayers; ++l)
#pragma unroll
            for (int j = 0; j < 2; ++j)
                *reinterpret_cast<uint4 *>(smem + xoff[l] + canon_off(tid, fan_in(l) + 8 * j, kTcRows)) =
                    make_uint4(one2, one2, one2, one2);
    }
    const uint32_t mbar = smem_u32(smem + kTfBar);
    const uint32_t tslot = smem_u32(smem + kTfBar + 8);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(tslot) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *reinterpret_cast<volatile uint32_t *>(smem + kTfBar + 8);
    const uint32_t d_base = smem_u32(smem + kTfD), dlo_base = d_base + 8 * 2048;
    uint32_t x_base[kLayers];
#pragma unroll
    for (int l = 0; l < kLayers; ++l) x_base[l] = smem_u32(smem + xoff[l]);
    const uint32_t w_base[kLayers] = {smem_u32(smem + kTfW + kTcW0), smem_u32(smem + kTfW + kTcW1),
                                      smem_u32(smem + kTfW + kTcW1 + 8192), smem_u32(smem + kTfW + kTcW1 + 16384),
                                      smem_u32(smem + kTfW + kTcW4)};
    const uint32_t wt_base[kLayers] = {0, smem_u32(smem + kTfWT1), smem_u32(smem + kTfWT1 + 8192),
                                       smem_u32(smem + kTfWT1 + 16384), smem_u32(smem + kTfWT4)};
    const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
    const float wmean = *weight_sum / (float)n;
    uint32_t phase = 0;
    // the weights have landed (bounded wait, one decision for the block)
    bool ok = __syncthreads_and(mbar_wait(cbar, 0) ? 1 : 0) != 0, first = true;
    if (!ok && tid == 0) atomicOr(error, ERR_TIMEOUT);

    auto run = [&](auto issue) -> bool {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            issue();
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                         : "memory");
        }
        if (!__syncthreads_and(mbar_wait(mbar, phase) ? 1 : 0)) {
            if (tid == 0) atomicOr(error, ERR_TIMEOUT);
            return false;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        return true;
    };
    // dW_l += [delta_hi | delta_lo]^T x_l over the tile's 128 rows (8 MMAs of
    // 16 rows; MN-major operands: 8-row groups 128 B apart, 8-column groups
    // 2048 B apart)
    auto wgrad = [&](int l, bool acc) {
        const uint32_t idesc = idesc_bf16_mn(kTcRows, fan_in(l) + 16);
        for (int s2 = 0; s2 < kTcRows / 16; ++s2) {
            const uint64_t ad = smem_desc(d_base + (uint32_t)s2 * 256, 128, 2048);
            const uint64_t bd = smem_desc(x_base[l] + (uint32_t)s2 * 256, 128, 2048);
            const uint32_t en = (acc || s2 > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + tf_dcol(l)),
                "l"(ad), "l"(bd), "r"(idesc), "r"(en));
        }
    };
    auto read_acc = [&](float (&v)[64], uint32_t col, int ncols) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (16 * c >= ncols) break;
            float t[16];
            tmem_ld16(lane_addr + col + 16 * c, t);
#pragma unroll
            for (int i = 0; i < 16; ++i) v[16 * c + i] = t[i];
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    };
    // [delta_hi | delta_lo] row of this thread: 8-column chunks j of K = ncols
    auto put_delta = [&](const float *dv, int ncols) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t hi[4], lo[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i0 = 8 * j + 2 * k;
                const float c0 = i0 < ncols ? dv[i0] : 0.0f, c1 = i0 + 1 < ncols ? dv[i0 + 1] : 0.0f;
                const __nv_bfloat162 h = __floats2bfloat162_rn(c0, c1);
                const float2 hf = __bfloat1622float2(h);
                hi[k] = *reinterpret_cast<const uint32_t *>(&h);
                lo[k] = pack_bf16(c0 - hf.x, c1 - hf.y);
            }
            *reinterpret_cast<uint4 *>(smem + kTfD + canon_off(tid, 8 * j, kTcRows)) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
            *reinterpret_cast<uint4 *>(smem + kTfD + canon_off(tid, 64 + 8 * j, kTcRows)) =
                make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
    };

    for (uint32_t tile = blockIdx.x; ok && (uint64_t)tile * kTcRows < n; tile += gridDim.x) {
        const uint32_t r = tile * kTcRows + tid;
        const bool live = r < n;
        float p[3], d[3];
        uint32_t slot;
        load_row(pos, dir, nullptr, n, r, gp, p, d, slot);
#pragma unroll
        for (int j = 0; j < kIn / 8; ++j) {
            uint32_t q[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float v0, v1;
                encode_pair(p, d, 8 * j + 2 * k, v0, v1);
                q[k] = pack_bf16(v0, v1);
            }
            *reinterpret_cast<uint4 *>(smem + kTfX0 + canon_off(tid, 8 * j, kTcRows)) = make_uint4(q[0], q[1], q[2], q[3]);
        }
        uint64_t mask[4] = {0, 0, 0, 0};
        float v[64];
        for (int l = 0; l < kLayers && ok; ++l) {
            const int K = fan_in(l), N = fan_out(l);
            ok = run([&] { tc_mma_chain(taddr, x_base[l], w_base[l], kTcRows, N, K, false); });
            if (!ok) break;
            read_acc(v, 0, N);
            const float *b = bias + l * kHid;
            if (l < kLayers - 1) {
#pragma unroll
                for (int j = 0; j < kHid / 8; ++j) {
                    uint32_t q[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const float h0 = fmaxf(v[8 * j + 2 * k] + b[8 * j + 2 * k], 0.0f);
                        const float h1 = fmaxf(v[8 * j + 2 * k + 1] + b[8 * j + 2 * k + 1], 0.0f);
                        q[k] = pack_bf16(h0, h1);
                        if (q[k] & 0x7fffu) mask[l] |= 1ull << (8 * j + 2 * k);
                        if (q[k] & 0x7fff0000u) mask[l] |= 1ull << (8 * j + 2 * k + 1);
                    }
                    *reinterpret_cast<uint4 *>(smem + xoff[l + 1] + canon_off(tid, 8 * j, kTcRows)) =
                        make_uint4(q[0], q[1], q[2], q[3]);
                }
            } else {
                float y[kOut], dy[kOut];
#pragma unroll
                for (int i = 0; i < kOut; ++i) {
                    y[i] = v[i] + b[i];
                    dy[i] = 0.0f;
                }
                float lterm = 0.0f;
                if (live) {
                    const float c = wmean > 0.0f ? weight[r] / wmean : 0.0f;
                    const float lq = guide_loss_grad(y, sdir[3 * (size_t)r], sdir[3 * (size_t)r + 1],
                                                     sdir[3 * (size_t)r + 2], c / (float)n, dy);
                    lterm = -c * lq / (float)n;
                }
                for (int o = 16; o > 0; o >>= 1) lterm += __shfl_down_sync(0xffffffffu, lterm, o);
                if (lane == 0) atomicAdd(loss, lterm);
                put_delta(dy, kOut);
            }
        }
        // backward: delta_{l-1} = (delta_l W_l) masked by the ReLU of layer
        // l-1, together with dW_l
        for (int l = kLayers - 1; l >= 1 && ok; --l) {
            const int K = fan_out(l);
            const bool acc = !first;
            ok = run([&] {
                tc_mma_chain(taddr, d_base, wt_base[l], kTcRows, kHid, K, false);
                tc_mma_chain(taddr, dlo_base, wt_base[l], kTcRows, kHid, K, true);
                wgrad(l, acc);
            });
            if (!ok) break;
            read_acc(v, 0, kHid);
            const uint64_t m = mask[l - 1];
#pragma unroll
            for (int i = 0; i < kHid; ++i)
                if (!((m >> i) & 1ull)) v[i] = 0.0f;
            put_delta(v, kHid);
        }
        if (ok) ok = run([&] { wgrad(0, !first); });
        first = false;
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    // add the CTA's weight gradients: rows m < 64 of dW_l carry the high part
    // of output m, rows 64 + m the low part
    if (ok && !first) {
        float *lo = reinterpret_cast<float *>(smem + kTfD);  // [64 rows][96]
        for (int l = 0; l < kLayers; ++l) {
            const int in = fan_in(l), N = in + 16, O = fan_out(l);
            float row[96];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                if (16 * c >= N) break;
                float t[16];
                tmem_ld16(lane_addr + tf_dcol(l) + 16 * c, t);
#pragma unroll
                for (int i = 0; i < 16; ++i) row[16 * c + i] = t[i];
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            __syncthreads();
            if (tid >= 64)
                for (int i = 0; i <= in; ++i) lo[(tid - 64) * 96 + i] = row[i];
            __syncthreads();
            if (tid < O) {
                float *G = grad + w_off(l) + (size_t)tid * in;
                for (int i = 0; i < in; ++i) atomicAdd(G + i, row[i] + lo[tid * 96 + i]);
                atomicAdd(grad + b_off(l) + tid, row[in] + lo[tid * 96 + in]);
            }
        }
    }
    if (!ok) {
        // MMAs or the weight copy still in flight: wait again (bounded) before freeing their memory
        mbar_wait(mbar, phase);
        mbar_wait(cbar, 0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(taddr) : "memory");
}

// Weight gradients of all layers in one launch (layer l = block z):
// dW[o][i] += sum over rows of deltaT[o][r] actT[i][r] (tensor cores, K = rows;
// delta as BF16 high + low parts), bias gradient db[o] += sum deltaT[o][r].
// Each warp computes one 16 x 8 tile (16 outputs, 8 inputs) over a chunk of
// kWgradRows rows and adds it with atomics; block x = (output tile, group of
// 4 input tiles), block y = row chunk. Measured per training step of 16,384
// rows: five launches of 256-row chunks 0.15 ms.
constexpr uint32_t kWgradRows = 512;

__host__ __device__ constexpr int wgrad_blocks_x(int l)
{
    return (l == kLayers - 1 ? kOut : kHid) / 16 * (((l == 0 ? kIn : kHid) / 8 + 3) / 4);
}

__global__ void __launch_bounds__(128) k_guide_wgrad(TrainBuffers tb, uint32_t n, float *grad)
{
    const int l = (int)blockIdx.z;
    if ((int)blockIdx.x >= wgrad_blocks_x(l)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int fan_in_l = l == 0 ? kIn : kHid;
    const int in_tiles = fan_in_l / 8, groups = (in_tiles + 3) / 4;
    const int o0 = 16 * (blockIdx.x / groups);
    const int it = 4 * (blockIdx.x % groups) + warp;
    const uint32_t k0 = kWgradRows * blockIdx.y, k1 = min(n, k0 + kWgradRows);
    const float *dT = tb.deltaT[l];
    const __nv_bfloat16 *aT = tb.actT[l];
    const uint32_t stride = tb.rows;
    if (it < in_tiles) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const __nv_bfloat16 *col = aT + (size_t)(8 * it + g) * stride;
        for (uint32_t k = k0; k < k1; k += 16) {
            // A[m = o][k = row]: a0 (o0+g, k+2tig..+1), a1 (o0+g+8, ...), a2 (o0+g, k+8+2tig..), a3 (o0+g+8, k+8+..)
            uint32_t ahi[4], alo[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int o = o0 + g + ((q & 1) ? 8 : 0);
                const uint32_t kk = k + 2 * tig + ((q & 2) ? 8 : 0);
                const float v0 = kk < k1 ? dT[(size_t)o * stride + kk] : 0.0f;
                const float v1 = kk + 1 < k1 ? dT[(size_t)o * stride + kk + 1] : 0.0f;
                const __nv_bfloat162 hb = __floats2bfloat162_rn(v0, v1);
                const float2 hf = __bfloat1622float2(hb);
                ahi[q] = *reinterpret_cast<const uint32_t *>(&hb);
                alo[q] = pack_bf16(v0 - hf.x, v1 - hf.y);
            }
            // B[k = row][n = input]: b0 (rows k+2tig..+1, input 8it+g), b1 (rows k+8+2tig..)
            const uint32_t kk = k + 2 * tig;
            uint32_t b0 = 0, b1 = 0;
            if (kk + 1 < k1) b0 = ld_pair(col + kk);
            else if (kk < k1) b0 = (uint32_t) * reinterpret_cast<const uint16_t *>(col + kk);
            if (kk + 9 < k1) b1 = ld_pair(col + kk + 8);
            else if (kk + 8 < k1) b1 = (uint32_t) * reinterpret_cast<const uint16_t *>(col + kk + 8);
            mma_bf16(acc, ahi, b0, b1);
            mma_bf16(acc, alo, b0, b1);
        }
        float *G = grad + w_off(l);
        const int i = 8 * it + 2 * tig;
        atomicAdd(&G[(o0 + g) * fan_in_l + i], acc[0]);
        atomicAdd(&G[(o0 + g) * fan_in_l + i + 1], acc[1]);
        atomicAdd(&G[(o0 + g + 8) * fan_in_l + i], acc[2]);
        atomicAdd(&G[(o0 + g + 8) * fan_in_l + i + 1], acc[3]);
    }
    // bias gradient: in the first input-tile group, warp 0's lanes 0..15 sum the
    // chunk's rows of outputs o0 + lane
    if (blockIdx.x % groups == 0 && warp == 0 && lane < 16) {
        float sum = 0.0f;
        const float *row = dT + (size_t)(o0 + lane) * stride;
        for (uint32_t k = k0; k < k1; ++k) sum += row[k];
        atomicAdd(grad + b_off(l) + o0 + lane, sum);
    }
}

// Sum of the sample weights into *sum (zeroed before).
__global__ void k_guide_weight_sum(const float *w, uint32_t n, float *sum)
{
    float v = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += w[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, v);
}

__global__ void k_guide_adam(float *params, float *m, float *v, const float *grad, int t, float lr, float b1, float b2,
                             float eps, __nv_bfloat16 *wb, unsigned char *img)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumParams) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    const float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    params[i] = p;
    // BF16 weight copy and weight image (biases stay FP32)
    for (int l = 0; l < kLayers; ++l)
        if (i >= w_off(l) && i < b_off(l)) store_weight(wb, img, l, i - w_off(l), p);
}

__global__ void k_guide_export(const float *params, __nv_bfloat16 *wb, unsigned char *img)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumParams) return;
    for (int l = 0; l < kLayers; ++l)
        if (i >= w_off(l) && i < b_off(l)) store_weight(wb, img, l, i - w_off(l), params[i]);
}

// The network input of each row (80 columns), as the forward pass forms it
// before rounding to BF16.
__global__ void k_guide_encode(GuideParams gp, const float *pos, const float *dir, uint32_t n, float *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 40u) return;
    const uint32_t r = i / 40, c = 2 * (i % 40);
    float p[3], d[3];
    uint32_t slot;
    load_row(pos, dir, nullptr, n, r, gp, p, d, slot);
    float v0, v1;
    encode_pair(p, d, (int)c, v0, v1);
    out[(size_t)r * kIn + c] = v0;
    out[(size_t)r * kIn + c + 1] = v1;
}

__global__ void k_guide_sample(const float *y, const float *u, uint32_t n, float *dir, float *pdf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GuideLobes L = guide_decode(y + (size_t)i * kGuideOut);
    float wx, wy, wz;
    guide_sample(L, u[3 * (size_t)i], u[3 * (size_t)i + 1], u[3 * (size_t)i + 2], wx, wy, wz);
    dir[3 * (size_t)i] = wx, dir[3 * (size_t)i + 1] = wy, dir[3 * (size_t)i + 2] = wz;
    pdf[i] = guide_pdf(L, wx, wy, wz);
}

__global__ void k_guide_pdf(const float *y, const float *dir, uint32_t n, uint32_t y_stride, float *pdf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GuideLobes L = guide_decode(y + (size_t)(y_stride ? i : 0) * kGuideOut);
    pdf[i] = guide_pdf(L, dir[3 * (size_t)i], dir[3 * (size_t)i + 1], dir[3 * (size_t)i + 2]);
}

constexpr size_t kInferSmem = sizeof(SmemWeights);
constexpr size_t kTrainSmem = sizeof(SmemWeights) + sizeof(SmemWeightsT) + 4 * 16 * kOut * sizeof(float);

}  // namespace
}  // namespace dr

struct dr_guide {
    dr_context *ctx = nullptr;
    dr_guide_config cfg{};
    float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    __nv_bfloat16 *wb = nullptr;
    unsigned char *img = nullptr;  // weight image of the tcgen05 kernels (kImgBytes)
    float *scalars = nullptr;  // [0] sum of the batch's sample weights, [1] loss
    dr::TrainBuffers tb{};
    void *tb_mem = nullptr;
    uint32_t capacity = 0;
    int step = 0;
};

using namespace dr;

namespace {

GuideParams guide_params(const dr_guide *g)
{
    GuideParams p{};
    for (int a = 0; a < 3; ++a) p.center[a] = g->cfg.center[a];
    p.half = g->cfg.half_extent > 0.0f ? g->cfg.half_extent : 1.0f;
    return p;
}

void free_guide(dr_guide *g)
{
    if (!g) return;
    cudaFree(g->params);
    cudaFree(g->m);
    cudaFree(g->v);
    cudaFree(g->grad);
    cudaFree(g->wb);
    cudaFree(g->img);
    cudaFree(g->scalars);
    cudaFree(g->tb_mem);
    delete g;
}

dr_status ensure_train_capacity(dr_guide *g, uint32_t n)
{
    if (n <= g->capacity) return DR_OK;
    DR_CUDA(cudaDeviceSynchronize());
    cudaFree(g->tb_mem);
    g->tb_mem = nullptr;
    g->capacity = 0;
    const uint32_t rows = (n + 63) & ~63u;
    size_t bytes = 0;
    for (int l = 0; l < kLayers; ++l) bytes += (size_t)fan_out(l) * rows * 4 + (size_t)fan_in(l) * rows * 2 + 512;
    DR_CUDA(dev_malloc(&g->tb_mem, bytes));
    char *p = static_cast<char *>(g->tb_mem);
    for (int l = 0; l < kLayers; ++l) {
        g->tb.deltaT[l] = reinterpret_cast<float *>(p);
        p += ((size_t)fan_out(l) * rows * 4 + 255) & ~size_t(255);
        g->tb.actT[l] = reinterpret_cast<__nv_bfloat16 *>(p);
        p += ((size_t)fan_in(l) * rows * 2 + 255) & ~size_t(255);
    }
    g->tb.rows = rows;
    g->capacity = rows;
    return DR_OK;
}

// loss and gradients (grad buffer) of one batch
dr_status run_gradients(dr_guide *g, const float *pos, const float *dir, const float *sdir, const float *weight,
                        uint32_t n, cudaStream_t st)
{
    // the per-layer delta and activation buffers serve the mma.sync path only
    // (the tcgen05 kernel keeps them on chip)
    if (g->cfg.infer_kernel == DR_GUIDE_INFER_MMA_SYNC) {
        const dr_status r = ensure_train_capacity(g, n);
        if (r != DR_OK) return r;
    }
    DR_CUDA(cudaMemsetAsync(g->grad, 0, kNumParams * sizeof(float), st));
    DR_CUDA(cudaMemsetAsync(g->scalars, 0, 2 * sizeof(float), st));
    k_guide_weight_sum<<<std::min<unsigned>((n + 255) / 256, 64), 256, 0, st>>>(weight, n, g->scalars);
    const GuideParams gp = guide_params(g);
    if (g->cfg.infer_kernel == DR_GUIDE_INFER_TCGEN05) {
        // one CTA per SM (its shared memory and 512 tensor-memory columns)
        const unsigned tiles = (n + kTcRows - 1) / kTcRows;
        const unsigned blocks = std::min<unsigned>(tiles, (unsigned)g->ctx->num_sms);
        k_guide_train_fused<<<blocks, 128, kTfSmem, st>>>(g->img, g->params, gp, pos, dir, sdir, weight, n,
                                                           g->scalars, g->grad, g->scalars + 1, g->ctx->d_error);
    } else {
        k_guide_train_fb<<<(n + 63) / 64, 128, kTrainSmem, st>>>(g->wb, g->params, gp, pos, dir, sdir, weight, n,
                                                                 g->scalars, g->tb, g->scalars + 1);
        int bx = 0;
        for (int l = 0; l < kLayers; ++l) bx = std::max(bx, wgrad_blocks_x(l));
        const dim3 grid((unsigned)bx, (n + kWgradRows - 1) / kWgradRows, (unsigned)kLayers);
        k_guide_wgrad<<<grid, 128, 0, st>>>(g->tb, n, g->grad);
    }
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

}  // namespace

namespace dr {

// Rewrites rows list[0 .. *count) of y (or rows 0 .. n_fixed) in the decoded
// layout, after the mma.sync inference (whose rows are spread over 4 lanes).
__global__ void __launch_bounds__(128) k_guide_decode_rows(const uint32_t *list, const uint32_t *count, uint32_t n_fixed,
                                                           float *y)
{
    const uint32_t n = count ? *count : n_fixed;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float *row = y + (size_t)(list ? list[i] : i) * kGuideOut;
        guide_store_decoded(row, guide_mix(row));
    }
}

cudaError_t launch_guide_infer(const dr_guide *g, const float *pos, const float *dir, const uint32_t *list,
                               const uint32_t *count, uint32_t max_rows, float *y, cudaStream_t st, bool decoded)
{
    if (max_rows == 0) return cudaSuccess;
    if (g->cfg.infer_kernel == DR_GUIDE_INFER_TCGEN05) {
        const unsigned tiles = (max_rows + kTcRows - 1) / kTcRows;
        const unsigned blocks = std::min<unsigned>(tiles, (unsigned)g->ctx->num_sms * DR_INFER_CTAS_PER_SM);
        k_guide_infer_tc<<<blocks, 128, kTcSmem, st>>>(g->img, g->params, guide_params(g), pos, dir, list, count,
                                                       max_rows, y, g->ctx->d_error, decoded);
    } else {
        const unsigned tiles = (max_rows + 15) / 16;
        const unsigned blocks = std::min<unsigned>((tiles + 3) / 4, (unsigned)g->ctx->num_sms * 4);
        k_guide_infer<<<blocks, 128, kInferSmem, st>>>(g->wb, g->params, guide_params(g), pos, dir, list, count,
                                                       max_rows, y);
        if (decoded)
            k_guide_decode_rows<<<std::min<unsigned>((max_rows + 127) / 128, (unsigned)g->ctx->num_sms * 8), 128, 0,
                                  st>>>(list, count, max_rows, y);
    }
    return cudaGetLastError();
}

uint32_t guide_steps(const dr_guide *g) { return (uint32_t)g->step; }

dr_status guide_train_step(dr_guide *g, const float *pos, const float *dir, const float *sdir, const float *weight,
                           uint32_t n, cudaStream_t st)
{
    return dr_guide_train_step(g, pos, dir, sdir, weight, n, st);
}

}  // namespace dr

extern "C" {

uint32_t dr_guide_num_params(void) { return (uint32_t)kNumParams; }

dr_status dr_guide_create(dr_context *ctx, const dr_guide_config *cfg, dr_guide **out)
{
    DR_CHECK_ARG(ctx && out, "dr_guide_create: NULL argument");
    *out = nullptr;
    DR_CUDA(cudaSetDevice(ctx->device));
    static bool attr = false;
    if (!attr) {
        DR_CUDA(cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
        DR_CUDA(cudaFuncSetAttribute(k_guide_train_fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
        DR_CUDA(cudaFuncSetAttribute(k_guide_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
        DR_CUDA(cudaFuncSetAttribute(k_guide_train_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTfSmem));
        attr = true;
    }
    auto *g = new (std::nothrow) dr_guide;
    if (!g) return fail(DR_ERR_OUT_OF_MEMORY, "dr_guide_create: host allocation failed");
    g->ctx = ctx;
    if (cfg) g->cfg = *cfg;
    if (g->cfg.learning_rate <= 0.0f) g->cfg.learning_rate = 1e-3f;
    if (g->cfg.beta1 <= 0.0f) g->cfg.beta1 = 0.9f;
    if (g->cfg.beta2 <= 0.0f) g->cfg.beta2 = 0.999f;
    if (g->cfg.epsilon <= 0.0f) g->cfg.epsilon = 1e-8f;
    if (g->cfg.half_extent <= 0.0f) g->cfg.half_extent = 1.0f;
    if (g->cfg.infer_kernel > DR_GUIDE_INFER_MMA_SYNC) {
        free_guide(g);
        return fail(DR_ERR_INVALID_ARGUMENT, "dr_guide_create: unknown inference kernel");
    }
    cudaError_t e;
    if ((e = dev_malloc(&g->params, kNumParams * 4)) != cudaSuccess || (e = dev_malloc(&g->m, kNumParams * 4)) != cudaSuccess ||
        (e = dev_malloc(&g->v, kNumParams * 4)) != cudaSuccess || (e = dev_malloc(&g->grad, kNumParams * 4)) != cudaSuccess ||
        (e = dev_malloc(&g->wb, kNumWeights * 2)) != cudaSuccess || (e = dev_malloc(&g->img, kImgBytes)) != cudaSuccess || (e = dev_malloc(&g->scalars, 16)) != cudaSuccess ||
        (e = cudaMemset(g->m, 0, kNumParams * 4)) != cudaSuccess || (e = cudaMemset(g->v, 0, kNumParams * 4)) != cudaSuccess ||
        (e = cudaMemset(g->scalars, 0, 16)) != cudaSuccess) {
        free_guide(g);
        return cuda_fail(e, "dr_guide_create");
    }
    // He-uniform initialisation (ReLU), last layer scaled by 0.1, zero biases
    std::mt19937_64 rng(g->cfg.seed);
    std::vector<float> p(kNumParams, 0.0f);
    for (int l = 0; l < kLayers; ++l) {
        const float bound = std::sqrt(6.0f / (float)fan_in(l)) * (l == kLayers - 1 ? 0.1f : 1.0f);
        std::uniform_real_distribution<float> U(-bound, bound);
        for (int i = 0; i < fan_out(l) * fan_in(l); ++i) p[w_off(l) + i] = U(rng);
    }
    const dr_status r = dr_guide_set_params(g, p.data(), kNumParams);
    if (r != DR_OK) {
        free_guide(g);
        return r;
    }
    *out = g;
    return DR_OK;
}

dr_status dr_guide_destroy(dr_guide *g)
{
    if (!g) return DR_OK;
    cudaSetDevice(g->ctx->device);
    cudaDeviceSynchronize();
    free_guide(g);
    return DR_OK;
}

dr_status dr_guide_set_params(dr_guide *g, const float *host, uint32_t n)
{
    DR_CHECK_ARG(g && host && n == (uint32_t)kNumParams, "dr_guide_set_params: bad argument");
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(cudaMemcpy(g->params, host, kNumParams * 4, cudaMemcpyHostToDevice));
    DR_CUDA(cudaMemset(g->m, 0, kNumParams * 4));
    DR_CUDA(cudaMemset(g->v, 0, kNumParams * 4));
    g->step = 0;
    k_guide_export<<<(kNumParams + 255) / 256, 256>>>(g->params, g->wb, g->img);
    DR_CUDA(cudaGetLastError());
    DR_CUDA(cudaDeviceSynchronize());
    return DR_OK;
}

// State blob: a header (magic, version, parameter count, Adam step), the
// configuration, then params, m and v (FP32, kNumParams each).
namespace {
constexpr uint32_t kStateMagic = 0x53475244u;  // "DRGS"
constexpr uint32_t kStateVersion = 1;
struct StateHeader {
    uint32_t magic, version, num_params, step;
    dr_guide_config cfg;
};
constexpr uint64_t kStateBytes = sizeof(StateHeader) + 3ull * kNumParams * sizeof(float);
}  // namespace

uint64_t dr_guide_state_bytes(void) { return kStateBytes; }

dr_status dr_guide_get_state(dr_guide *g, void *host, uint64_t bytes)
{
    DR_CHECK_ARG(g && host, "dr_guide_get_state: NULL argument");
    if (bytes != kStateBytes)
        return fail(DR_ERR_INVALID_ARGUMENT, "dr_guide_get_state: the state takes %llu bytes, got %llu",
                    (unsigned long long)kStateBytes, (unsigned long long)bytes);
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(cudaDeviceSynchronize());
    StateHeader h{kStateMagic, kStateVersion, (uint32_t)kNumParams, (uint32_t)g->step, g->cfg};
    auto *out = static_cast<unsigned char *>(host);
    memcpy(out, &h, sizeof h);
    float *f = reinterpret_cast<float *>(out + sizeof h);
    DR_CUDA(cudaMemcpy(f, g->params, kNumParams * 4, cudaMemcpyDeviceToHost));
    DR_CUDA(cudaMemcpy(f + kNumParams, g->m, kNumParams * 4, cudaMemcpyDeviceToHost));
    DR_CUDA(cudaMemcpy(f + 2 * kNumParams, g->v, kNumParams * 4, cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_guide_set_state(dr_guide *g, const void *host, uint64_t bytes)
{
    DR_CHECK_ARG(g && host, "dr_guide_set_state: NULL argument");
    if (bytes != kStateBytes)
        return fail(DR_ERR_INVALID_ARGUMENT, "dr_guide_set_state: the state takes %llu bytes, got %llu",
                    (unsigned long long)kStateBytes, (unsigned long long)bytes);
    StateHeader h;
    memcpy(&h, host, sizeof h);
    DR_CHECK_ARG(h.magic == kStateMagic && h.version == kStateVersion && h.num_params == (uint32_t)kNumParams,
                 "dr_guide_set_state: not a guiding-network state of this version");
    const float *f = reinterpret_cast<const float *>(static_cast<const unsigned char *>(host) + sizeof h);
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(cudaDeviceSynchronize());
    DR_CUDA(cudaMemcpy(g->params, f, kNumParams * 4, cudaMemcpyHostToDevice));
    DR_CUDA(cudaMemcpy(g->m, f + kNumParams, kNumParams * 4, cudaMemcpyHostToDevice));
    DR_CUDA(cudaMemcpy(g->v, f + 2 * kNumParams, kNumParams * 4, cudaMemcpyHostToDevice));
    g->cfg = h.cfg;
    g->step = (int)h.step;
    k_guide_export<<<(kNumParams + 255) / 256, 256>>>(g->params, g->wb, g->img);
    DR_CUDA(cudaGetLastError());
    DR_CUDA(cudaDeviceSynchronize());
    return DR_OK;
}

dr_status dr_guide_get_params(dr_guide *g, float *host, uint32_t n)
{
    DR_CHECK_ARG(g && host && n == (uint32_t)kNumParams, "dr_guide_get_params: bad argument");
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(cudaDeviceSynchronize());
    DR_CUDA(cudaMemcpy(host, g->params, kNumParams * 4, cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_guide_infer(dr_guide *g, const float *pos_dev, const float *dir_dev, uint32_t n, float *y_dev, void *stream)
{
    DR_CHECK_ARG(g && (n == 0 || (pos_dev && dir_dev && y_dev)), "dr_guide_infer: NULL argument");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(launch_guide_infer(g, pos_dev, dir_dev, nullptr, nullptr, n, y_dev, static_cast<cudaStream_t>(stream)));
    return DR_OK;
}

dr_status dr_guide_gradients(dr_guide *g, const float *pos_dev, const float *dir_dev, const float *sdir_dev,
                             const float *weight_dev, uint32_t n, float *loss_host, float *grad_host)
{
    DR_CHECK_ARG(g && n > 0 && pos_dev && dir_dev && sdir_dev && weight_dev, "dr_guide_gradients: bad argument");
    DR_CUDA(cudaSetDevice(g->ctx->device));
    dr_status r = run_gradients(g, pos_dev, dir_dev, sdir_dev, weight_dev, n, nullptr);
    if (r != DR_OK) return r;
    DR_CUDA(cudaDeviceSynchronize());
    if (loss_host) DR_CUDA(cudaMemcpy(loss_host, g->scalars + 1, 4, cudaMemcpyDeviceToHost));
    if (grad_host) DR_CUDA(cudaMemcpy(grad_host, g->grad, kNumParams * 4, cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_guide_train_step(dr_guide *g, const float *pos_dev, const float *dir_dev, const float *sdir_dev,
                              const float *weight_dev, uint32_t n, void *stream)
{
    DR_CHECK_ARG(g && pos_dev && dir_dev && sdir_dev && weight_dev, "dr_guide_train_step: NULL argument");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(g->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    dr_status r = run_gradients(g, pos_dev, dir_dev, sdir_dev, weight_dev, n, st);
    if (r != DR_OK) return r;
    ++g->step;
    const float lr = g->cfg.warmup_steps && (uint32_t)g->step < g->cfg.warmup_steps
                         ? g->cfg.learning_rate * (float)g->step / (float)g->cfg.warmup_steps
                         : g->cfg.learning_rate;
    k_guide_adam<<<(kNumParams + 255) / 256, 256, 0, st>>>(g->params, g->m, g->v, g->grad, g->step, lr,
                                                           g->cfg.beta1, g->cfg.beta2, g->cfg.epsilon, g->wb, g->img);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_guide_encode(dr_guide *g, const float *pos_dev, const float *dir_dev, uint32_t n, float *out_dev)
{
    DR_CHECK_ARG(g && (n == 0 || (pos_dev && dir_dev && out_dev)), "dr_guide_encode: NULL argument");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(g->ctx->device));
    k_guide_encode<<<(n * 40 + 255) / 256, 256>>>(guide_params(g), pos_dev, dir_dev, n, out_dev);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_guide_mixture_sample(const float *y_dev, const float *u_dev, uint32_t n, float *dir_dev, float *pdf_dev,
                                  void *stream)
{
    DR_CHECK_ARG(n == 0 || (y_dev && u_dev && dir_dev && pdf_dev), "dr_guide_mixture_sample: NULL argument");
    if (n == 0) return DR_OK;
    k_guide_sample<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(y_dev, u_dev, n, dir_dev, pdf_dev);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_guide_mixture_pdf(const float *y_dev, uint32_t y_per_row, const float *dir_dev, uint32_t n, float *pdf_dev,
                               void *stream)
{
    DR_CHECK_ARG(n == 0 || (y_dev && dir_dev && pdf_dev), "dr_guide_mixture_pdf: NULL argument");
    if (n == 0) return DR_OK;
    k_guide_pdf<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(y_dev, dir_dev, n, y_per_row, pdf_dev);
    DR_CUDA(cudaGetLastError());
    return DR_OK;
}

dr_status dr_guide_last_loss(dr_guide *g, float *loss_host)
{
    DR_CHECK_ARG(g && loss_host, "dr_guide_last_loss: NULL argument");
    DR_CUDA(cudaSetDevice(g->ctx->device));
    DR_CUDA(cudaMemcpy(loss_host, g->scalars + 1, 4, cudaMemcpyDeviceToHost));
    return DR_OK;
}

}  // extern "C"
