// trace_wide.cuh -- closest-hit and any-hit traversal of the compressed
// 8-wide BVH (node layout in dr_internal.h).
//
// After Ylitie, Karras and Laine (HPG 2017): a ray keeps the current "node
// group" (the internal children of one node still to visit, as a bit mask in
// the ray's octant order) and the "triangle group" (the hit leaf triangles of
// the last node, as a 24-bit mask). One node fetch tests 8 child boxes, which
// the lanes of a warp do in lockstep. Culling and the candidate rule are the
// same as the binary traversal (enter <= best, smaller t or equal t with a
// smaller triangle index), so the result equals a brute-force scan.
#pragma once

#include "dr_internal.h"
#include "tri_device.cuh"

#include <climits>
#include <cstring>

#if defined(__CUDA_ARCH__)
#define DR_LD(p) __ldg(p)
#else
#define DR_LD(p) (*(p))
#endif

namespace dr {

struct Wide8Args {
    const Bvh8Node *nodes;
    const float4 *tri_ref;
    const float4 *tri_wt;
    const int32_t *prim;
    uint32_t num_nodes;
    uint32_t *error;
    uint32_t stack_limit;  // stack entries a ray may use (kWideStack; lower only for tests)
};

constexpr int kWideStack = 64;

// Per-child decisions of the node test as selects instead of branches
// (measured: 3.71 vs 3.74 Grays/s, so off).
#ifndef DR_NODE_SELECTS
#define DR_NODE_SELECTS 0
#endif
// Hit masks without a per-child internal/leaf branch: 1 = each child ORs its
// metadata's hit-mask bits; 2 = each child sets its slot bit and the hit leaf
// slots' metadata is read after the loop (measured: 4.38 -> 4.43 Grays/s).
#ifndef DR_NODE_META_BITS
#define DR_NODE_META_BITS 2
#endif
// Slab times from byte permutes folded into one FMA per plane (slab_axis).
#ifndef DR_FAST_SLAB
#define DR_FAST_SLAB 1
#endif
// Packed FP32 pairs (fma.rn.f32x2) for the slab FMAs of slots j and j + 4:
// each half rounds as the scalar FMA does, so results are unchanged. At 64
// registers the pairs spill (4.86 -> 4.61 Grays/s); the public kernels turn
// them on with a 73-register budget (trace.cu), the renderer keeps them off.
#ifndef DR_PACKED_SLAB
#define DR_PACKED_SLAB 0
#endif
// Grid planes through FP16 in the closest-hit traversal of the persistent
// kernels: one byte permute places bytes j and j + 2 of a plane word under
// FP16 exponent bits (1024 + q, exact), two conversions (cvt.f32.f16) make
// them FP32, so half of the extraction leaves the ALU pipe (the busiest: 69 %
// of cycles) for the FMA pipe; the slab constants fold 1024 instead of 2^15
// (slab_axis_h). Measured on the incoherent workload (2^20 triangles, 16.8 M
// rays): closest hit 3.334 -> 3.269 ms; any hit 2.843 -> 2.915 ms, so any-hit
// traversal keeps the byte permutes.
#ifndef DR_HALF_CVT
#define DR_HALF_CVT 1
#endif
// FP16 path only: near/far plane words chosen by integer multiply-adds on the
// FMA pipe instead of selects (DR_SEL_IMAD; it spills: 3.269 -> 3.417 ms),
// and the hit bits accumulated by FP32 FMAs of set.le.f32 results instead of
// predicated ORs (DR_HIT_FSET: 3.269 -> 3.192 ms on the incoherent workload).
#ifndef DR_SEL_IMAD
#define DR_SEL_IMAD 0
#endif
#ifndef DR_HIT_FSET
#define DR_HIT_FSET 1
#endif
// Independent accumulators of the FMA hit bits (1, 2 or 4), summed at the end
// (exact: distinct powers of two below 256). Measured on the incoherent
// workload: 1 chain 3.194-3.195 ms, 2 chains 3.215-3.216 ms; 4 spill.
#ifndef DR_HIT_CHAINS
#define DR_HIT_CHAINS 1
#endif
// The FP16 path's slab FMAs as scalar FMAs instead of packed pairs (fewer
// registers). Measured: 3.283 ms at 7 blocks per SM, 3.371 ms at 8 (64
// registers, spills); packed pairs 3.192 ms at 7 blocks, 3.308 ms at 8.
#ifndef DR_HALF_SCALAR
#define DR_HALF_SCALAR 0
#endif
// The same accumulation in the packed and scalar node tests (any hit,
// renderer): measured without effect (any hit 2.842 / 2.844 ms), so off.
#ifndef DR_HIT_FSET_ALL
#define DR_HIT_FSET_ALL 0
#endif
// Children in slot order instead of the ray's octant order (off: an
// experiment; results are the same, only the visiting order changes).
#ifndef DR_NO_OCT_ORDER
#define DR_NO_OCT_ORDER 0
#endif
// The internal hit mask moved from slot to traversal order (bit s -> bit
// s ^ oct) by one lookup in a 2 KB shared-memory table per block
// instead of three conditional swaps, in the persistent kernels: 1 all of
// them, 2 the any-hit ones. Measured on the incoherent workload: any hit
// 2.842 -> 2.791 ms with the table; closest hit 3.192 -> 3.307 ms, and
// 3.275 / 3.285 ms with 6 / 4 shared stack entries, which give back the L1
// the table takes (with the table the closest-hit kernel spills 26 bytes at
// its 72 registers). So only the any-hit kernels use it (many-light 1080p
// render, 16 spp: 40.46-40.55 -> 40.40-40.43 ms).
#ifndef DR_OCT_LUT
#define DR_OCT_LUT 2
#endif
// (Measured and dropped, same workload: the children in slot order instead of
// the ray's octant order, 3.19 -> 3.71 ms; 128-byte nodes that store the
// grid planes as FP16 words, so that no byte permute or near/far select is
// left, 3.96 ms: the node loads cost more than the instructions saved.)
// Prefetch into L1 of the next sibling node when a node is chosen (off).
#ifndef DR_PREFETCH_NEXT
#define DR_PREFETCH_NEXT 0
#endif
// Three-input min/max instructions in the box test.
#ifndef DR_MINMAX3
#define DR_MINMAX3 1
#endif

// Byte j of w as a float. On the device: a byte permute builds the FP32 bit
// pattern of 2^23 + byte, and one exact subtraction removes 2^23 (avoids the
// integer-to-float conversion pipe).
__host__ __device__ __forceinline__ float byte_f(uint32_t w, int j)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (uint32_t)j)) - 8388608.0f;
#else
    return (float)((w >> (8 * j)) & 0xffu);
#endif
}

// 2^23 + 256 * (byte j of w), exactly, as a float: one byte permute, no
// conversion and no subtraction (the offset is folded into the slab constants).
__host__ __device__ __forceinline__ float byte_q(uint32_t w, int j)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7404u | ((uint32_t)j << 4)));
#else
    const uint32_t bits = 0x4B000000u | (((w >> (8 * j)) & 0xffu) << 8);
    float f;
    memcpy(&f, &bits, 4);
    return f;
#endif
}

// Three-input minimum and maximum (one instruction each on sm_100 and later).
__host__ __device__ __forceinline__ float max3f(float a, float b, float c)
{
#if defined(__CUDA_ARCH__) && DR_MINMAX3
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}

__host__ __device__ __forceinline__ float min3f(float a, float b, float c)
{
#if defined(__CUDA_ARCH__) && DR_MINMAX3
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

__host__ __device__ __forceinline__ float exp2_bits(uint32_t biased)
{
    const uint32_t bits = biased << 23;
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

__host__ __device__ __forceinline__ float bits_f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

__host__ __device__ __forceinline__ int lowest_bit(uint32_t m)
{
#if defined(__CUDA_ARCH__)
    return __ffs(m) - 1;
#else
    return __builtin_ctz(m);
#endif
}

__host__ __device__ __forceinline__ int popcount(uint32_t m)
{
#if defined(__CUDA_ARCH__)
    return __popc(m);
#else
    return __builtin_popcount(m);
#endif
}

__host__ __device__ __forceinline__ uint32_t nonzero_bytes(uint32_t x)
{
    return ((x & 0xffu) != 0u) + ((x & 0xff00u) != 0u) + ((x & 0xff0000u) != 0u) + ((x & 0xff000000u) != 0u);
}

// Slab constants of one axis for the folded evaluation t = fma(byte_q, A, B):
// with a = grid step * 1/d and b = (node origin - o) * 1/d, the plain slab time
// of grid plane q is fl(q * a + b). Here A = a / 256 (exact) and
// B = fl(b - 2^15 a) -+ off, so that byte_q(q) * A + B = q * a + b + (B - X)
// where X = b - 2^15 a exactly. The rounding of X is at most 2^-24 |X| and that
// of B at most 2^-24 |B|, so off = 2^-21 |fl(X)| + 1e-30 keeps the near time at
// or below, and the far time at or above, the plain times (rounding is
// monotonic): every box the plain test accepts is accepted, and the traversal
// result is unchanged.
struct SlabAxis {
    float a, near_b, far_b;
};

__host__ __device__ __forceinline__ SlabAxis slab_axis(float a, float b)
{
    const float x = fmaf(-32768.0f, a, b);
    const float off = fmaf(fabsf(x), 0x1p-21f, 1e-30f);
    return SlabAxis{a * 0.00390625f, x - off, x + off};
}

// The same constants for grid values 1024 + q (DR_HALF_CVT): A = a,
// B = fl(b - 1024 a) -+ off, with the bound of slab_axis.
__host__ __device__ __forceinline__ SlabAxis slab_axis_h(float a, float b)
{
    const float x = fmaf(-1024.0f, a, b);
    const float off = fmaf(fabsf(x), 0x1p-21f, 1e-30f);
    return SlabAxis{a, x - off, x + off};
}

#if defined(__CUDA_ARCH__)
// 1.0f when a <= b, else 0.0f (false for NaN operands, as the comparison)
__device__ __forceinline__ float set_le(float a, float b)
{
    float r;
    asm("set.le.f32.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ uint32_t mad_u32(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// Bytes j and j + 2 of w as the FP32 values 1024 + q (j = 0 or 1).
__device__ __forceinline__ float2 byte_pair_h(uint32_t w, uint32_t j)
{
    const uint32_t h = __byte_perm(w, 0x64u, 0x4240u + 0x101u * j);
    float lo, hi;
    asm("{\n .reg .b16 l, h;\n mov.b32 {l, h}, %2;\n cvt.f32.f16 %0, l;\n cvt.f32.f16 %1, h;\n}" : "=f"(lo), "=f"(hi) : "r"(h));
    return make_float2(lo, hi);
}
#endif

// Tests the 8 child boxes of `node` against [0, tmax]; returns the internal
// hit mask in traversal order (bit k = slot k ^ oct) and the triangle mask.
// HALF: grid planes through FP16 (DR_HALF_CVT).
template <bool HALF = false, bool LUT = false>
__host__ __device__ __forceinline__ void wide_node_test(const Bvh8Node *node, const DevRay &r, uint32_t oct, float tmax,
                                                        uint32_t &child_base, uint32_t &imask, uint32_t &hit_internal,
                                                        uint32_t &tri_base, uint32_t &tri_mask, uint32_t &nboxes,
                                                        const uint8_t *oct_lut = nullptr)
{
    const uint4 w0 = DR_LD(&node->w[0]);
    const uint4 w1 = DR_LD(&node->w[1]);
    const uint4 wx = DR_LD(&node->w[2]);
    const uint4 wy = DR_LD(&node->w[3]);
    const uint4 wz = DR_LD(&node->w[4]);
    const float px = bits_f(w0.x), py = bits_f(w0.y), pz = bits_f(w0.z);
    const float sx = exp2_bits(w0.w & 0xffu), sy = exp2_bits((w0.w >> 8) & 0xffu), sz = exp2_bits((w0.w >> 16) & 0xffu);
    imask = w0.w >> 24;
    child_base = w1.x;
    tri_base = w1.y;
    // slab time of grid coordinate q on each axis: t = q * a + b
    const float ax = sx * r.inv.x, ay = sy * r.inv.y, az = sz * r.inv.z;
    const float bx = (px - r.o.x) * r.inv.x, by = (py - r.o.y) * r.inv.y, bz = (pz - r.o.z) * r.inv.z;
#if DR_FAST_SLAB
    const SlabAxis cx = slab_axis(ax, bx), cy = slab_axis(ay, by), cz = slab_axis(az, bz);
#endif
    // near/far words by direction sign
    const bool fx = r.inv.x < 0.0f, fy = r.inv.y < 0.0f, fz = r.inv.z < 0.0f;
    const uint32_t nx0 = fx ? wx.z : wx.x, nx1 = fx ? wx.w : wx.y, fx0 = fx ? wx.x : wx.z, fx1 = fx ? wx.y : wx.w;
    const uint32_t ny0 = fy ? wy.z : wy.x, ny1 = fy ? wy.w : wy.y, fy0 = fy ? wy.x : wy.z, fy1 = fy ? wy.y : wy.w;
    const uint32_t nz0 = fz ? wz.z : wz.x, nz1 = fz ? wz.w : wz.y, fz0 = fz ? wz.x : wz.z, fz1 = fz ? wz.y : wz.w;
    hit_internal = 0;
    tri_mask = 0;
    uint32_t boxes = 0, hit_bits = 0;
#if DR_FAST_SLAB && DR_NODE_META_BITS == 2 && defined(__CUDA_ARCH__)
    if (HALF) {
#if DR_SEL_IMAD
    // s = 1 for a negative direction: near = lo + s (hi - lo), far = hi - s (hi - lo)
    const uint32_t sgx = __float_as_uint(r.inv.x) >> 31, sgy = __float_as_uint(r.inv.y) >> 31,
                   sgz = __float_as_uint(r.inv.z) >> 31;
    const uint32_t ngx = 0u - sgx, ngy = 0u - sgy, ngz = 0u - sgz, m1 = 0xffffffffu;
    const uint32_t dx0 = mad_u32(wx.x, m1, wx.z), dx1 = mad_u32(wx.y, m1, wx.w);
    const uint32_t dy0 = mad_u32(wy.x, m1, wy.z), dy1 = mad_u32(wy.y, m1, wy.w);
    const uint32_t dz0 = mad_u32(wz.x, m1, wz.z), dz1 = mad_u32(wz.y, m1, wz.w);
    const uint32_t hnx0 = mad_u32(sgx, dx0, wx.x), hnx1 = mad_u32(sgx, dx1, wx.y);
    const uint32_t hfx0 = mad_u32(ngx, dx0, wx.z), hfx1 = mad_u32(ngx, dx1, wx.w);
    const uint32_t hny0 = mad_u32(sgy, dy0, wy.x), hny1 = mad_u32(sgy, dy1, wy.y);
    const uint32_t hfy0 = mad_u32(ngy, dy0, wy.z), hfy1 = mad_u32(ngy, dy1, wy.w);
    const uint32_t hnz0 = mad_u32(sgz, dz0, wz.x), hnz1 = mad_u32(sgz, dz1, wz.y);
    const uint32_t hfz0 = mad_u32(ngz, dz0, wz.z), hfz1 = mad_u32(ngz, dz1, wz.w);
#else
    const uint32_t hnx0 = nx0, hnx1 = nx1, hfx0 = fx0, hfx1 = fx1, hny0 = ny0, hny1 = ny1, hfy0 = fy0, hfy1 = fy1;
    const uint32_t hnz0 = nz0, hnz1 = nz1, hfz0 = fz0, hfz1 = fz1;
#endif
#if DR_HIT_FSET
    float hit_acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#endif
    // slots 4h + j and 4h + j + 2 (bytes j and j + 2 of word h) as pairs
    const SlabAxis hx = slab_axis_h(ax, bx), hy = slab_axis_h(ay, by), hz = slab_axis_h(az, bz);
    const float2 Ax = make_float2(hx.a, hx.a), NBx = make_float2(hx.near_b, hx.near_b),
                 FBx = make_float2(hx.far_b, hx.far_b);
    const float2 Ay = make_float2(hy.a, hy.a), NBy = make_float2(hy.near_b, hy.near_b),
                 FBy = make_float2(hy.far_b, hy.far_b);
    const float2 Az = make_float2(hz.a, hz.a), NBz = make_float2(hz.near_b, hz.near_b),
                 FBz = make_float2(hz.far_b, hz.far_b);
    const float2 farS = make_float2(kBoxFarScale, kBoxFarScale);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (uint32_t j = 0; j < 2; ++j) {
#if DR_HALF_SCALAR
            auto ffma_s = [](float2 q, float2 a, float2 b) { return make_float2(fmaf(q.x, a.x, b.x), fmaf(q.y, a.y, b.y)); };
            const float2 tnx = ffma_s(byte_pair_h(h ? hnx1 : hnx0, j), Ax, NBx);
            const float2 tfx = ffma_s(byte_pair_h(h ? hfx1 : hfx0, j), Ax, FBx);
            const float2 tny = ffma_s(byte_pair_h(h ? hny1 : hny0, j), Ay, NBy);
            const float2 tfy = ffma_s(byte_pair_h(h ? hfy1 : hfy0, j), Ay, FBy);
            const float2 tnz = ffma_s(byte_pair_h(h ? hnz1 : hnz0, j), Az, NBz);
            const float2 tfz = ffma_s(byte_pair_h(h ? hfz1 : hfz0, j), Az, FBz);
            const float2 tmx = make_float2(fminf(min3f(tfx.x, tfy.x, tfz.x), tmax) * kBoxFarScale,
                                           fminf(min3f(tfx.y, tfy.y, tfz.y), tmax) * kBoxFarScale);
#else
            const float2 tnx = __ffma2_rn(byte_pair_h(h ? hnx1 : hnx0, j), Ax, NBx);
            const float2 tfx = __ffma2_rn(byte_pair_h(h ? hfx1 : hfx0, j), Ax, FBx);
            const float2 tny = __ffma2_rn(byte_pair_h(h ? hny1 : hny0, j), Ay, NBy);
            const float2 tfy = __ffma2_rn(byte_pair_h(h ? hfy1 : hfy0, j), Ay, FBy);
            const float2 tnz = __ffma2_rn(byte_pair_h(h ? hnz1 : hnz0, j), Az, NBz);
            const float2 tfz = __ffma2_rn(byte_pair_h(h ? hfz1 : hfz0, j), Az, FBz);
            const float2 tmx = __fmul2_rn(make_float2(fminf(min3f(tfx.x, tfy.x, tfz.x), tmax),
                                                      fminf(min3f(tfx.y, tfy.y, tfz.y), tmax)), farS);
#endif
            const uint32_t s0 = 4u * h + j;
#if DR_HIT_FSET
            float &hit_f = hit_acc[DR_HIT_CHAINS == 4 ? 2 * h + (int)j : DR_HIT_CHAINS == 2 ? h : 0];
            hit_f = fmaf(set_le(fmaxf(max3f(tnx.x, tny.x, tnz.x), 0.0f), tmx.x), (float)(1u << s0),
                         fmaf(set_le(fmaxf(max3f(tnx.y, tny.y, tnz.y), 0.0f), tmx.y), (float)(1u << (s0 + 2)), hit_f));
#else
            if (fmaxf(max3f(tnx.x, tny.x, tnz.x), 0.0f) <= tmx.x) hit_bits |= 1u << s0;
            if (fmaxf(max3f(tnx.y, tny.y, tnz.y), 0.0f) <= tmx.y) hit_bits |= 1u << (s0 + 2);
#endif
        }
    }
#if DR_HIT_FSET
    // a sum of distinct powers of two below 256 is exact: 2^23 + sum has it in
    // its low mantissa bits
    const float hit_f = DR_HIT_CHAINS == 4   ? (hit_acc[0] + hit_acc[1]) + (hit_acc[2] + hit_acc[3])
                        : DR_HIT_CHAINS == 2 ? hit_acc[0] + hit_acc[1]
                                             : hit_acc[0];
    hit_bits = __float_as_uint(hit_f + 8388608.0f) & 0xffu;
#endif
    } else
#endif
    {
#if DR_PACKED_SLAB && DR_FAST_SLAB && DR_NODE_META_BITS == 2 && defined(__CUDA_ARCH__)
    // slots j and j + 4 share byte j of the two words of each plane: their six
    // slab FMAs and the far-time scaling run as packed FP32 pairs (each lane of
    // a pair rounds as the scalar instruction would)
    const float2 Ax = make_float2(cx.a, cx.a), NBx = make_float2(cx.near_b, cx.near_b),
                 FBx = make_float2(cx.far_b, cx.far_b);
    const float2 Ay = make_float2(cy.a, cy.a), NBy = make_float2(cy.near_b, cy.near_b),
                 FBy = make_float2(cy.far_b, cy.far_b);
    const float2 Az = make_float2(cz.a, cz.a), NBz = make_float2(cz.near_b, cz.near_b),
                 FBz = make_float2(cz.far_b, cz.far_b);
    const float2 farS = make_float2(kBoxFarScale, kBoxFarScale);
#if DR_HIT_FSET_ALL
    float hit_f = 0.0f;
#endif
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 tnx = __ffma2_rn(make_float2(byte_q(nx0, j), byte_q(nx1, j)), Ax, NBx);
        const float2 tfx = __ffma2_rn(make_float2(byte_q(fx0, j), byte_q(fx1, j)), Ax, FBx);
        const float2 tny = __ffma2_rn(make_float2(byte_q(ny0, j), byte_q(ny1, j)), Ay, NBy);
        const float2 tfy = __ffma2_rn(make_float2(byte_q(fy0, j), byte_q(fy1, j)), Ay, FBy);
        const float2 tnz = __ffma2_rn(make_float2(byte_q(nz0, j), byte_q(nz1, j)), Az, NBz);
        const float2 tfz = __ffma2_rn(make_float2(byte_q(fz0, j), byte_q(fz1, j)), Az, FBz);
        const float2 tmx = __fmul2_rn(make_float2(fminf(min3f(tfx.x, tfy.x, tfz.x), tmax),
                                                  fminf(min3f(tfx.y, tfy.y, tfz.y), tmax)), farS);
#if DR_HIT_FSET_ALL
        hit_f = fmaf(set_le(fmaxf(max3f(tnx.x, tny.x, tnz.x), 0.0f), tmx.x), (float)(1u << j),
                     fmaf(set_le(fmaxf(max3f(tnx.y, tny.y, tnz.y), 0.0f), tmx.y), (float)(1u << (j + 4)), hit_f));
#else
        if (fmaxf(max3f(tnx.x, tny.x, tnz.x), 0.0f) <= tmx.x) hit_bits |= 1u << j;
        if (fmaxf(max3f(tnx.y, tny.y, tnz.y), 0.0f) <= tmx.y) hit_bits |= 1u << (j + 4);
#endif
    }
#if DR_HIT_FSET_ALL
    hit_bits = __float_as_uint(hit_f + 8388608.0f) & 0xffu;
#endif
#else
#if DR_HIT_FSET_ALL && defined(__CUDA_ARCH__)
    float hit_fs = 0.0f;
#endif
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int j = s & 3;
        const uint32_t wnx = s < 4 ? nx0 : nx1, wfx = s < 4 ? fx0 : fx1;
        const uint32_t wny = s < 4 ? ny0 : ny1, wfy = s < 4 ? fy0 : fy1;
        const uint32_t wnz = s < 4 ? nz0 : nz1, wfz = s < 4 ? fz0 : fz1;
#if DR_FAST_SLAB
        const float tnx = fmaf(byte_q(wnx, j), cx.a, cx.near_b), tfx = fmaf(byte_q(wfx, j), cx.a, cx.far_b);
        const float tny = fmaf(byte_q(wny, j), cy.a, cy.near_b), tfy = fmaf(byte_q(wfy, j), cy.a, cy.far_b);
        const float tnz = fmaf(byte_q(wnz, j), cz.a, cz.near_b), tfz = fmaf(byte_q(wfz, j), cz.a, cz.far_b);
#else
        const float tnx = fmaf(byte_f(wnx, j), ax, bx), tfx = fmaf(byte_f(wfx, j), ax, bx);
        const float tny = fmaf(byte_f(wny, j), ay, by), tfy = fmaf(byte_f(wfy, j), ay, by);
        const float tnz = fmaf(byte_f(wnz, j), az, bz), tfz = fmaf(byte_f(wfz, j), az, bz);
#endif
        const float tmin = fmaxf(max3f(tnx, tny, tnz), 0.0f);
        const float tmx = fminf(min3f(tfx, tfy, tfz), tmax) * kBoxFarScale;
#if DR_NODE_META_BITS == 2
        // one bit per slot; the metadata is read after the loop
#if DR_HIT_FSET_ALL && defined(__CUDA_ARCH__)
        hit_fs = fmaf(set_le(tmin, tmx), (float)(1u << s), hit_fs);
#else
        if (tmin <= tmx) hit_bits |= 1u << s;
#endif
#else
        const uint32_t meta = ((s < 4 ? w1.z : w1.w) >> (8 * j)) & 0xffu;
        if (meta != 0) ++boxes;
#endif
#if DR_NODE_META_BITS == 2
#elif DR_NODE_META_BITS
        // the child's bits of the node's hit mask: its triangles (bits 0-23)
        // or, for an internal child, bit 24 + s; an empty slot has none
        if (tmin <= tmx) hit_bits |= (meta >> 5) << (meta & 31u);
#elif DR_NODE_SELECTS
        // the same decisions as selects (no per-child branches)
        const uint32_t hit = (tmin <= tmx && meta != 0) ? 1u : 0u;
        const uint32_t internal = (imask >> s) & 1u;
        hit_internal |= (hit & internal) << (s ^ oct);
        tri_mask |= (hit & (internal ^ 1u)) ? (meta >> 5) << (meta & 31u) : 0u;
#else
        if (tmin <= tmx && meta != 0) {
            if ((imask >> s) & 1u) hit_internal |= 1u << (s ^ oct);
            else tri_mask |= (meta >> 5) << (meta & 31u);
        }
#endif
    }
#if DR_HIT_FSET_ALL && defined(__CUDA_ARCH__) && DR_NODE_META_BITS == 2
    hit_bits = __float_as_uint(hit_fs + 8388608.0f) & 0xffu;
#endif
#endif
    }
#if DR_NODE_META_BITS
#if DR_NODE_META_BITS == 2
    // leaf slots hit: their triangle bits from the metadata; empty slots have
    // metadata 0 and add nothing
    for (uint32_t lm = hit_bits & ~imask & 0xffu; lm != 0; lm &= lm - 1u) {
        const uint32_t sl = (uint32_t)lowest_bit(lm);
        const uint32_t meta = ((sl < 4 ? w1.z : w1.w) >> (8 * (sl & 3u))) & 0xffu;
        tri_mask |= (meta >> 5) << (meta & 31u);
    }
    boxes = nonzero_bytes(w1.z) + nonzero_bytes(w1.w);  // read by counting builds only
    uint32_t m = hit_bits & imask;
#else
    tri_mask = hit_bits & 0x00ffffffu;
    uint32_t m = hit_bits >> 24;
#endif
    // internal hits from slot order to traversal order: bit s -> bit s ^ oct
#if !DR_NO_OCT_ORDER
    if (LUT) {
        m = oct_lut[(oct << 8) | m];
    } else {
        if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
        if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
        if (oct & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    }
#endif
    hit_internal = m;
#endif
    nboxes = boxes;
}

__host__ __device__ __forceinline__ uint32_t ray_octant(const DevRay &r)
{
    return (r.v.x < 0.0f ? 1u : 0u) | (r.v.y < 0.0f ? 2u : 0u) | (r.v.z < 0.0f ? 4u : 0u);
}

// Resumable traversal state of one ray (for the persistent kernels).
struct WideState {
    DevRay r;
    WtSetup w;
    uint32_t oct, node;
    float best_t;
    int32_t best_prim;
    uint2 group;
    int sp;
    bool have_node;
    uint32_t tbase, tmask;  // triangles waiting to be tested (persistent kernels)
};

template <int MODE>
__host__ __device__ __forceinline__ void wide_init(WideState &s, const DevRay &r, uint32_t root)
{
    s.r = r;
    if (MODE == 1) s.w = wt_setup(r.v);
    s.oct = DR_NO_OCT_ORDER ? 0u : ray_octant(r);
    s.best_t = r.tmax;
    s.best_prim = INT_MAX;
    s.node = root;
    s.group = make_uint2(0, 0);
    s.sp = 0;
    s.have_node = true;
    s.tbase = 0;
    s.tmask = 0;
}

// Stack entry of a postponed triangle group: y carries this flag above the
// triangle mask (node groups keep y < 2^16).
constexpr uint32_t kTriGroupFlag = 0x80000000u;

// Node test of the persistent kernels: the node's internal hits become the
// current group, its hit leaf triangles the pending triangle group.
template <int MODE, bool HALF = false, bool LUT = false>
__device__ __forceinline__ void wide_visit(const Wide8Args &a, WideState &s, unsigned long long &nn,
                                           unsigned long long &nb, const uint8_t *oct_lut = nullptr)
{
    uint32_t child_base, imask, hit_int, nbx, tri_base, tri_mask;
    wide_node_test<HALF, LUT>(a.nodes + s.node, s.r, s.oct, s.best_t, child_base, imask, hit_int, tri_base, tri_mask,
                              nbx, oct_lut);
    ++nn;
    nb += nbx;
    s.group = make_uint2(child_base, (hit_int << 8) | imask);
    s.tbase = tri_base;
    s.tmask = tri_mask;
    s.have_node = false;
}

// Tests the pending triangles; true when an any-hit query is answered.
template <int MODE, bool ANY>
__device__ __forceinline__ bool wide_triangles(const Wide8Args &a, WideState &s, unsigned long long &nt)
{
    uint32_t m = s.tmask;
    s.tmask = 0;
    while (m) {
        const int b = lowest_bit(m);
        m &= m - 1u;
        const uint32_t k = s.tbase + (uint32_t)b;
        ++nt;
        float t;
        const bool ok = MODE == 1 ? tri_test_wt(a.tri_wt, k, s.r, s.w, ANY ? s.r.tmax : s.best_t, t)
                                  : tri_test_ref(a.tri_ref, k, s.r, ANY ? s.r.tmax : s.best_t, t);
        if (ok) {
            if (ANY) return true;
            const int32_t prim = DR_LD(a.prim + k);
            if (t < s.best_t || prim < s.best_prim) {
                s.best_t = t;
                s.best_prim = prim;
            }
        }
    }
    return false;
}

// Traversal stack of one lane in the persistent kernels: the first S entries
// in shared memory (a per-warp array, one column per lane: 256 B per entry
// and warp), the rest in local memory. Measured on the incoherent workload:
// local only 3.74, 8 entries 3.83, 16 entries 3.82 Grays/s (before the later
// node-test changes); 4 and 8 entries 4.37 Grays/s after them; with the
// FP16 planes and FMA hit bits, closest hit 0 / 4 / 8 entries 3.233 / 3.200 /
// 3.192 ms (4 entries leave the SM more L1 and gain nothing). The public
// kernels use DR_SMEM_STACK entries; the renderer's depth is a schedule knob
// (dr_render_config.stack), chosen by the autotuner.
#ifndef DR_SMEM_STACK
#define DR_SMEM_STACK 8
#endif
template <int S>
struct LaneStackT {
    uint2 *shared;  // this lane's column: entry i at shared[32 * i]
    uint2 local[kWideStack > S ? kWideStack - S : 1];
    __device__ __forceinline__ void put(int i, uint2 v)
    {
        if (S > 0 && i < S) shared[32 * i] = v;
        else local[i - S] = v;
    }
    __device__ __forceinline__ uint2 get(int i) const
    {
        if (S > 0 && i < S) return shared[32 * i];
        return local[i - S];
    }
};
using LaneStack = LaneStackT<DR_SMEM_STACK>;

// Next node: from the current group, else from the stack (a popped triangle
// group becomes pending and is tested first). True when the ray is finished.
template <bool ANY, class Stack>
__device__ __forceinline__ bool wide_advance(const Wide8Args &a, WideState &s, Stack &stack)
{
    if ((s.group.y >> 8) == 0) {
        if (s.sp == 0) return true;
        const uint2 e = stack.get(--s.sp);
        if (e.y & kTriGroupFlag) {
            s.tbase = e.x;
            s.tmask = e.y & ~kTriGroupFlag;
            return false;
        }
        s.group = e;
    }
    const uint32_t hits = s.group.y >> 8;
    const int k = lowest_bit(hits);
    const uint32_t rest = hits & (hits - 1u);
    const uint32_t slot = (uint32_t)k ^ s.oct;
    const uint32_t imask = s.group.y & 0xffu;
    s.node = s.group.x + (uint32_t)popcount(imask & ((1u << slot) - 1u));
    s.have_node = true;
    s.group.y = (rest << 8) | imask;
#if DR_PREFETCH_NEXT && defined(__CUDA_ARCH__)
    if (rest) {
        // the next sibling is likely the node after this one: start its fetch
        const uint32_t slot2 = (uint32_t)lowest_bit(rest) ^ s.oct;
        const Bvh8Node *nx = a.nodes + s.group.x + (uint32_t)popcount(imask & ((1u << slot2) - 1u));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(nx));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(reinterpret_cast<const char *>(nx) + 64));
    }
#endif
    if (rest) {
        if ((uint32_t)s.sp >= a.stack_limit) {
            atomicOr(a.error, ERR_STACK_OVERFLOW);
            return true;
        }
        stack.put(s.sp++, s.group);
        s.group.y = imask;
    }
    return false;
}

// Node group on the stack: x = child_base, y = (internal hit mask << 8) | imask.
template <int MODE, bool ANY>
__host__ __device__ __forceinline__ bool wide_traverse(const Wide8Args &a, const DevRay &r, uint32_t root,
                                                       float &best_t, int32_t &best_prim,
                                                       unsigned long long *nodes_out, unsigned long long *boxes_out,
                                                       unsigned long long *tris_out)
{
    best_t = r.tmax;
    best_prim = INT_MAX;
    if (root == kNoRoot) return false;
    WtSetup w;
    if (MODE == 1) w = wt_setup(r.v);
    const uint32_t oct = DR_NO_OCT_ORDER ? 0u : ray_octant(r);
    uint2 stack[kWideStack];
    int sp = 0;
    // the root is visited directly
    uint32_t node = root;
    bool have_node = true;
    uint2 group = make_uint2(0, 0);
    unsigned long long nn = 0, nb = 0, nt = 0;
    while (true) {
        uint32_t tri_base = 0, tri_mask = 0;
        if (have_node) {
            uint32_t child_base, imask, hit_int, nbx;
            wide_node_test(a.nodes + node, r, oct, best_t, child_base, imask, hit_int, tri_base, tri_mask, nbx);
            ++nn;
            nb += nbx;
            group = make_uint2(child_base, (hit_int << 8) | imask);
            have_node = false;
        }
        // triangles of the last node
        while (tri_mask) {
            const int b = lowest_bit(tri_mask);
            tri_mask &= tri_mask - 1u;
            const uint32_t k = tri_base + (uint32_t)b;
            ++nt;
            float t;
            const bool ok = MODE == 1 ? tri_test_wt(a.tri_wt, k, r, w, ANY ? r.tmax : best_t, t)
                                      : tri_test_ref(a.tri_ref, k, r, ANY ? r.tmax : best_t, t);
            if (ok) {
                if (ANY) {
                    if (nodes_out) {
                        *nodes_out += nn;
                        *boxes_out += nb;
                        *tris_out += nt;
                    }
                    return true;
                }
                const int32_t prim = DR_LD(a.prim + k);
                if (t < best_t || prim < best_prim) {
                    best_t = t;
                    best_prim = prim;
                }
            }
        }
        // next internal child: from the current group, else from the stack
        if ((group.y >> 8) == 0) {
            if (sp == 0) break;
            group = stack[--sp];
        }
        const uint32_t hits = group.y >> 8;
        const int k = lowest_bit(hits);
        const uint32_t rest = hits & (hits - 1u);
        const uint32_t slot = (uint32_t)k ^ oct;
        const uint32_t imask = group.y & 0xffu;
        node = group.x + (uint32_t)popcount(imask & ((1u << slot) - 1u));
        have_node = true;
        group.y = (rest << 8) | imask;
        if (rest) {
            if ((uint32_t)sp >= a.stack_limit) {
#if defined(__CUDA_ARCH__)
                atomicOr(a.error, ERR_STACK_OVERFLOW);
#endif
                break;
            }
            stack[sp++] = group;
            group.y = imask;  // the current group is now empty
        }
    }
    if (nodes_out) {
        *nodes_out += nn;
        *boxes_out += nb;
        *tris_out += nt;
    }
    return false;
}

}  // namespace dr
