// tri_device.cuh -- device ray/box and ray/triangle tests for sm_103a.
//
// This header is compiled with -fmad=false: no multiply/add pair is contracted
// into an FMA unless written as fmaf(), so the triangle tests below round
// exactly like the FP32 source expressions they restate.
#pragma once

#include "dr_internal.h"

#include <cmath>
#include <cstdint>

#if defined(__CUDA_ARCH__)
#define DR_LDG(p) __ldg(p)
#else
#define DR_LDG(p) (*(p))
#endif

namespace dr {

struct DevRay {
    float3 o, v, inv, ooi;
    float tmax;
};

// Reciprocal that maps a zero (or denormal) direction component to +-1e30 so
// slab times stay finite and ordered.
__host__ __device__ __forceinline__ float safe_rcp(float x)
{
    return 1.0f / (fabsf(x) >= 1e-30f ? x : copysignf(1e-30f, x));
}

// Ray from values (origin, direction, tmax); false for a non-finite origin or
// direction, or a zero direction.
__host__ __device__ __forceinline__ bool make_dev_ray(float3 o, float3 v, float tmax, DevRay &r)
{
    r.o = o;
    r.tmax = tmax;
    r.v = v;
    r.inv = make_float3(safe_rcp(v.x), safe_rcp(v.y), safe_rcp(v.z));
    r.ooi = make_float3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
    using std::isfinite;
    const bool finite = isfinite(o.x) && isfinite(o.y) && isfinite(o.z) && isfinite(v.x) && isfinite(v.y) &&
                        isfinite(v.z);
    const bool nonzero = !(v.x == 0.0f && v.y == 0.0f && v.z == 0.0f);
    return finite && nonzero;
}

// Ray i of a GLOBAL-memory dr_ray array (read through the read-only path).
__host__ __device__ __forceinline__ bool load_ray(const dr_ray *rays, uint64_t i, DevRay &r)
{
    const float4 *p = reinterpret_cast<const float4 *>(rays) + 2 * i;
    const float4 a = DR_LDG(p), b = DR_LDG(p + 1);
    return make_dev_ray(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), a.w, r);
}

// Relative margin of the box tests: a child counts as hit when its entry time
// is at most kBoxFarScale x its exit time. The FP32 slab times carry an error
// of a few ulps of |t| (the reciprocal, the origin term and the final
// rounding); a margin of 2^-19 |t| covers it at any distance of the ray origin,
// and the slack of the stored boxes covers the part proportional to the box
// coordinates. Boxes accepted in excess only cost extra visits.
constexpr float kBoxFarScale = 1.0f + 0x1p-19f;

// Slab test of both children of a two-box node against [0, tmax]. Boxes are
// stored widened (conservative) and the exit time carries kBoxFarScale, so
// the FMA form of the slab times is safe.
__host__ __device__ __forceinline__ void intersect_children(const float4 c0xy, const float4 c1xy, const float4 cz,
                                                   const DevRay &r, float tmax,
                                                   float &t0, float &t1, bool &h0, bool &h1)
{
    const float a0 = fmaf(c0xy.x, r.inv.x, -r.ooi.x), a1 = fmaf(c0xy.y, r.inv.x, -r.ooi.x);
    const float b0 = fmaf(c0xy.z, r.inv.y, -r.ooi.y), b1 = fmaf(c0xy.w, r.inv.y, -r.ooi.y);
    const float d0 = fmaf(cz.x, r.inv.z, -r.ooi.z), d1 = fmaf(cz.y, r.inv.z, -r.ooi.z);
    const float e0 = fmaf(c1xy.x, r.inv.x, -r.ooi.x), e1 = fmaf(c1xy.y, r.inv.x, -r.ooi.x);
    const float f0 = fmaf(c1xy.z, r.inv.y, -r.ooi.y), f1 = fmaf(c1xy.w, r.inv.y, -r.ooi.y);
    const float g0 = fmaf(cz.z, r.inv.z, -r.ooi.z), g1 = fmaf(cz.w, r.inv.z, -r.ooi.z);
    const float lo0 = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(d0, d1), 0.0f));
    const float hi0 = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(d0, d1), tmax));
    const float lo1 = fmaxf(fmaxf(fminf(e0, e1), fminf(f0, f1)), fmaxf(fminf(g0, g1), 0.0f));
    const float hi1 = fminf(fminf(fmaxf(e0, e1), fmaxf(f0, f1)), fminf(fmaxf(g0, g1), tmax));
    h0 = lo0 <= hi0 * kBoxFarScale;
    h1 = lo1 <= hi1 * kBoxFarScale;
    t0 = lo0;
    t1 = lo1;
}

// testTriangleIntersection (DevilRay include/tracing/IntersectionTestsImpl.hpp:
// 253-297) on a precomputed record {A, n, B-A, C-A} given as its three float4
// words. The t of a hit and the hit/miss decision are bit-identical to the
// reference; the test stops after t when t cannot beat (best_t, best_prim)
// under the smaller-t-then-smaller-index rule. Returns true when the triangle
// beats the current best.
__host__ __device__ __forceinline__ bool tri_test_ref_words(const float4 r0, const float4 r1, const float4 r2,
                                                            const DevRay &r, float best_t, float &t_out)
{
    float nx = r0.w, ny = r1.x, nz = r1.y;
    const float px = r.o.x - r0.x, py = r.o.y - r0.y, pz = r.o.z - r0.z;
    float dp = px * nx + py * ny + pz * nz;
    if (dp < 0) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
        dp = -dp;
    }
    const float d = -(r.v.x * nx + r.v.y * ny + r.v.z * nz);
    if (d < 1e-7f) return false;
    const float t = dp / d;
    if (!(t <= best_t)) return false;
    const float BAx = r1.z, BAy = r1.w, BAz = r2.x;
    const float CAx = r2.y, CAy = r2.z, CAz = r2.w;
    const float hx = r.o.x + r.v.x * t, hy = r.o.y + r.v.y * t, hz = r.o.z + r.v.z * t;
    const float ax = hx - r0.x, ay = hy - r0.y, az = hz - r0.z;
    // n_1 = (p - A) x (C - A), n_2 = (B - A) x (p - A), n_f = (A - B) x (A - C)
    const float n1x = ay * CAz - az * CAy, n1y = az * CAx - ax * CAz, n1z = ax * CAy - ay * CAx;
    const float n2x = BAy * az - BAz * ay, n2y = BAz * ax - BAx * az, n2z = BAx * ay - BAy * ax;
    const float nfx = BAy * CAz - BAz * CAy, nfy = BAz * CAx - BAx * CAz, nfz = BAx * CAy - BAy * CAx;
    const float s = nfx * nfx + nfy * nfy + nfz * nfz;
    const float wB = (nfx * n1x + nfy * n1y + nfz * n1z) / s;
    const float wC = (nfx * n2x + nfy * n2y + nfz * n2z) / s;
    const float wA = 1 - wB - wC;
    if (wA < 0 || wB < 0 || wC < 0) return false;
    t_out = t;
    return true;
}

// The same on record k of a GLOBAL-memory record array (read-only path; the
// third word is read only when t can still beat the best).
__host__ __device__ __forceinline__ bool tri_test_ref(const float4 *__restrict__ rec, uint32_t k, const DevRay &r,
                                             float best_t, float &t_out)
{
    const float4 r0 = DR_LDG(rec + 3 * k);
    const float4 r1 = DR_LDG(rec + 3 * k + 1);
    float nx = r0.w, ny = r1.x, nz = r1.y;
    const float px = r.o.x - r0.x, py = r.o.y - r0.y, pz = r.o.z - r0.z;
    float dp = px * nx + py * ny + pz * nz;
    if (dp < 0) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
        dp = -dp;
    }
    const float d = -(r.v.x * nx + r.v.y * ny + r.v.z * nz);
    if (d < 1e-7f) return false;
    const float t = dp / d;
    if (!(t <= best_t)) return false;
    return tri_test_ref_words(r0, r1, DR_LDG(rec + 3 * k + 2), r, best_t, t_out);
}

// Per-ray setup of the watertight test (Woop, Benthin, Wald, JCGT 2013).
struct WtSetup {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__host__ __device__ __forceinline__ float comp(const float3 &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

__host__ __device__ __forceinline__ WtSetup wt_setup(const float3 &d)
{
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    if (comp(d, kz) < 0.0f) {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    WtSetup w;
    w.kx = kx;
    w.ky = ky;
    w.kz = kz;
    const float dz = comp(d, kz);
    w.Sx = comp(d, kx) / dz;
    w.Sy = comp(d, ky) / dz;
    w.Sz = 1.0f / dz;
    return w;
}

// Watertight two-sided test on a record {A, B, C} given as its three float4 words.
__host__ __device__ __forceinline__ bool tri_test_wt_words(const float4 r0, const float4 r1, const float4 r2,
                                                           const DevRay &r, const WtSetup &w, float best_t,
                                                           float &t_out)
{
    const float3 a = make_float3(r0.x - r.o.x, r0.y - r.o.y, r0.z - r.o.z);
    const float3 b = make_float3(r0.w - r.o.x, r1.x - r.o.y, r1.y - r.o.z);
    const float3 c = make_float3(r1.z - r.o.x, r1.w - r.o.y, r2.x - r.o.z);
    const float akz = comp(a, w.kz), bkz = comp(b, w.kz), ckz = comp(c, w.kz);
    const float Ax = comp(a, w.kx) - w.Sx * akz;
    const float Ay = comp(a, w.ky) - w.Sy * akz;
    const float Bx = comp(b, w.kx) - w.Sx * bkz;
    const float By = comp(b, w.ky) - w.Sy * bkz;
    const float Cx = comp(c, w.kx) - w.Sx * ckz;
    const float Cy = comp(c, w.ky) - w.Sy * ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = w.Sz * akz, Bz = w.Sz * bkz, Cz = w.Sz * ckz;
    const float T = U * Az + V * Bz + W * Cz;
    if (det < 0.0f ? T > 0.0f : T < 0.0f) return false;
    const float rcp = 1.0f / det;
    const float t = T * rcp;
    if (!(t <= best_t)) return false;
    t_out = t;
    return true;
}

// The same on record k of a GLOBAL-memory record array.
__host__ __device__ __forceinline__ bool tri_test_wt(const float4 *__restrict__ rec, uint32_t k, const DevRay &r,
                                            const WtSetup &w, float best_t, float &t_out)
{
    return tri_test_wt_words(DR_LDG(rec + 3 * k), DR_LDG(rec + 3 * k + 1), DR_LDG(rec + 3 * k + 2), r, w, best_t,
                             t_out);
}

}  // namespace dr
