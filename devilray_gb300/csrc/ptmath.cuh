// ptmath.cuh -- portable FP32 sin/cos/acos and the Philox4x32-10 generator,
// usable on host and device.
//
// The reference samples directions with std::sin/std::cos/std::acos
// (include/tracing/DistributionSamplers.hpp:8-20); platform math libraries
// round those differently, so the renderer evaluates them with the
// polynomials below instead. Every step is an FP32 add, multiply, divide or
// sqrt with IEEE round-to-nearest (no FMA contraction), so host and device
// produce the same bits. Accuracy: <= 1.5 ulp for sin/cos on [0, 2pi],
// <= 1.3 ulp for acos on [-1, 1] (coefficients: ptmath_coefficients.py;
// range reduction after Cody and Waite, "Software Manual for the Elementary
// Functions", 1980).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DR_HD __host__ __device__ __forceinline__
#else
#define DR_HD inline
#endif

namespace dr {
namespace pt {

DR_HD float poly_s(float t)
{
    return -0.166666672f + t * (0.00833333191f + t * (-0.00019840071f + t * 2.72486977e-06f));
}

DR_HD float poly_c(float t)
{
    return -0.5f + t * (0.0416666679f + t * (-0.00138888799f + t * (2.47987373e-05f + t * -2.71550363e-07f)));
}

DR_HD float poly_a(float t)
{
    return 0.166666672f +
           t * (0.0749999434f +
                t * (0.0446470045f +
                     t * (0.0302793793f + t * (0.0235377513f + t * (0.0108257942f + t * 0.0306509901f)))));
}

DR_HD float round_half_even(float x)
{
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return __builtin_rintf(x);
#endif
}

DR_HD float sqrt_rn(float x)
{
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}

// sin and cos of x (|x| < 2^11).
DR_HD void sincos(float x, float &s, float &c)
{
    const float k = round_half_even(x * 0.636619772f);
    const float r = ((x - k * 1.5703125f) - k * 0.000483826792f) - k * 2.56328292e-12f;
    const float r2 = r * r;
    const float sr = r + (r * r2) * poly_s(r2);
    const float cr = 1.0f + r2 * poly_c(r2);
    const int q = ((int)k) & 3;
    if (q == 0) {
        s = sr;
        c = cr;
    } else if (q == 1) {
        s = cr;
        c = -sr;
    } else if (q == 2) {
        s = -sr;
        c = -cr;
    } else {
        s = -cr;
        c = sr;
    }
}

DR_HD float asin_small(float x)
{
    const float t = x * x;
    return x + (x * t) * poly_a(t);
}

// acos(z) for z in [-1, 1].
DR_HD float acos(float z)
{
    const float az = z < 0.0f ? -z : z;
    if (az <= 0.5f) return 1.57079637f - asin_small(z);
    if (z > 0.0f) return 2.0f * asin_small(sqrt_rn((1.0f - z) * 0.5f));
    return 3.14159274f - 2.0f * asin_small(sqrt_rn((1.0f + z) * 0.5f));
}

// Philox4x32 with 10 rounds (Salmon, Moraes, Dror and Shaw, "Parallel Random
// Numbers: As Easy as 1, 2, 3", SC 2011).
DR_HD void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                         uint32_t out[4])
{
    for (int round = 0; round < 10; ++round) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// 24-bit uniform in [0, 1).
DR_HD float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }

}  // namespace pt
}  // namespace dr
