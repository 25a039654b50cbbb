// oracle_ptmath.hpp -- the oracle's copy of the portable FP32 sin/cos/acos
// and of the integrator's random-number layout (TEST INFRASTRUCTURE).
//
// The GPU renderer evaluates the reference's sphere sampling with fixed
// polynomials (sin/cos: Taylor-like fits on |r| <= pi/4 after Cody-Waite
// reduction; acos through asin on |x| <= 1/2) and draws its uniforms from
// Philox4x32-10 indexed by (pixel, sample, dimension). The oracle restates the
// same arithmetic here so both sides produce the same bits; the oracle can also
// use the platform's std::sin/std::cos/std::acos (the reference's own calls).
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle {
namespace ptm {

inline float poly_s(float t) { return -0.166666672f + t * (0.00833333191f + t * (-0.00019840071f + t * 2.72486977e-06f)); }
inline float poly_c(float t)
{
    return -0.5f + t * (0.0416666679f + t * (-0.00138888799f + t * (2.47987373e-05f + t * -2.71550363e-07f)));
}
inline float poly_a(float t)
{
    return 0.166666672f +
           t * (0.0749999434f +
                t * (0.0446470045f +
                     t * (0.0302793793f + t * (0.0235377513f + t * (0.0108257942f + t * 0.0306509901f)))));
}

inline void sincos(float x, float &s, float &c)
{
    const float k = std::nearbyint(x * 0.636619772f);
    const float r = ((x - k * 1.5703125f) - k * 0.000483826792f) - k * 2.56328292e-12f;
    const float r2 = r * r;
    const float sr = r + (r * r2) * poly_s(r2);
    const float cr = 1.0f + r2 * poly_c(r2);
    const int q = ((int)k) & 3;
    if (q == 0) { s = sr; c = cr; }
    else if (q == 1) { s = cr; c = -sr; }
    else if (q == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
}

inline float asin_small(float x)
{
    const float t = x * x;
    return x + (x * t) * poly_a(t);
}

inline float acos(float z)
{
    const float az = z < 0.0f ? -z : z;
    if (az <= 0.5f) return 1.57079637f - asin_small(z);
    if (z > 0.0f) return 2.0f * asin_small(std::sqrt((1.0f - z) * 0.5f));
    return 3.14159274f - 2.0f * asin_small(std::sqrt((1.0f + z) * 0.5f));
}

inline void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4])
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
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

inline float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }

// Dimension layout of one path sample: camera jitter 0,1; bounce b uses
// base = 4 + 12 b: +0,+1 sphere sample, +2 Fresnel, +3,+4 light object,
// +5,+6 light triangle, +7,+8 point on the triangle.
constexpr uint32_t kStreamTag = 0x44526E67u;
inline uint32_t dim_camera(int k) { return (uint32_t)k; }
inline uint32_t dim_bounce(int b, int k) { return 4u + 12u * (uint32_t)b + (uint32_t)k; }

inline float uniform(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim)
{
    uint32_t out[4];
    philox(pixel, sample, dim >> 2, kStreamTag, (uint32_t)seed, (uint32_t)(seed >> 32), out);
    return u01(out[dim & 3]);
}

}  // namespace ptm
}  // namespace oracle
