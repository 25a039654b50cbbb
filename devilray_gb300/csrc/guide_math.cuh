// guide_math.cuh -- the 8-lobe von Mises-Fisher mixture of the path-guiding
// network: decoding the network output, density, sampling and the gradient of
// the training loss. Device and host (the host side serves tests).
//
// Output y of the network, per lobe j: y[5j] logit (weights = softmax),
// y[5j+1] log-concentration (kappa = exp(clamp(., -4, 7))), y[5j+2..5j+4] the
// unnormalised mean direction. vMF density on the unit sphere:
//   p(w) = kappa / (2 pi (1 - e^{-2 kappa})) exp(kappa (mu . w - 1)).
// Sampling follows Jakob, "Numerically stable sampling of the von Mises
// Fisher distribution on S^2" (2012).
#pragma once

#include <cmath>
#include <cstdint>

namespace dr {

constexpr int kGuideLobes = 8;
constexpr int kGuideOut = 40;      // used outputs
constexpr float kGuideLogKMin = -4.0f, kGuideLogKMax = 7.0f;

struct GuideLobes {
    float pi[kGuideLobes];
    float kappa[kGuideLobes];
    float mu[kGuideLobes][3];
};

__host__ __device__ inline float guide_exp(float x) { return expf(x); }

__host__ __device__ inline GuideLobes guide_decode(const float *y)
{
    GuideLobes L;
    float mx = y[0];
    for (int j = 1; j < kGuideLobes; ++j) mx = fmaxf(mx, y[5 * j]);
    float s = 0.0f;
    for (int j = 0; j < kGuideLobes; ++j) {
        L.pi[j] = guide_exp(y[5 * j] - mx);
        s += L.pi[j];
    }
    const float inv = 1.0f / s;
    for (int j = 0; j < kGuideLobes; ++j) {
        L.pi[j] *= inv;
        L.kappa[j] = guide_exp(fminf(fmaxf(y[5 * j + 1], kGuideLogKMin), kGuideLogKMax));
        const float mx3 = y[5 * j + 2], my = y[5 * j + 3], mz = y[5 * j + 4];
        const float n2 = mx3 * mx3 + my * my + mz * mz;
        if (n2 < 1e-24f) {
            L.mu[j][0] = 0.0f, L.mu[j][1] = 0.0f, L.mu[j][2] = 1.0f;
        } else {
            const float r = 1.0f / sqrtf(n2);
            L.mu[j][0] = mx3 * r, L.mu[j][1] = my * r, L.mu[j][2] = mz * r;
        }
    }
    return L;
}

// vMF density of one lobe at cosine c between mean and direction.
__host__ __device__ inline float vmf_pdf(float kappa, float c)
{
    // kappa / (2 pi (1 - e^{-2 kappa})): for small kappa use the series 1 / (4 pi (1 - kappa + ...))
    const float e2 = guide_exp(-2.0f * kappa);
    const float norm = kappa > 1e-3f ? kappa / (6.28318530718f * (1.0f - e2)) : 1.0f / (12.5663706144f * (1.0f - kappa));
    return norm * guide_exp(kappa * (c - 1.0f));
}

__host__ __device__ inline float guide_pdf(const GuideLobes &L, float wx, float wy, float wz)
{
    float p = 0.0f;
    for (int j = 0; j < kGuideLobes; ++j) {
        const float c = L.mu[j][0] * wx + L.mu[j][1] * wy + L.mu[j][2] * wz;
        p += L.pi[j] * vmf_pdf(L.kappa[j], c);
    }
    return p;
}

// Samples the vMF lobe of concentration k and unit mean (mx, my, mz) from
// (u1, u2).
__host__ __device__ inline void vmf_sample(float k, float mx, float my, float mz, float u1, float u2, float &wx,
                                           float &wy, float &wz)
{
    // cosine to the mean: w = 1 + log(u1 + (1 - u1) e^{-2k}) / k
    float w = 1.0f + logf(u1 + (1.0f - u1) * guide_exp(-2.0f * k)) / k;
    w = fminf(fmaxf(w, -1.0f), 1.0f);
    const float sr = sqrtf(fmaxf(0.0f, 1.0f - w * w));
    const float phi = 6.28318530718f * u2;
    float sp, cp;
#if defined(__CUDA_ARCH__)
    sincosf(phi, &sp, &cp);
#else
    sp = sinf(phi);
    cp = cosf(phi);
#endif
    // orthonormal basis around mu (Duff et al., "Building an Orthonormal Basis, Revisited", 2017)
    const float sign = copysignf(1.0f, mz);
    const float a = -1.0f / (sign + mz);
    const float b = mx * my * a;
    const float t1x = 1.0f + sign * mx * mx * a, t1y = sign * b, t1z = -sign * mx;
    const float t2x = b, t2y = sign + my * my * a, t2z = -my;
    wx = w * mx + sr * (cp * t1x + sp * t2x);
    wy = w * my + sr * (cp * t1y + sp * t2y);
    wz = w * mz + sr * (cp * t1z + sp * t2z);
}

// Samples a direction: lobe by u0, then the lobe's vMF from (u1, u2).
__host__ __device__ inline void guide_sample(const GuideLobes &L, float u0, float u1, float u2, float &wx, float &wy,
                                             float &wz)
{
    int j = 0;
    float acc = L.pi[0];
    while (j < kGuideLobes - 1 && u0 >= acc) {
        ++j;
        acc += L.pi[j];
    }
    vmf_sample(L.kappa[j], L.mu[j][0], L.mu[j][1], L.mu[j][2], u1, u2, wx, wy, wz);
}

// Loss term -c log q(w) of one sample and its gradient with respect to y
// (scale = c / batch size); returns log q.
__host__ __device__ inline float guide_loss_grad(const float *y, float wx, float wy, float wz, float scale, float *dy)
{
    const GuideLobes L = guide_decode(y);
    float t[kGuideLobes], cosang[kGuideLobes];
    float mx = -3.0e38f;
    for (int j = 0; j < kGuideLobes; ++j) {
        cosang[j] = L.mu[j][0] * wx + L.mu[j][1] * wy + L.mu[j][2] * wz;
        const float k = L.kappa[j];
        const float lognorm = k > 1e-3f ? logf(k) - 1.83787706641f - log1pf(-guide_exp(-2.0f * k))
                                         : -2.53102424697f - log1pf(-k);
        t[j] = logf(L.pi[j]) + lognorm + k * (cosang[j] - 1.0f);
        mx = fmaxf(mx, t[j]);
    }
    float s = 0.0f;
    for (int j = 0; j < kGuideLobes; ++j) s += guide_exp(t[j] - mx);
    const float logq = mx + logf(s);
    for (int j = 0; j < kGuideLobes; ++j) {
        const float resp = guide_exp(t[j] - logq);
        dy[5 * j] = -scale * (resp - L.pi[j]);
        const float k = L.kappa[j];
        const float r = y[5 * j + 1];
        const bool clamped = r < kGuideLogKMin || r > kGuideLogKMax;
        // d log p / d kappa = 1/kappa - 2 / (e^{2 kappa} - 1) + cos - 1
        const float dk = 1.0f / k - 2.0f / expm1f(2.0f * k) + cosang[j] - 1.0f;
        dy[5 * j + 1] = clamped ? 0.0f : -scale * resp * dk * k;
        const float m0 = y[5 * j + 2], m1 = y[5 * j + 3], m2 = y[5 * j + 4];
        const float n = sqrtf(m0 * m0 + m1 * m1 + m2 * m2);
        if (n < 1e-12f) {
            dy[5 * j + 2] = dy[5 * j + 3] = dy[5 * j + 4] = 0.0f;
        } else {
            const float g = -scale * resp * k / n;
            dy[5 * j + 2] = g * (wx - cosang[j] * L.mu[j][0]);
            dy[5 * j + 3] = g * (wy - cosang[j] * L.mu[j][1]);
            dy[5 * j + 4] = g * (wz - cosang[j] * L.mu[j][2]);
        }
    }
    return logq;
}

#if defined(__CUDACC__)
// The mixture as the shading kernel uses it: the network output decoded once
// per vertex, each lobe's vMF normalisation folded into its weight, so that a
// density evaluation costs one exponential per lobe. Every loop over the lobes
// is unrolled with constant indices, which keeps the mixture in registers (a
// lobe picked by a run-time index would put the whole mixture in local memory).
struct GuideMix {
    float c[kGuideLobes];      // pi_j kappa_j / (2 pi (1 - e^{-2 kappa_j}))
    float pi[kGuideLobes];     // mixture weights (lobe choice when sampling)
    float kappa[kGuideLobes];
    float mx[kGuideLobes], my[kGuideLobes], mz[kGuideLobes];  // unit mean directions
};

// From the 40 network outputs v (in registers).
__device__ __forceinline__ GuideMix guide_mix_values(const float (&v)[kGuideOut])
{
    GuideMix M;
    float mx = v[0];
#pragma unroll
    for (int j = 1; j < kGuideLobes; ++j) mx = fmaxf(mx, v[5 * j]);
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        M.pi[j] = __expf(v[5 * j] - mx);
        s += M.pi[j];
    }
    const float inv = 1.0f / s;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        M.pi[j] *= inv;
        const float k = __expf(fminf(fmaxf(v[5 * j + 1], kGuideLogKMin), kGuideLogKMax));
        M.kappa[j] = k;
        // kappa >= e^-4, so 1 - e^{-2 kappa} >= 0.036 and needs no series
        M.c[j] = M.pi[j] * k / (6.28318530718f * (1.0f - __expf(-2.0f * k)));
        const float a = v[5 * j + 2], b = v[5 * j + 3], c = v[5 * j + 4];
        const float n2 = a * a + b * b + c * c;
        const bool deg = n2 < 1e-24f;
        const float r = deg ? 0.0f : rsqrtf(n2);
        M.mx[j] = a * r, M.my[j] = b * r, M.mz[j] = deg ? 1.0f : c * r;
    }
    return M;
}

__device__ __forceinline__ GuideMix guide_mix(const float *y)
{
    float v[kGuideOut];
#pragma unroll
    for (int i = 0; i < kGuideOut / 4; ++i) {
        const float4 q = reinterpret_cast<const float4 *>(y)[i];
        v[4 * i] = q.x, v[4 * i + 1] = q.y, v[4 * i + 2] = q.z, v[4 * i + 3] = q.w;
    }
    return guide_mix_values(v);
}

// Decoded layout for the shading kernel: five arrays of 8 floats (c_j,
// kappa_j, mu_j x, y, z), 16-byte aligned.
__device__ __forceinline__ void guide_store_decoded(float *y, const GuideMix &M)
{
    float4 *d = reinterpret_cast<float4 *>(y);
    d[0] = make_float4(M.c[0], M.c[1], M.c[2], M.c[3]), d[1] = make_float4(M.c[4], M.c[5], M.c[6], M.c[7]);
    d[2] = make_float4(M.kappa[0], M.kappa[1], M.kappa[2], M.kappa[3]);
    d[3] = make_float4(M.kappa[4], M.kappa[5], M.kappa[6], M.kappa[7]);
    d[4] = make_float4(M.mx[0], M.mx[1], M.mx[2], M.mx[3]), d[5] = make_float4(M.mx[4], M.mx[5], M.mx[6], M.mx[7]);
    d[6] = make_float4(M.my[0], M.my[1], M.my[2], M.my[3]), d[7] = make_float4(M.my[4], M.my[5], M.my[6], M.my[7]);
    d[8] = make_float4(M.mz[0], M.mz[1], M.mz[2], M.mz[3]), d[9] = make_float4(M.mz[4], M.mz[5], M.mz[6], M.mz[7]);
}
#endif

}  // namespace dr
