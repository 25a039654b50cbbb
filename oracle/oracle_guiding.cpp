// oracle_guiding.cpp -- FP64 restatement of the path-guiding network (TEST
// INFRASTRUCTURE: the oracle of the GB300 guiding kernels; never linked into
// the product).
//
// The guiding distribution is not part of the reference (DevilRay has no
// learned sampling); this file restates the network the product trains, so
// its forward pass, loss, gradients and optimiser step can be checked:
//   input u (80): 12-frequency encoding of the normalised position
//     (for axis a, frequency k: sin(2^k pi p_a), cos(2^k pi p_a) at index
//     24 a + 2 k + {0, 1}), the 3 components of the direction input, 5 zeros;
//   4 hidden layers of 64 with ReLU, output layer 48 (40 used);
//   weights and layer inputs rounded to BF16, sums in FP64 (the product sums
//   in FP32 on tensor cores);
//   8-lobe von Mises-Fisher mixture from y: for lobe j, logit y[5j], kappa =
//   exp(clamp(y[5j+1], -4, 7)), mean direction y[5j+2..5j+4] normalised;
//   loss of a batch: -sum_i c_i log q(w_i | x_i) / B with c_i = w_i / mean(w)
//   (Mueller et al., "Neural Importance Sampling", 2019: the KL divergence
//   of q from the target, estimated with the tracer's weighted samples);
//   Adam (Kingma and Ba, 2015) with bias correction.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int kIn = 80, kHid = 64, kOut = 48, kLobes = 8;
constexpr int kLayers = 5;
const int kFanIn[kLayers] = {kIn, kHid, kHid, kHid, kHid};
const int kFanOut[kLayers] = {kHid, kHid, kHid, kHid, kOut};

// Offsets of W_l ([out][in]) and b_l in the flat parameter vector.
int w_off(int l)
{
    int o = 0;
    for (int i = 0; i < l; ++i) o += kFanOut[i] * kFanIn[i] + kFanOut[i];
    return o;
}
int b_off(int l) { return w_off(l) + kFanOut[l] * kFanIn[l]; }

// Round to the nearest BF16 value, ties to even (the CUDA __float2bfloat16_rn).
double bf16(double x)
{
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return f;  // inf / nan unchanged
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    u &= 0xffff0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

struct Lobes {
    double pi[kLobes], kappa[kLobes], mu[kLobes][3], mnorm[kLobes];
    bool kclamped[kLobes];
};

Lobes lobes_of(const double *y)
{
    Lobes L{};
    double mx = -1e300;
    for (int j = 0; j < kLobes; ++j) mx = std::max(mx, y[5 * j]);
    double s = 0;
    for (int j = 0; j < kLobes; ++j) s += std::exp(y[5 * j] - mx);
    for (int j = 0; j < kLobes; ++j) {
        L.pi[j] = std::exp(y[5 * j] - mx) / s;
        const double r = y[5 * j + 1];
        L.kclamped[j] = r < -4.0 || r > 7.0;
        L.kappa[j] = std::exp(std::min(std::max(r, -4.0), 7.0));
        const double mx3 = y[5 * j + 2], my = y[5 * j + 3], mz = y[5 * j + 4];
        double n = std::sqrt(mx3 * mx3 + my * my + mz * mz);
        L.mnorm[j] = n;
        if (n < 1e-12) {
            L.mu[j][0] = 0, L.mu[j][1] = 0, L.mu[j][2] = 1;
        } else {
            L.mu[j][0] = mx3 / n, L.mu[j][1] = my / n, L.mu[j][2] = mz / n;
        }
    }
    return L;
}

// log of the vMF density kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (mu.w - 1)}
double log_vmf(double kappa, double cosang)
{
    return std::log(kappa) - std::log(2.0 * M_PI) - std::log1p(-std::exp(-2.0 * kappa)) + kappa * (cosang - 1.0);
}

void forward(const float *params, const float *in, double acts[kLayers][kHid > kOut ? kHid : kOut], double *y,
             bool round_acts)
{
    double a[kIn];
    for (int i = 0; i < kIn; ++i) a[i] = bf16(in[i]);
    const double *prev = a;
    int prev_n = kIn;
    double buf[2][kHid];
    for (int l = 0; l < kLayers; ++l) {
        const float *W = params + w_off(l), *b = params + b_off(l);
        double *out = l == kLayers - 1 ? y : buf[l & 1];
        for (int o = 0; o < kFanOut[l]; ++o) {
            double z = 0;
            for (int i = 0; i < prev_n; ++i) z += bf16(W[o * kFanIn[l] + i]) * prev[i];
            z += b[o];
            if (l < kLayers - 1) {
                z = z > 0 ? z : 0;
                if (round_acts) z = bf16(z);
            }
            out[o] = z;
            acts[l][o] = z;
        }
        prev = out;
        prev_n = kFanOut[l];
    }
}

}  // namespace

extern "C" {

int32_t or_mlp_num_params(void) { return w_off(kLayers); }

void or_guide_encode(const float *pos, const float *dir, const float *center, float half, float *out)
{
    for (int a = 0; a < 3; ++a) {
        double p = ((double)pos[a] - center[a]) / half;
        p = std::min(1.0, std::max(-1.0, p));
        for (int k = 0; k < 12; ++k) {
            const double ang = std::ldexp(p, k) * M_PI;
            out[24 * a + 2 * k] = (float)std::sin(ang);
            out[24 * a + 2 * k + 1] = (float)std::cos(ang);
        }
    }
    out[72] = dir[0], out[73] = dir[1], out[74] = dir[2];
    for (int i = 75; i < 80; ++i) out[i] = 0.0f;
}

void or_mlp_forward(const float *params, const float *inputs, int32_t n, float *out)
{
    double acts[kLayers][kHid];
    double y[kOut];
    for (int32_t r = 0; r < n; ++r) {
        forward(params, inputs + (size_t)r * kIn, acts, y, true);
        for (int o = 0; o < kOut; ++o) out[(size_t)r * kOut + o] = (float)y[o];
    }
}

double or_vmf_mixture_log_pdf(const float *yf, const float *w)
{
    double y[kOut];
    for (int i = 0; i < 40; ++i) y[i] = yf[i];
    const Lobes L = lobes_of(y);
    double mx = -1e300, t[kLobes];
    for (int j = 0; j < kLobes; ++j) {
        const double c = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
        t[j] = std::log(L.pi[j]) + log_vmf(L.kappa[j], c);
        mx = std::max(mx, t[j]);
    }
    double s = 0;
    for (int j = 0; j < kLobes; ++j) s += std::exp(t[j] - mx);
    return mx + std::log(s);
}

// Loss of a batch and its gradient with respect to every parameter (FP64).
void or_mlp_loss_grad(const float *params, const float *inputs, const float *dirs, const float *weights, int32_t n,
                      double *loss_out, double *grad)
{
    const int np = or_mlp_num_params();
    std::fill(grad, grad + np, 0.0);
    double wsum = 0;
    for (int32_t r = 0; r < n; ++r) wsum += weights[r];
    const double wmean = n ? wsum / n : 1.0;
    double loss = 0;
    for (int32_t r = 0; r < n; ++r) {
        const float *in = inputs + (size_t)r * kIn;
        double acts[kLayers][kHid];
        double y[kOut];
        forward(params, in, acts, y, true);
        const double c = wmean > 0 ? weights[r] / wmean : 0.0;
        const float *w = dirs + 3 * (size_t)r;
        const Lobes L = lobes_of(y);
        double t[kLobes], mx = -1e300, cosang[kLobes];
        for (int j = 0; j < kLobes; ++j) {
            cosang[j] = L.mu[j][0] * w[0] + L.mu[j][1] * w[1] + L.mu[j][2] * w[2];
            t[j] = std::log(L.pi[j]) + log_vmf(L.kappa[j], cosang[j]);
            mx = std::max(mx, t[j]);
        }
        double s = 0;
        for (int j = 0; j < kLobes; ++j) s += std::exp(t[j] - mx);
        const double logq = mx + std::log(s);
        loss += -c * logq / n;
        // d(-c log q / n) / dy
        double dy[kOut] = {0};
        const double g = c / n;
        for (int j = 0; j < kLobes; ++j) {
            const double resp = std::exp(t[j] - logq);
            dy[5 * j] = -g * (resp - L.pi[j]);
            const double kap = L.kappa[j];
            const double dlogp_dk = 1.0 / kap - 2.0 / std::expm1(2.0 * kap) + cosang[j] - 1.0;
            dy[5 * j + 1] = L.kclamped[j] ? 0.0 : -g * resp * dlogp_dk * kap;
            if (L.mnorm[j] >= 1e-12) {
                for (int a = 0; a < 3; ++a) {
                    const double d = kap * (w[a] - cosang[j] * L.mu[j][a]) / L.mnorm[j];
                    dy[5 * j + 2 + a] = -g * resp * d;
                }
            }
        }
        // backward through the layers (ReLU; the layer inputs as rounded)
        double delta[kOut];
        std::copy(dy, dy + kOut, delta);
        for (int l = kLayers - 1; l >= 0; --l) {
            const float *W = params + w_off(l);
            double in_l[kIn];
            int nin = kFanIn[l];
            if (l == 0)
                for (int i = 0; i < kIn; ++i) in_l[i] = bf16(in[i]);
            else
                for (int i = 0; i < nin; ++i) in_l[i] = acts[l - 1][i];
            for (int o = 0; o < kFanOut[l]; ++o) {
                grad[b_off(l) + o] += delta[o];
                for (int i = 0; i < nin; ++i) grad[w_off(l) + o * nin + i] += delta[o] * in_l[i];
            }
            if (l == 0) break;
            double prev[kHid];
            for (int i = 0; i < nin; ++i) {
                double z = 0;
                for (int o = 0; o < kFanOut[l]; ++o) z += bf16(W[o * nin + i]) * delta[o];
                prev[i] = acts[l - 1][i] > 0 ? z : 0.0;
            }
            std::copy(prev, prev + nin, delta);
        }
    }
    *loss_out = loss;
}

// Adam step on FP32 master parameters with moments m, v (t = step number >= 1).
void or_adam_step(float *params, float *m, float *v, const float *grad, int32_t n, int32_t t, float lr, float beta1,
                  float beta2, float eps)
{
    const float c1 = 1.0f - std::pow(beta1, (float)t), c2 = 1.0f - std::pow(beta2, (float)t);
    for (int32_t i = 0; i < n; ++i) {
        m[i] = beta1 * m[i] + (1.0f - beta1) * grad[i];
        v[i] = beta2 * v[i] + (1.0f - beta2) * grad[i] * grad[i];
        const float mh = m[i] / c1, vh = v[i] / c2;
        params[i] -= lr * mh / (std::sqrt(vh) + eps);
    }
}

}  // extern "C"
