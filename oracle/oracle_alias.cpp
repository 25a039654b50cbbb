// oracle_alias.cpp -- CPU restatement of DevilRay's alias-table build and
// sampling, plus the CPU restatement of the device's sweep-pairing build
// (TEST INFRASTRUCTURE: the oracle of the GB300 kernels).

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <random>
#include <vector>

namespace {

constexpr int UNINITIALIZED = -1;

// ensurePALarger (src/DistributionSamplers.cpp:29-37)
void ensurePALarger(or_alias_entry &e)
{
    if (e.p_A < 0.5f) {
        e.p_A = 1 - e.p_A;
        std::swap(e.A, e.B);
        std::swap(e.pdf_A, e.pdf_B);
    }
}

}  // namespace

extern "C" {

// generateAliasTable (src/DistributionSamplers.cpp:39-149). The pairing order
// comes from two std::priority_queue max-heaps ordered by p_A; using the same
// container and comparator reproduces the reference's tie behaviour exactly.
void or_alias_build_ref(const float *weights, int32_t n_in, or_alias_entry *out)
{
    const size_t n = (size_t)std::max(0, n_in);
    std::vector<float> filtered;
    filtered.reserve(n);
    for (size_t i = 0; i < n; ++i) filtered.push_back(std::max(0.f, weights[i]));
    const float total = std::accumulate(filtered.begin(), filtered.end(), 0.f);

    for (size_t i = 0; i < n; ++i) out[i] = or_alias_entry{0, 0, 0, 0, 0};
    if (n == 0) return;
    if (total < 1e-5f) {  // generateUniformAliasTable (:13-27)
        const float uniformPdf = 1.0f / n;
        for (size_t i = 0; i < n; ++i) out[i] = or_alias_entry{1, uniformPdf, 0, (int32_t)i, UNINITIALIZED};
        return;
    }

    or_alias_entry *ptr = out;
    const auto prio = [](const or_alias_entry &a, const or_alias_entry &b) { return a.p_A < b.p_A; };
    std::priority_queue<or_alias_entry, std::vector<or_alias_entry>, decltype(prio)> overfull(prio);
    std::priority_queue<or_alias_entry, std::vector<or_alias_entry>, decltype(prio)> underfull(prio);

    for (size_t i = 0; i < n; ++i) {
        const float p = filtered[i] / total;
        const or_alias_entry e{n * p, 0, 0, (int32_t)i, UNINITIALIZED};
        if (e.p_A > 1) overfull.push(e);
        else if (e.p_A < 1) underfull.push(e);
        else *ptr++ = e;
    }
    while (!underfull.empty() || !overfull.empty()) {
        if (underfull.empty() || overfull.empty()) break;
        auto under = underfull.top();
        auto over = overfull.top();
        underfull.pop();
        overfull.pop();
        under.B = over.A;
        over.p_A = over.p_A + under.p_A - 1;
        ensurePALarger(under);
        *ptr++ = under;
        if (over.p_A > 1) overfull.push(over);
        else if (over.p_A < 1) underfull.push(over);
        else {
            ensurePALarger(over);
            *ptr++ = over;
        }
    }
    while (!underfull.empty()) {
        auto e = underfull.top();
        underfull.pop();
        e.p_A = 1;
        *ptr++ = e;
    }
    while (!overfull.empty()) {
        auto e = overfull.top();
        overfull.pop();
        e.p_A = 1;
        *ptr++ = e;
    }
    std::vector<float> pdfs(n);
    for (size_t i = 0; i < n; ++i) pdfs[i] = filtered[i] / total;
    for (size_t i = 0; i < n; ++i) {
        out[i].pdf_A = pdfs[out[i].A];
        if (out[i].B >= 0 && (size_t)out[i].B < n) out[i].pdf_B = pdfs[out[i].B];
        else out[i].pdf_B = 0.0f;
    }
}

// Sweep-pairing build (Huebschle-Schneider and Sanders, "Parallel Weighted
// Random Sampling", ACM TOMS 2022, sweeping construction) evaluated in exact
// fixed point (64-bit weights, 128-bit running sums), so that the sequential form below and the parallel
// device form (prefix sums + binary searches) produce the same table bit for
// bit. Slot i always holds item i; its alias is the heavy item whose surplus
// covers slot i's deficit. The p_A >= 0.5 convention of the reference
// (ensurePALarger) is applied to every slot.
//
//   m_i  = floor(w_i * 2^s)            (w_i clamped at 0; s from the largest w,
//                                       so that W = sum m_i < 2^61)
//   a_i  = n * m_i - W                 (light if a_i < 0, heavy otherwise)
//   light slot k:  p = n m_k / W,  alias = first heavy whose running surplus
//                  exceeds the deficits of the lights before k
//   heavy slot j:  p = (W + R_j) / W, alias = next heavy, where R_j <= 0 is its
//                  surplus left after the lights it covers
void or_alias_build_sweep(const float *weights, int32_t n_in, or_alias_entry *out)
{
    const int64_t n = std::max(0, n_in);
    if (n == 0) return;
    int emax = -1000;
    for (int64_t i = 0; i < n; ++i) {
        const float w = weights[i] > 0.0f ? weights[i] : 0.0f;
        if (w > 0.0f && std::isfinite(w)) {
            int e;
            std::frexp(w, &e);
            emax = std::max(emax, e);
        }
    }
    int lg = 0;
    while ((int64_t(1) << lg) < n + 1) ++lg;
    std::vector<int64_t> m((size_t)n);
    int64_t W = 0;
    const int s = 61 - lg - emax;
    for (int64_t i = 0; i < n; ++i) {
        const float w = weights[i] > 0.0f && std::isfinite(weights[i]) ? weights[i] : 0.0f;
        m[i] = emax == -1000 ? 0 : (int64_t)std::ldexp((double)w, s);
        W += m[i];
    }
    const float Wf = emax == -1000 ? 0.0f : (float)std::ldexp((double)W, -s);
    if (!(Wf >= 1e-5f)) {
        const float uniformPdf = 1.0f / (float)n;
        for (int64_t i = 0; i < n; ++i) out[i] = or_alias_entry{1, uniformPdf, 0, (int32_t)i, -1};
        return;
    }
    // Running sums of deficits and surpluses reach n * W (< 2^88): 128-bit.
    using i128 = __int128;
    std::vector<int64_t> lights, heavies;
    std::vector<i128> Dexcl, Sincl;
    i128 D = 0, S = 0;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t a = n * m[i] - W;
        if (a < 0) {
            lights.push_back(i);
            Dexcl.push_back(D);
            D += -a;
        } else {
            heavies.push_back(i);
            S += a;
            Sincl.push_back(S);
        }
    }
    const double Wd = (double)W;
    auto pdfOf = [&](int64_t i) { return (float)((double)m[i] / Wd); };
    // lights: alias = first heavy h with Sincl[h] > Dexcl[k]
    size_t h = 0;
    for (size_t k = 0; k < lights.size(); ++k) {
        while (h < heavies.size() && !(Sincl[h] > Dexcl[k])) ++h;
        const int64_t i = lights[k];
        or_alias_entry e;
        e.A = (int32_t)i;
        e.p_A = (float)((double)(n * m[i]) / Wd);
        e.pdf_A = pdfOf(i);
        e.B = h < heavies.size() ? (int32_t)heavies[h] : -1;
        e.pdf_B = e.B >= 0 ? pdfOf(e.B) : 0.0f;
        if (e.B < 0) e.p_A = 1.0f;
        ensurePALarger(e);
        out[i] = e;
    }
    // heavies: k_end = first light with Dexcl[k] >= Sincl[j]; R = Sincl[j] - D(k_end)
    size_t k = 0;
    for (size_t j = 0; j < heavies.size(); ++j) {
        while (k < lights.size() && !(Dexcl[k] >= Sincl[j])) ++k;
        const i128 Dk = k < lights.size() ? Dexcl[k] : D;
        const int64_t R = (int64_t)(Sincl[j] - Dk);  // in [-W, 0]
        const int64_t i = heavies[j];
        or_alias_entry e;
        e.A = (int32_t)i;
        e.pdf_A = pdfOf(i);
        if (j + 1 < heavies.size()) {
            e.p_A = (float)((double)(W + R) / Wd);
            e.B = (int32_t)heavies[j + 1];
            e.pdf_B = pdfOf(e.B);
        } else {
            e.p_A = 1.0f;
            e.B = -1;
            e.pdf_B = 0.0f;
        }
        if (e.p_A == 1.0f) {
            e.B = -1;
            e.pdf_B = 0.0f;
        }
        ensurePALarger(e);
        out[i] = e;
    }
}

// sample (include/tracing/DistributionSamplers.hpp:64-88), with the two
// uniforms passed in.
void or_alias_sample(const or_alias_entry *table, int32_t n, float u0, float u1,
                     int32_t *index, float *pdf)
{
    const size_t size = (size_t)n;
    float findex = u0 * size;
    if (findex == size) findex = size - 1;
    const int idx = static_cast<int>(findex);
    const or_alias_entry &e = table[idx];
    if (u1 <= e.p_A) {
        *index = e.A;
        *pdf = e.pdf_A;
    } else {
        *index = e.B;
        *pdf = e.pdf_B;
    }
}

void or_lognormal_input(int32_t n, uint32_t seed, float *out)
{
    std::mt19937 rng(seed);
    std::lognormal_distribution<float> dist(0.0f, 1.0f);
    for (int32_t i = 0; i < n; ++i) out[i] = dist(rng);
}

// Philox4x32 with 10 rounds (Salmon, Moraes, Dror and Shaw, "Parallel Random
// Numbers: As Easy as 1, 2, 3", SC'11): multipliers 0xD2511F53/0xCD9E8D57,
// Weyl key increments 0x9E3779B9/0xBB67AE85.
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n1 = lo1;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        const uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

}  // extern "C"
