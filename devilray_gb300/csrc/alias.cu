// alias.cu -- alias-table build and sampling on the device.
//
// Two builds:
//  * reference mode: the pairing of DevilRay's generateAliasTable
//    (src/DistributionSamplers.cpp:39-149) -- a sequential float total and two
//    max-heaps ordered by p_A -- run by one thread with heaps whose sift
//    operations follow the standard binary-heap algorithm of the C++ library
//    the reference uses (push: sift the new element up while its parent
//    compares lower; pop: move the last element to the top position's hole
//    path along the larger child, preferring the right child on ties, then sift
//    up). Bit-identical to the reference; O(n log n) on one thread.
//  * sweep mode (default): the sweeping construction of Huebschle-Schneider
//    and Sanders ("Parallel Weighted Random Sampling", ACM TOMS 2022) in exact
//    fixed point (64-bit weights, 128-bit prefix sums), so it is order
//    independent and bit-identical to its CPU restatement in the oracle.
//    Slot i holds item i; lights are aliased to the heavy item whose surplus
//    covers them (prefix sums + binary search), heavies to the next heavy.

#include "dr_internal.h"
#include "alias_kernels.cuh"

#include <climits>

namespace dr {

using i128 = __int128;

// ---- reference-compatible build ------------------------------------------------

struct HeapItem {
    float p;
    int32_t a;
};

__host__ __device__ __forceinline__ void heap_push(HeapItem *h, int32_t &len, HeapItem v)
{
    int32_t hole = len++;
    int32_t parent = (hole - 1) / 2;
    while (hole > 0 && h[parent].p < v.p) {
        h[hole] = h[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    h[hole] = v;
}

// Removes the top element (the caller read it before).
__host__ __device__ __forceinline__ void heap_pop(HeapItem *h, int32_t &len)
{
    if (len > 1) {
        const int32_t n = len - 1;  // size of the heap without the moved-out top
        const HeapItem value = h[n];
        h[n] = h[0];
        int32_t hole = 0, child = 0;
        while (child < (n - 1) / 2) {
            child = 2 * (child + 1);
            if (h[child].p < h[child - 1].p) --child;
            h[hole] = h[child];
            hole = child;
        }
        if ((n & 1) == 0 && child == (n - 2) / 2) {
            child = 2 * (child + 1);
            h[hole] = h[child - 1];
            hole = child - 1;
        }
        int32_t parent = (hole - 1) / 2;
        while (hole > 0 && h[parent].p < value.p) {
            h[hole] = h[parent];
            hole = parent;
            parent = (hole - 1) / 2;
        }
        h[hole] = value;
    }
    --len;
}

__host__ __device__ __forceinline__ void ensure_pa_larger(dr_alias_entry &e)
{
    if (e.p_A < 0.5f) {
        e.p_A = 1 - e.p_A;
        const int32_t t = e.A;
        e.A = e.B;
        e.B = t;
        const float f = e.pdf_A;
        e.pdf_A = e.pdf_B;
        e.pdf_B = f;
    }
}

// One table, one thread: filter, sequential total, heap pairing, entries in
// processing order, then the pdf fill (src/DistributionSamplers.cpp:39-149).
__device__ void alias_ref_build_one(const float *__restrict__ w, uint32_t n, dr_alias_entry *__restrict__ out,
                                    HeapItem *under, HeapItem *over, float *filtered, bool fill_pdfs,
                                    float *total_out)
{
    float total = 0.f;
    for (uint32_t i = 0; i < n; ++i) {
        const float fi = (0.f < w[i]) ? w[i] : 0.f;  // std::max(0.f, w[i])
        filtered[i] = fi;
        total = total + fi;
    }
    if (total_out) *total_out = total;
    if (n == 0) return;
    if (total < 1e-5f) {
        const float u = 1.0f / (float)n;
        for (uint32_t i = 0; i < n; ++i) out[i] = dr_alias_entry{1.0f, u, 0.0f, (int32_t)i, -1};
        return;
    }
    int32_t nu = 0, no = 0;
    uint32_t ptr = 0;
    const float fn = (float)n;
    for (uint32_t i = 0; i < n; ++i) {
        const float p = filtered[i] / total;
        const HeapItem e{fn * p, (int32_t)i};
        if (e.p > 1) heap_push(over, no, e);
        else if (e.p < 1) heap_push(under, nu, e);
        else out[ptr++] = dr_alias_entry{e.p, 0.f, 0.f, e.a, -1};
    }
    while (nu > 0 && no > 0) {
        HeapItem u = under[0];
        HeapItem o = over[0];
        heap_pop(under, nu);
        heap_pop(over, no);
        dr_alias_entry ue{u.p, 0.f, 0.f, u.a, o.a};
        o.p = o.p + u.p - 1;
        ensure_pa_larger(ue);
        out[ptr++] = ue;
        if (o.p > 1) heap_push(over, no, o);
        else if (o.p < 1) heap_push(under, nu, o);
        else {
            dr_alias_entry oe{o.p, 0.f, 0.f, o.a, -1};
            ensure_pa_larger(oe);
            out[ptr++] = oe;
        }
    }
    while (nu > 0) {
        const HeapItem e = under[0];
        heap_pop(under, nu);
        out[ptr++] = dr_alias_entry{1.0f, 0.f, 0.f, e.a, -1};
    }
    while (no > 0) {
        const HeapItem e = over[0];
        heap_pop(over, no);
        out[ptr++] = dr_alias_entry{1.0f, 0.f, 0.f, e.a, -1};
    }
    if (fill_pdfs) {
        for (uint32_t i = 0; i < n; ++i) {
            dr_alias_entry &e = out[i];
            e.pdf_A = filtered[e.A] / total;
            e.pdf_B = (e.B >= 0 && (uint32_t)e.B < n) ? filtered[e.B] / total : 0.0f;
        }
    }
}

__global__ void k_alias_ref_pair(const float *__restrict__ w, uint32_t n, dr_alias_entry *__restrict__ out,
                                 HeapItem *under, HeapItem *over, float *filtered, float *total_out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    alias_ref_build_one(w, n, out, under, over, filtered, false, total_out);
}

// pdf fill (src/DistributionSamplers.cpp:135-146) of the single-table build, parallel.
__global__ void k_alias_ref_pdfs(uint32_t n, dr_alias_entry *__restrict__ out, const float *__restrict__ filtered,
                                 const float *__restrict__ total_in)
{
    const float total = *total_in;
    if (total < 1e-5f) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dr_alias_entry e = out[i];
        e.pdf_A = filtered[e.A] / total;
        e.pdf_B = (e.B >= 0 && (uint32_t)e.B < n) ? filtered[e.B] / total : 0.0f;
        out[i] = e;
    }
}

// Many independent tables, one thread each: table s covers entries
// [begin[s], begin[s] + count[s]) of w and out (object-local indices).
__global__ void k_alias_ref_segments(const float *__restrict__ w, const uint32_t *__restrict__ begin,
                                     const uint32_t *__restrict__ count, uint32_t nseg,
                                     dr_alias_entry *__restrict__ out, HeapItem *heaps, float *filtered)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const uint32_t b = begin[s], n = count[s];
    alias_ref_build_one(w + b, n, out + b, heaps + 2 * (size_t)b, heaps + 2 * (size_t)b + n, filtered + b, true,
                        nullptr);
}

// ---- sweep build -----------------------------------------------------------------------

__device__ __forceinline__ float clamp_weight(float w) { return (w > 0.0f && isfinite(w)) ? w : 0.0f; }

__device__ __forceinline__ int float_exponent(float w)
{
    int e;
    frexpf(w, &e);
    return e;
}

// Warp-level inclusive scan of a 128-bit value.
__device__ __forceinline__ i128 warp_scan_i128(i128 v)
{
    const int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long lo = (unsigned long long)v;
        const long long hi = (long long)(v >> 64);
        const unsigned long long lo_o = __shfl_up_sync(0xffffffffu, lo, off);
        const long long hi_o = __shfl_up_sync(0xffffffffu, hi, off);
        const i128 o = ((i128)hi_o << 64) | (i128)lo_o;
        if (lane >= off) v += o;
    }
    return v;
}

__device__ __forceinline__ int warp_scan_int(int v)
{
    const int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    return v;
}

// Block-wide exclusive scan of (count, D, S) triples; returns the block total
// through `total`. blockDim.x == kSweepBlock.
struct Agg {
    int32_t lights;
    int32_t pad;
    i128 D;
    i128 S;
};

__device__ Agg block_exclusive_scan(Agg v, Agg &total)
{
    __shared__ int s_cnt[kSweepBlock / 32];
    __shared__ i128 s_D[kSweepBlock / 32];
    __shared__ i128 s_S[kSweepBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c_inc = warp_scan_int(v.lights);
    const i128 d_inc = warp_scan_i128(v.D);
    const i128 s_inc = warp_scan_i128(v.S);
    if (lane == 31) {
        s_cnt[warp] = c_inc;
        s_D[warp] = d_inc;
        s_S[warp] = s_inc;
    }
    __syncthreads();
    if (warp == 0) {
        constexpr int nw = kSweepBlock / 32;
        int c = lane < nw ? s_cnt[lane] : 0;
        i128 d = lane < nw ? s_D[lane] : (i128)0;
        i128 s = lane < nw ? s_S[lane] : (i128)0;
        c = warp_scan_int(c);
        d = warp_scan_i128(d);
        s = warp_scan_i128(s);
        if (lane < nw) {
            s_cnt[lane] = c;
            s_D[lane] = d;
            s_S[lane] = s;
        }
    }
    __syncthreads();
    Agg out;
    const int c_before = warp > 0 ? s_cnt[warp - 1] : 0;
    const i128 d_before = warp > 0 ? s_D[warp - 1] : (i128)0;
    const i128 s_before = warp > 0 ? s_S[warp - 1] : (i128)0;
    out.lights = c_before + c_inc - v.lights;
    out.D = d_before + d_inc - v.D;
    out.S = s_before + s_inc - v.S;
    out.pad = 0;
    total.lights = s_cnt[kSweepBlock / 32 - 1];
    total.D = s_D[kSweepBlock / 32 - 1];
    total.S = s_S[kSweepBlock / 32 - 1];
    total.pad = 0;
    __syncthreads();
    return out;
}

struct SweepScalars {
    int emax;
    int lg;
    int shift;
    int uniform;
    unsigned long long W;
    int32_t num_lights;
    int32_t num_heavies;
    i128 D_total;
};

__device__ __forceinline__ long long fixed_weight(float w, const SweepScalars &sc)
{
    if (sc.emax == INT_MIN) return 0;
    return (long long)ldexp((double)clamp_weight(w), sc.shift);
}

__global__ void k_sweep_init(SweepScalars *sc, uint32_t n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        sc->emax = INT_MIN;
        int lg = 0;
        while ((1ll << lg) < (long long)n + 1) ++lg;
        sc->lg = lg;
        sc->W = 0;
        sc->uniform = 0;
    }
}

__global__ void k_sweep_exponent(const float *__restrict__ w, uint32_t n, SweepScalars *sc)
{
    int e = INT_MIN;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = clamp_weight(w[i]);
        if (x > 0.0f) e = max(e, float_exponent(x));
    }
    for (int off = 16; off > 0; off >>= 1) e = max(e, __shfl_down_sync(0xffffffffu, e, off));
    if ((threadIdx.x & 31) == 0 && e != INT_MIN) atomicMax(&sc->emax, e);
}

__global__ void k_sweep_sum(const float *__restrict__ w, uint32_t n, SweepScalars *sc)
{
    __shared__ SweepScalars s;
    if (threadIdx.x == 0) {
        s = *sc;
        s.shift = 61 - s.lg - s.emax;
    }
    __syncthreads();
    unsigned long long acc = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc += (unsigned long long)fixed_weight(w[i], s);
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&sc->W, acc);
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->shift = s.shift;
}

// Per tile of kSweepBlock items: (light count, deficit sum, surplus sum).
__global__ void k_sweep_tile_aggregates(const float *__restrict__ w, uint32_t n, const SweepScalars *sc, Agg *tiles)
{
    const SweepScalars s = *sc;
    const uint32_t i = blockIdx.x * kSweepBlock + threadIdx.x;
    Agg v{0, 0, 0, 0};
    if (i < n) {
        const long long a = (long long)n * fixed_weight(w[i], s) - (long long)s.W;
        if (a < 0) {
            v.lights = 1;
            v.D = (i128)(-a);
        } else {
            v.S = (i128)a;
        }
    }
    Agg total;
    block_exclusive_scan(v, total);
    if (threadIdx.x == 0) tiles[blockIdx.x] = total;
}

// One block: exclusive scan over the tile aggregates (in place).
__global__ void k_sweep_scan_tiles(Agg *tiles, uint32_t num_tiles, SweepScalars *sc, uint32_t n)
{
    Agg carry{0, 0, 0, 0};
    for (uint32_t base = 0; base < num_tiles; base += kSweepBlock) {
        const uint32_t t = base + threadIdx.x;
        Agg v = t < num_tiles ? tiles[t] : Agg{0, 0, 0, 0};
        Agg total;
        Agg ex = block_exclusive_scan(v, total);
        if (t < num_tiles) {
            Agg o;
            o.lights = carry.lights + ex.lights;
            o.D = carry.D + ex.D;
            o.S = carry.S + ex.S;
            o.pad = 0;
            tiles[t] = o;
        }
        carry.lights += total.lights;
        carry.D += total.D;
        carry.S += total.S;
    }
    if (threadIdx.x == 0) {
        sc->num_lights = carry.lights;
        sc->num_heavies = (int32_t)n - carry.lights;
        sc->D_total = carry.D;
        const float Wf = sc->emax == INT_MIN ? 0.0f : (float)ldexp((double)sc->W, -sc->shift);
        sc->uniform = !(Wf >= 1e-5f);
    }
}

// Writes the light / heavy lists in index order with their running sums.
__global__ void k_sweep_scatter(const float *__restrict__ w, uint32_t n, const SweepScalars *sc, const Agg *tiles,
                                int32_t *lights, i128 *Dexcl, int32_t *heavies, i128 *Sincl)
{
    const SweepScalars s = *sc;
    const uint32_t i = blockIdx.x * kSweepBlock + threadIdx.x;
    Agg v{0, 0, 0, 0};
    long long a = 0;
    if (i < n) {
        a = (long long)n * fixed_weight(w[i], s) - (long long)s.W;
        if (a < 0) {
            v.lights = 1;
            v.D = (i128)(-a);
        } else {
            v.S = (i128)a;
        }
    }
    Agg total;
    const Agg ex = block_exclusive_scan(v, total);
    if (i < n) {
        const Agg base = tiles[blockIdx.x];
        const int32_t light_rank = base.lights + ex.lights;
        if (a < 0) {
            lights[light_rank] = (int32_t)i;
            Dexcl[light_rank] = base.D + ex.D;
        } else {
            const int32_t heavy_rank = (int32_t)i - light_rank;
            heavies[heavy_rank] = (int32_t)i;
            Sincl[heavy_rank] = base.S + ex.S + v.S;
        }
    }
}

__device__ __forceinline__ float pdf_of(long long m, unsigned long long W) { return (float)((double)m / (double)W); }

__global__ void k_sweep_assign(const float *__restrict__ w, uint32_t n, const SweepScalars *sc,
                               const int32_t *__restrict__ lights, const i128 *__restrict__ Dexcl,
                               const int32_t *__restrict__ heavies, const i128 *__restrict__ Sincl,
                               dr_alias_entry *__restrict__ out)
{
    const SweepScalars s = *sc;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (s.uniform) {
        out[t] = dr_alias_entry{1.0f, 1.0f / (float)n, 0.0f, (int32_t)t, -1};
        return;
    }
    const int32_t nl = s.num_lights, nh = s.num_heavies;
    const double Wd = (double)s.W;
    dr_alias_entry e;
    int32_t slot;
    if ((int32_t)t < nl) {
        const int32_t k = (int32_t)t;
        const int32_t i = lights[k];
        slot = i;
        const long long m = fixed_weight(w[i], s);
        const i128 d = Dexcl[k];
        // first heavy h with Sincl[h] > d
        int32_t lo = 0, hi = nh;
        while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (Sincl[mid] > d) hi = mid;
            else lo = mid + 1;
        }
        e.A = i;
        e.p_A = (float)((double)((long long)n * m) / Wd);
        e.pdf_A = pdf_of(m, s.W);
        if (lo < nh) {
            e.B = heavies[lo];
            e.pdf_B = pdf_of(fixed_weight(w[e.B], s), s.W);
        } else {
            e.B = -1;
            e.pdf_B = 0.0f;
            e.p_A = 1.0f;
        }
    } else {
        const int32_t j = (int32_t)t - nl;
        const int32_t i = heavies[j];
        slot = i;
        const i128 sj = Sincl[j];
        // first light k with Dexcl[k] >= Sincl[j]
        int32_t lo = 0, hi = nl;
        while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (Dexcl[mid] >= sj) hi = mid;
            else lo = mid + 1;
        }
        const i128 Dk = lo < nl ? Dexcl[lo] : s.D_total;
        const long long R = (long long)(sj - Dk);
        e.A = i;
        e.pdf_A = pdf_of(fixed_weight(w[i], s), s.W);
        if (j + 1 < nh) {
            e.p_A = (float)((double)((long long)s.W + R) / Wd);
            e.B = heavies[j + 1];
            e.pdf_B = pdf_of(fixed_weight(w[e.B], s), s.W);
        } else {
            e.p_A = 1.0f;
            e.B = -1;
            e.pdf_B = 0.0f;
        }
        if (e.p_A == 1.0f) {
            e.B = -1;
            e.pdf_B = 0.0f;
        }
    }
    ensure_pa_larger(e);
    out[slot] = e;
}

// ---- sweep build of many small tables, one thread per table ---------------------------

// The sweep build of one table by one thread: the same fixed-point quantities
// (m_i, W, a_i = n m_i - W) as the parallel kernels above and the same
// assignment rules, evaluated by two cursors that walk the lights and the
// heavies in index order instead of prefix sums and binary searches. O(n), no
// scratch memory; the table equals the parallel build's bit for bit.
__device__ void alias_sweep_build_one(const float *__restrict__ w, uint32_t n, dr_alias_entry *__restrict__ out)
{
    if (n == 0) return;
    SweepScalars s;
    s.emax = INT_MIN;
    for (uint32_t i = 0; i < n; ++i) {
        const float x = clamp_weight(w[i]);
        if (x > 0.0f) s.emax = max(s.emax, float_exponent(x));
    }
    int lg = 0;
    while ((1ll << lg) < (long long)n + 1) ++lg;
    s.lg = lg;
    s.shift = 61 - lg - s.emax;
    unsigned long long W = 0;
    for (uint32_t i = 0; i < n; ++i) W += (unsigned long long)fixed_weight(w[i], s);
    const float Wf = s.emax == INT_MIN ? 0.0f : (float)ldexp((double)W, -s.shift);
    if (!(Wf >= 1e-5f)) {
        const float u = 1.0f / (float)n;
        for (uint32_t i = 0; i < n; ++i) out[i] = dr_alias_entry{1.0f, u, 0.0f, (int32_t)i, -1};
        return;
    }
    const double Wd = (double)W;
    const long long nn = (long long)n;
    auto surplus = [&](uint32_t i) { return nn * fixed_weight(w[i], s) - (long long)W; };  // a_i
    auto next_heavy = [&](uint32_t i) {
        while (i < n && surplus(i) < 0) ++i;
        return i;
    };
    auto next_light = [&](uint32_t i) {
        while (i < n && surplus(i) >= 0) ++i;
        return i;
    };
    // lights: alias = first heavy h whose inclusive surplus sum exceeds the
    // deficits of the lights before this one
    {
        uint32_t h = next_heavy(0);
        i128 S = h < n ? (i128)surplus(h) : (i128)0;
        i128 D = 0;
        for (uint32_t i = next_light(0); i < n; i = next_light(i + 1)) {
            while (h < n && !(S > D)) {
                h = next_heavy(h + 1);
                if (h < n) S += (i128)surplus(h);
            }
            const long long m = fixed_weight(w[i], s);
            dr_alias_entry e;
            e.A = (int32_t)i;
            e.p_A = (float)((double)(nn * m) / Wd);
            e.pdf_A = pdf_of(m, W);
            if (h < n) {
                e.B = (int32_t)h;
                e.pdf_B = pdf_of(fixed_weight(w[h], s), W);
            } else {
                e.B = -1;
                e.pdf_B = 0.0f;
                e.p_A = 1.0f;
            }
            ensure_pa_larger(e);
            out[i] = e;
            D += (i128)(-surplus(i));
        }
    }
    // heavies: R = inclusive surplus sum - deficits of the lights before the
    // first light not covered by it; alias = the next heavy
    {
        uint32_t k = next_light(0);
        i128 Dk = 0, S = 0;
        for (uint32_t j = next_heavy(0); j < n;) {
            S += (i128)surplus(j);
            while (k < n && !(Dk >= S)) {
                Dk += (i128)(-surplus(k));
                k = next_light(k + 1);
            }
            const long long R = (long long)(S - Dk);
            const uint32_t jn = next_heavy(j + 1);
            dr_alias_entry e;
            e.A = (int32_t)j;
            e.pdf_A = pdf_of(fixed_weight(w[j], s), W);
            if (jn < n) {
                e.p_A = (float)((double)((long long)W + R) / Wd);
                e.B = (int32_t)jn;
                e.pdf_B = pdf_of(fixed_weight(w[jn], s), W);
            } else {
                e.p_A = 1.0f;
                e.B = -1;
                e.pdf_B = 0.0f;
            }
            if (e.p_A == 1.0f) {
                e.B = -1;
                e.pdf_B = 0.0f;
            }
            ensure_pa_larger(e);
            out[j] = e;
            j = jn;
        }
    }
}

// Many independent sweep tables, one thread each (segments as k_alias_ref_segments).
__global__ void k_alias_sweep_segments(const float *__restrict__ w, const uint32_t *__restrict__ begin,
                                       const uint32_t *__restrict__ count, uint32_t nseg,
                                       dr_alias_entry *__restrict__ out)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const uint32_t b = begin[s];
    alias_sweep_build_one(w + b, count[s], out + b);
}

// ---- sampling ------------------------------------------------------------------------------

// sample() (include/tracing/DistributionSamplers.hpp:64-88) with the two
// uniforms of draw i at uniforms[2i], uniforms[2i+1].
__global__ void k_alias_sample(const dr_alias_entry *__restrict__ table, uint32_t n, const float *__restrict__ u,
                               uint64_t draws, int32_t *__restrict__ index, float *__restrict__ pdf)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= draws) return;
    const float2 r = reinterpret_cast<const float2 *>(u)[i];
    int32_t idx;
    float p;
    alias_sample(table, n, r.x, r.y, idx, p);
    index[i] = idx;
    pdf[i] = p;
}

// ---- launchers -------------------------------------------------------------------------------

size_t alias_scratch_bytes(uint32_t n, int mode)
{
    if (mode == DR_ALIAS_REFERENCE) return 256 + (size_t)n * (8 + 8 + 4) + 64;
    const size_t tiles = (n + kSweepBlock - 1) / kSweepBlock;
    return 512 + tiles * sizeof(Agg) + (size_t)n * (4 + 4 + 16 + 16) + 256;
}

static inline char *align256(char *p) { return reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255)); }

cudaError_t launch_alias_build(const float *w, uint32_t n, dr_alias_entry *out, int mode, void *scratch,
                               size_t scratch_bytes, int num_sms, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (scratch_bytes < alias_scratch_bytes(n, mode)) return cudaErrorInvalidValue;
    char *p = align256(static_cast<char *>(scratch));
    if (mode == DR_ALIAS_REFERENCE) {
        float *total = reinterpret_cast<float *>(p);
        p = align256(p + 16);
        HeapItem *under = reinterpret_cast<HeapItem *>(p);
        HeapItem *over = under + n;
        float *filtered = reinterpret_cast<float *>(over + n);
        k_alias_ref_pair<<<1, 32, 0, st>>>(w, n, out, under, over, filtered, total);
        const int blocks = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms * 4);
        k_alias_ref_pdfs<<<blocks, 256, 0, st>>>(n, out, filtered, total);
        return cudaGetLastError();
    }
    SweepScalars *sc = reinterpret_cast<SweepScalars *>(p);
    p = align256(p + sizeof(SweepScalars));
    const uint32_t tiles = (n + kSweepBlock - 1) / kSweepBlock;
    Agg *tile_agg = reinterpret_cast<Agg *>(p);
    p = align256(p + tiles * sizeof(Agg));
    i128 *Dexcl = reinterpret_cast<i128 *>(p);
    i128 *Sincl = Dexcl + n;
    int32_t *lights = reinterpret_cast<int32_t *>(Sincl + n);
    int32_t *heavies = lights + n;
    const int grid = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms * 8);
    k_sweep_init<<<1, 32, 0, st>>>(sc, n);
    k_sweep_exponent<<<grid, 256, 0, st>>>(w, n, sc);
    k_sweep_sum<<<grid, 256, 0, st>>>(w, n, sc);
    k_sweep_tile_aggregates<<<tiles, kSweepBlock, 0, st>>>(w, n, sc, tile_agg);
    k_sweep_scan_tiles<<<1, kSweepBlock, 0, st>>>(tile_agg, tiles, sc, n);
    k_sweep_scatter<<<tiles, kSweepBlock, 0, st>>>(w, n, sc, tile_agg, lights, Dexcl, heavies, Sincl);
    k_sweep_assign<<<(n + 255) / 256, 256, 0, st>>>(w, n, sc, lights, Dexcl, heavies, Sincl, out);
    return cudaGetLastError();
}

cudaError_t launch_alias_ref_segments(const float *w, uint32_t total_n, const uint32_t *begin, const uint32_t *count,
                                     uint32_t nseg, dr_alias_entry *out, void *scratch, size_t scratch_bytes,
                                     cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    if (scratch_bytes < (size_t)total_n * (2 * sizeof(HeapItem) + sizeof(float)) + 512) return cudaErrorInvalidValue;
    char *p = align256(static_cast<char *>(scratch));
    HeapItem *heaps = reinterpret_cast<HeapItem *>(p);
    float *filtered = reinterpret_cast<float *>(heaps + 2 * (size_t)total_n);
    k_alias_ref_segments<<<(nseg + 63) / 64, 64, 0, st>>>(w, begin, count, nseg, out, heaps, filtered);
    return cudaGetLastError();
}

cudaError_t launch_alias_sweep_segments(const float *w, const uint32_t *begin, const uint32_t *count, uint32_t nseg,
                                       dr_alias_entry *out, cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    k_alias_sweep_segments<<<(nseg + 63) / 64, 64, 0, st>>>(w, begin, count, nseg, out);
    return cudaGetLastError();
}

cudaError_t launch_alias_sample(const dr_alias_entry *table, uint32_t n, const float *u, uint64_t draws,
                                int32_t *index, float *pdf, cudaStream_t st)
{
    if (draws == 0) return cudaSuccess;
    const uint64_t blocks = (draws + 255) / 256;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    k_alias_sample<<<(unsigned)blocks, 256, 0, st>>>(table, n, u, draws, index, pdf);
    return cudaGetLastError();
}

}  // namespace dr
