// tri_batch.cuh -- warp triangle batches for the persistent wide traversal.
//
// The leaf triangles a node test finds are not tested by their own lane.
// Their records are staged into the warp's shared-memory batch by bulk
// asynchronous copies (cp.async.bulk, completing on the warp's mbarrier) while
// the lanes go on to their next nodes. When the batch is full, or enough lanes
// wait for their results, the warp tests the whole batch at once, one
// (ray, triangle) pair per lane, and each ray keeps the smallest (t, index) of
// its pairs. A lane's per-node triangle loop ran with 1-2 of 32 lanes active;
// the batch runs with up to 32. The closest hit is the same: every pair is
// tested, and the minimum over pairs does not depend on the order.
#pragma once

#include "mbarrier.cuh"
#include "trace_wide.cuh"

namespace dr {

// Pairs per warp batch (one per lane when full).
constexpr uint32_t kTriBatch = 32;

// Shared-memory batch of one warp.
struct alignas(16) TriBatch {
    float4 rec[kTriBatch][3];          // staged triangle records (48 B each)
    unsigned long long key[32];        // per owner lane: min of (t, original index)
    uint64_t bar;                      // mbarrier of the staging copies
    uint32_t tri[kTriBatch];           // leaf-order triangle of each pair
    uint32_t tbits[32];                // per owner lane: the exact t of the winner
    uint8_t owner[kTriBatch];          // owner lane of each pair
    uint32_t any;                      // any-hit: owner lanes with a hit
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tb_init(TriBatch &B, int lane)
{
    B.key[lane] = ~0ull;
    if (lane == 0) {
        B.any = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&B.bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();
}

// Stages the records of `tmask` (bits relative to tbase) into slots from
// `slot`, one bulk copy per run of consecutive triangles.
__device__ __forceinline__ void tb_append(TriBatch &B, const float4 *recs, uint32_t slot, uint32_t tbase,
                                          uint32_t tmask, int lane)
{
    const uint32_t bar = smem_u32(&B.bar);
    const uint32_t bytes = 48u * (uint32_t)__popc(tmask);
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
    uint32_t m = tmask;
    while (m) {
        const int lo = __ffs(m) - 1;
        const uint32_t run = (uint32_t)__ffs(~(m >> lo)) - 1u;
        for (uint32_t r = 0; r < run; ++r) {
            B.tri[slot + r] = tbase + (uint32_t)lo + r;
            B.owner[slot + r] = (uint8_t)lane;
        }
        const float4 *src = recs + 3 * (size_t)(tbase + (uint32_t)lo);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                         smem_u32(&B.rec[slot][0])),
                     "l"(src), "r"(48u * run), "r"(bar)
                     : "memory");
        slot += run;
        m &= ~(((1u << run) - 1u) << lo);
    }
}

// Bounded wait of the whole warp for the staging copies of the current phase
// (one decision for the warp).
__device__ __forceinline__ bool tb_wait(TriBatch &B, uint32_t phase)
{
    return __all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&B.bar), phase, kMbarWaitPolls));
}

// Tests the batch's n pairs, one per lane. Closest hit: each owner lane's
// (best_t, best_prim) takes the smallest (t, index) of its pairs. Any hit:
// returns true for owner lanes with a hit. `phase` flips. If the staging
// copies do not land within the wait's limit, the warp sets ERR_TIMEOUT,
// waits once more (bounded) so that no copy is left writing its shared
// memory, tests nothing and sets `aborted`: the caller stops the warp (the
// rays it held keep no result; the call reports DR_ERR_TIMEOUT).
template <int MODE, bool ANY>
__device__ __forceinline__ bool tb_flush(const Wide8Args &a, TriBatch &B, uint32_t n, uint32_t &phase, WideState &s,
                                         int lane, unsigned long long &nt, bool &aborted)
{
    constexpr unsigned FULL = 0xffffffffu;
    __syncwarp();
    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&B.bar)) : "memory");
    if (!tb_wait(B, phase)) {
        if (lane == 0) atomicOr(a.error, ERR_TIMEOUT);
        tb_wait(B, phase);
        aborted = true;
        return false;
    }
    phase ^= 1u;
    const bool have = (uint32_t)lane < n;
    const int owner = have ? (int)B.owner[lane] : lane;
    // the owner's ray and bound
    DevRay r;
    r.o.x = __shfl_sync(FULL, s.r.o.x, owner);
    r.o.y = __shfl_sync(FULL, s.r.o.y, owner);
    r.o.z = __shfl_sync(FULL, s.r.o.z, owner);
    r.v.x = __shfl_sync(FULL, s.r.v.x, owner);
    r.v.y = __shfl_sync(FULL, s.r.v.y, owner);
    r.v.z = __shfl_sync(FULL, s.r.v.z, owner);
    const float bound = __shfl_sync(FULL, ANY ? s.r.tmax : s.best_t, owner);
    WtSetup w{};
    if (MODE == 1) {
        const int k = __shfl_sync(FULL, s.w.kx | (s.w.ky << 2) | (s.w.kz << 4), owner);
        w.kx = k & 3;
        w.ky = (k >> 2) & 3;
        w.kz = (k >> 4) & 3;
        w.Sx = __shfl_sync(FULL, s.w.Sx, owner);
        w.Sy = __shfl_sync(FULL, s.w.Sy, owner);
        w.Sz = __shfl_sync(FULL, s.w.Sz, owner);
    }
    bool hit = false;
    float t = 0.0f;
    unsigned long long key = 0;
    if (have) {
        ++nt;
        const float4 r0 = B.rec[lane][0], r1 = B.rec[lane][1], r2 = B.rec[lane][2];
        hit = MODE == 1 ? tri_test_wt_words(r0, r1, r2, r, w, bound, t) : tri_test_ref_words(r0, r1, r2, r, bound, t);
        if (hit) {
            if (ANY) {
                atomicOr(&B.any, 1u << owner);
            } else {
                const uint32_t prim = (uint32_t)DR_LD(a.prim + B.tri[lane]);
                // t >= 0 (t + 0 turns -0 into +0), so its bits order like its value
                key = ((unsigned long long)__float_as_uint(t + 0.0f) << 32) | prim;
                atomicMin(&B.key[owner], key);
            }
        }
    }
    __syncwarp();
    bool found = false;
    if (ANY) {
        found = (B.any >> lane) & 1u;
        __syncwarp();
        if (lane == 0) B.any = 0;
    } else {
        if (hit && B.key[owner] == key) B.tbits[owner] = __float_as_uint(t);
        __syncwarp();
        const unsigned long long k = B.key[lane];
        if (k != ~0ull) {
            const float tk = __uint_as_float(B.tbits[lane]);
            const int32_t pk = (int32_t)(uint32_t)(k & 0xffffffffull);
            if (tk < s.best_t || (tk == s.best_t && pk < s.best_prim)) {
                s.best_t = tk;
                s.best_prim = pk;
            }
            B.key[lane] = ~0ull;
        }
    }
    // the records are rewritten by the next copies (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncwarp();
    return found;
}

}  // namespace dr
