// persistent.cuh -- persistent-warp traversal over the compressed 8-wide BVH.
//
// A warp keeps all 32 lanes busy: whenever lanes have finished their ray they
// take the next ray indices from a chunk the warp reserved with one atomic add
// (up to 64 indices per chunk), so a slow ray no longer idles the other 31 lanes of
// its warp (Aila and Laine, "Understanding the Efficiency of Ray Traversal on
// GPUs", HPG 2009, persistent threads with dynamic fetch). Each loop iteration
// advances every active lane by one to DR_INNER_STEPS_* nodes (8 boxes each)
// and then handles the leaf triangles found. The traversal of a single ray is
// unchanged, so results stay bit-identical.
#pragma once

#include "trace_kernels.cuh"
#include "trace_wide.cuh"
#include "tri_batch.cuh"

namespace dr {

// Largest ray-index chunk a warp reserves at once. Measured (incoherent
// closest hit / many-light 1080p render / box room): 64 -> 4.45 Grays/s,
// 51.9 ms, 2.50 ms; 128 -> 4.44, 52.6, 2.62; 256 -> 4.38, 52.9, 2.67.
#ifndef DR_PERSISTENT_CHUNK
#define DR_PERSISTENT_CHUNK 64
#endif
constexpr uint32_t kPersistentChunk = DR_PERSISTENT_CHUNK;

// Resident blocks per SM the persistent kernels are compiled for (8 blocks of
// 128 threads: at most 64 registers per thread).
#ifndef DR_P8_MIN_BLOCKS
#define DR_P8_MIN_BLOCKS 8
#endif
constexpr int kP8MinBlocks = DR_P8_MIN_BLOCKS;

// A warp refills its idle lanes once at least this many are idle (or all are):
// fewer, fuller refills (measured on the incoherent workload: 1 -> 3.68,
// 4 -> 3.78, 8 -> 3.78, 16 -> 3.54 Grays/s with one node test per loop
// iteration; with up to 4: 2 -> 4.88, 4 -> 4.89, 8 -> 4.86, 16 -> 4.41).
#ifndef DR_REFILL_MIN
#define DR_REFILL_MIN 4
#endif
// A lane postpones its leaf triangles while fewer than this many lanes of its
// warp have triangles to test (0: never). Measured on the incoherent workload
// (2^20 triangles, 16.8 M rays): 0 -> 3.75, 4 -> 3.67, 8..16 -> 3.66 Grays/s,
// so it stays off; results are identical either way.
#ifndef DR_POSTPONE_MIN
#define DR_POSTPONE_MIN 0
#endif
// Which traversals send their leaf triangles through the warp's staged
// triangle batch (tri_batch.cuh) instead of each lane's own loop: the public
// closest-hit and any-hit kernels, the renderer's path rays and shadow rays.
// Measured (incoherent workload: 2^20 triangles, 16.8 M rays, 23 % hits;
// many-light 1080p and box-room renders, 16 spp): closest hit 3.81 -> 4.37
// Grays/s and any hit 3.43 -> 3.35 ms with the batch; the renders 51.9 ->
// 53.4 ms and 2.50 -> 2.90 ms with the path rays batched, 53.0 and 2.87 ms
// with the shadow rays batched. Path and shadow rays of a closed scene nearly
// all hit, and the batch delays the early exits and the shrinking closest-hit
// bound that then prune the traversal; the public rays mostly miss, so the
// batch only saves issue slots.
#ifndef DR_TRI_BATCH_CLOSEST
#define DR_TRI_BATCH_CLOSEST 1
#endif
#ifndef DR_TRI_BATCH_ANY
#define DR_TRI_BATCH_ANY 1
#endif
#ifndef DR_TRI_BATCH_PATHS
#define DR_TRI_BATCH_PATHS 0
#endif
#ifndef DR_TRI_BATCH_SHADOW
#define DR_TRI_BATCH_SHADOW 0
#endif
// The batch is tested once it holds this many pairs, or once this many lanes
// wait for its results (their rays have no node left). Measured: 16 -> 4.38,
// 24 -> 4.37, 32 -> 4.24 Grays/s; 3, 6 or 10 waiting lanes all 4.37. With up
// to 4 node tests per iteration and the collapsed tree: 12 / 16 / 24 pairs ->
// 4.963 / 4.956 / 4.838 Grays/s closest hit, 2.92 / 2.95 / 3.04 ms any hit.
#ifndef DR_TRI_BATCH_FLUSH
#define DR_TRI_BATCH_FLUSH 12
#endif
#ifndef DR_TRI_BATCH_WAITERS
#define DR_TRI_BATCH_WAITERS 6
#endif
// Node tests per loop iteration: after its node test, a lane that found no
// leaf triangles goes on to its next node at once, up to this many nodes,
// while at least DR_INNER_MIN_LANES_* lanes of the warp can do so; the warp's
// triangle, batch and refill steps then run once for all of them (the
// "while-while" loop of Aila and Laine 2009). Separate counts for the
// traversals with warp triangle batches and for those with per-lane loops.
// Measured (incoherent closest hit and any hit, 2^20 triangles, 16.8 M rays;
// many-light 1080p render, 16 spp), with at least 16 lanes:
//   batch steps 1 / 2 / 3 / 4 / 6 / 8: 4.43 / 4.78 / 4.83 / 4.86 / 4.72 /
//   4.70 Grays/s closest hit, 3.36 / 3.08 / 3.05 / 2.99 / 3.08 / 3.10 ms any
//   hit; 8 steps with at least 24 lanes 4.86, 28 lanes 4.65 Grays/s;
//   per-lane steps 1 / 2 / 3 / 4: render 52.2 / 50.0 / 50.1 / 49.4 ms;
//   4 batch steps with at least 12 / 16 / 20 / 24 lanes: 4.84 / 4.86 / 4.89 /
//   4.86 Grays/s; 4 per-lane steps with 24 lanes: render 50.8 ms. Letting
//   lanes with leaf triangles push them as a postponed group and go on in
//   the extra node tests: 4.96 -> 4.63 Grays/s. Re-measured with the FP16
//   planes and FMA hit bits (closest / any hit, ms): 4 steps with 20 lanes
//   3.192 / 2.793; 5 or 6 steps 3.208 / 2.803 and 3.213 / 2.809; 16 lanes
//   3.196 / 2.796; 24 lanes 3.233 / 2.820; batch flush at 10 or 16 pairs
//   3.198 / 2.784 and 3.198 / 2.823; refills at 2 or 6 idle lanes 3.191 /
//   2.790 and 3.193 / 2.794.
// Results do not depend on it.
#ifndef DR_INNER_STEPS_BATCH
#define DR_INNER_STEPS_BATCH 4
#endif
#ifndef DR_INNER_STEPS_LANE
#define DR_INNER_STEPS_LANE 4
#endif
#ifndef DR_INNER_MIN_LANES_BATCH
#define DR_INNER_MIN_LANES_BATCH 20
#endif
#ifndef DR_INNER_MIN_LANES_LANE
#define DR_INNER_MIN_LANES_LANE 16
#endif



// Indices a warp reserves at once: 128 when there is plenty of work, down to
// one per lane when few rays are left, so a small launch still spreads over
// many warps (warp-uniform). A nonzero `fixed` (a multiple of 32) overrides it.
__device__ __forceinline__ uint32_t persistent_chunk(uint64_t n, uint32_t fixed = 0)
{
    if (fixed) return fixed;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
    const uint64_t per = n / (warps ? warps : 1);
    uint32_t c = per >= kPersistentChunk ? kPersistentChunk : (uint32_t)((per + 31) & ~31ull);
    return c < 32 ? 32 : c;
}

// Ray source of the public entry points: ray i of a contiguous array, all rays
// in one hierarchy. A source's load() gives the ray and the root node of the
// hierarchy it is traced in (kNoRoot: nothing to traverse, the ray misses).
struct DirectSource {
    const dr_ray *rays;
    dr_hit *hits;
    uint8_t *occluded;
    uint32_t root;
    __device__ __forceinline__ bool load(uint64_t i, DevRay &r, uint32_t &node) const
    {
        node = root;
        return load_ray(rays, i, r);
    }
    __device__ __forceinline__ void closest(uint64_t i, float t, int32_t prim) const
    {
        reinterpret_cast<float2 *>(hits)[i] =
            prim != INT_MAX ? make_float2(t, __int_as_float(prim))
                            : make_float2(__int_as_float(0x7f800000), __int_as_float(-1));
    }
    __device__ __forceinline__ void any(uint64_t i, bool hit) const { occluded[i] = hit ? 1 : 0; }
};

template <int MODE, bool ANY, bool COUNT, bool BATCH, int STACK = DR_SMEM_STACK, class Source>
__device__ __forceinline__ void persistent_wide(const Wide8Args &a, const Source &src, uint64_t n,
                                                unsigned long long *counter, unsigned long long &nn,
                                                unsigned long long &nb, unsigned long long &nt,
                                                unsigned long long &nhits, uint32_t fixed_chunk = 0)
{
    constexpr unsigned FULL = 0xffffffffu;
    constexpr bool HALF = !ANY && DR_HALF_CVT;  // node tests with FP16 grid planes (closest hit)
    constexpr bool LUT = !DR_NO_OCT_ORDER && (DR_OCT_LUT == 1 || (DR_OCT_LUT == 2 && ANY));
    const uint8_t *oct_lut = nullptr;
    if constexpr (LUT) {
        // entry (oct << 8) | m: mask m with bit s moved to bit s ^ oct (every
        // thread of the block calls this function first)
        __shared__ uint8_t s_oct[8 * 256];
        for (uint32_t i = threadIdx.x; i < 8 * 256; i += blockDim.x) {
            const uint32_t o = i >> 8, m = i & 255u;
            uint32_t t = 0;
            for (uint32_t b = 0; b < 8; ++b) t |= ((m >> b) & 1u) << (b ^ o);
            s_oct[i] = (uint8_t)t;
        }
        __syncthreads();
        oct_lut = s_oct;
    }
    const int lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    WideState s;
    LaneStackT<STACK> stack;
    if constexpr (STACK > 0) {
        __shared__ uint2 s_stack[kTraceBlock / 32][STACK > 0 ? STACK : 1][32];
        stack.shared = &s_stack[threadIdx.x >> 5][0][threadIdx.x & 31];
    } else {
        stack.shared = nullptr;
    }
    TriBatch *batch = nullptr;
    if constexpr (BATCH) {
        __shared__ TriBatch s_batch[kTraceBlock / 32];
        batch = &s_batch[threadIdx.x >> 5];
        tb_init(*batch, lane);
    }
    const float4 *recs = MODE == 1 ? a.tri_wt : a.tri_ref;
    uint32_t nbatch = 0, phase = 0;  // warp-uniform
    uint32_t pend = 0;               // this lane's pairs in the batch
    bool waiting = false;            // no node left; results of its pairs pending
    uint64_t idx = 0;
    bool active = false, exhausted = false;
    uint64_t chunk_next = 0, chunk_end = 0;  // warp-uniform
    const uint32_t chunk = persistent_chunk(n, fixed_chunk);
    unsigned long long cn = 0, cb = 0, ct = 0, ch = 0;
    while (true) {
        unsigned want = __ballot_sync(FULL, !active);
        // refill once enough lanes are idle (or none is busy)
        if (DR_REFILL_MIN > 1 && want != FULL && __popc(want) < DR_REFILL_MIN) want = 0;
        while (want != 0 && !exhausted) {
            if (chunk_next == chunk_end) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(counter, (unsigned long long)chunk);
                b = __shfl_sync(FULL, b, 0);
                if (b >= n) {
                    exhausted = true;
                    break;
                }
                chunk_next = b;
                chunk_end = b + chunk < n ? b + chunk : n;
            }
            const uint32_t avail = (uint32_t)(chunk_end - chunk_next);
            const bool take = ((want >> lane) & 1u) && (uint32_t)__popc(want & lower) < avail;
            const unsigned took = __ballot_sync(FULL, take);
            if (take) {
                idx = chunk_next + (uint64_t)__popc(want & lower);
                DevRay r;
                uint32_t root;
                if (src.load(idx, r, root) && root != kNoRoot) {
                    wide_init<MODE>(s, r, root);
                    active = true;
                } else if (ANY) {
                    src.any(idx, false);
                } else {
                    src.closest(idx, 0.0f, INT_MAX);
                }
            }
            chunk_next += (uint64_t)__popc(took);
            want &= ~took;
        }
        const unsigned busy = __ballot_sync(FULL, active);
        if (busy == 0) {
            if (exhausted) break;
            continue;
        }
        bool done = false, found = false;
        bool fin = false;  // no node left (found during the extra node tests)
        if constexpr (BATCH) {
            // 1. node test(s)
            if (active && !waiting && s.have_node) wide_visit<MODE, HALF, LUT>(a, s, cn, cb, oct_lut);
#pragma unroll 1
            for (int k = 1; k < DR_INNER_STEPS_BATCH; ++k) {
                const bool go = active && !waiting && !fin && s.tmask == 0;
                if (__popc(__ballot_sync(FULL, go)) < DR_INNER_MIN_LANES_BATCH) break;
                if (go) {
                    fin = wide_advance<ANY>(a, s, stack);
                    if (!fin && s.have_node) wide_visit<MODE, HALF, LUT>(a, s, cn, cb, oct_lut);
                }
            }
            // 2. leaf triangles join the warp batch (whole groups, in lane
            //    order, while they fit); a group that does not fit waits for
            //    the next round
            const uint32_t c = active && !waiting ? (uint32_t)__popc(s.tmask) : 0u;
            uint32_t incl = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(FULL, incl, d);
                if (lane >= d) incl += v;
            }
            const bool fits = c != 0 && nbatch + incl <= kTriBatch;
            if (fits) {
                tb_append(*batch, recs, nbatch + incl - c, s.tbase, s.tmask, lane);
                pend += c;
                s.tmask = 0;
            }
            const bool overflow = __ballot_sync(FULL, c != 0 && !fits) != 0;
            nbatch += __reduce_max_sync(FULL, fits ? incl : 0u);
            // 3. next node; a ray with no node left waits for its pairs' results
            if (active && !waiting && s.tmask == 0) {
                done = fin || wide_advance<ANY>(a, s, stack);
                if (done && pend != 0) {
                    waiting = true;
                    done = false;
                }
            }
            // 4. test the batch when full, when enough lanes wait, or when
            //    nothing else can progress
            const unsigned waiters = __ballot_sync(FULL, waiting);
            if (nbatch != 0 && (overflow || nbatch >= DR_TRI_BATCH_FLUSH || __popc(waiters) >= DR_TRI_BATCH_WAITERS ||
                                waiters == __ballot_sync(FULL, active))) {
                bool aborted = false;
                const bool hit = tb_flush<MODE, ANY>(a, *batch, nbatch, phase, s, lane, ct, aborted);
                if (aborted) break;  // warp-uniform: the staging copies timed out
                nbatch = 0;
                if (active && pend != 0) {
                    pend = 0;
                    if (waiting) {
                        done = true;
                        found = hit;
                        waiting = false;
                    } else if (ANY && hit) {
                        done = found = true;
                    }
                }
            }
        } else {
            // 1. node test(s)
            if (active && s.have_node) wide_visit<MODE, HALF, LUT>(a, s, cn, cb, oct_lut);
#pragma unroll 1
            for (int k = 1; k < DR_INNER_STEPS_LANE; ++k) {
                const bool go = active && !fin && s.tmask == 0;
                if (__popc(__ballot_sync(FULL, go)) < DR_INNER_MIN_LANES_LANE) break;
                if (go) {
                    fin = wide_advance<ANY>(a, s, stack);
                    if (!fin && s.have_node) wide_visit<MODE, HALF, LUT>(a, s, cn, cb, oct_lut);
                }
            }
            // 2. leaf triangles: tested now when enough lanes of the warp have
            //    some (or the lane has no node to go to); otherwise pushed as a
            //    group and tested when popped (Ylitie, Karras and Laine 2017,
            //    triangle postponing). Results do not depend on the order of
            //    the tests.
            const bool has_tri = active && s.tmask != 0;
            const unsigned tri_lanes = __ballot_sync(FULL, has_tri);
            if (has_tri) {
                const bool postpone = DR_POSTPONE_MIN > 0 && __popc(tri_lanes) < DR_POSTPONE_MIN &&
                                      (s.group.y >> 8) != 0 && s.sp < kWideStack - 8;
                if (postpone) {
                    stack.put(s.sp++, make_uint2(s.tbase, s.tmask | kTriGroupFlag));
                    s.tmask = 0;
                } else if (wide_triangles<MODE, ANY>(a, s, ct)) {
                    done = found = true;
                }
            }
            // 3. next node
            if (active && !done && s.tmask == 0) done = fin || wide_advance<ANY>(a, s, stack);
        }
        if (active && done) {
            if (ANY) {
                src.any(idx, found);
            } else {
                src.closest(idx, s.best_t, s.best_prim);
                if (s.best_prim != INT_MAX) ++ch;
            }
            active = false;
        }
    }
    if (COUNT) {
        nn += cn;
        nb += cb;
        nt += ct;
        nhits += ch;
    }
}

}  // namespace dr
