// lbvh.cu -- device construction of the binary hierarchy (replaces the host
// binned-SAH build, and the reference's generateSimpleBBH, src/models/BBH.cpp:
// 38-115, when dr_build_config.builder = DR_BUILD_DEVICE_LBVH).
//
// Linear BVH after Karras, "Maximizing Parallelism in the Construction of
// BVHs, Octrees, and k-d Trees" (HPG 2012):
//   1. centroid bounds (block reductions + atomics on order-preserving keys);
//   2. 30-bit Morton codes of the centroids;
//   3. LSD radix sort of (code, triangle) pairs, 4 passes of 8 bits, stable
//      (warp match for ranks within a tile);
//   4. the binary radix tree: internal node i covers a key range found by
//      exponential and binary search on the common-prefix length delta
//      (ties between equal codes broken by the index);
//   5. boxes bottom-up: the second child to arrive at a node unions both;
//   6. the two-box node layout of the traversal (boxes widened by the scene's
//      slack and rounded outward) and the triangle records in leaf order;
//      or, for the 8-wide layout, the collapse of the radix tree into
//      compressed 8-wide nodes (below).
// Leaves of the binary layout hold one triangle, wide leaves up to three. The result is a valid hierarchy for the
// canonical closest-hit semantics: traversal results equal the host-built
// scene's bit for bit.

#include "dr_internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace dr {
namespace {

constexpr int kSortBlock = 256;
constexpr int kSortTile = 4096;  // keys per tile
constexpr int kSortWarps = kSortBlock / 32;
constexpr int kKeysPerWarp = kSortTile / kSortWarps;  // 512

__device__ __forceinline__ uint32_t ordered(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ float3 centroid(const float *pos, uint32_t i)
{
    const float *q = pos + 9 * (size_t)i;
    return make_float3((q[0] + q[3] + q[6]) * (1.0f / 3.0f), (q[1] + q[4] + q[7]) * (1.0f / 3.0f),
                       (q[2] + q[5] + q[8]) * (1.0f / 3.0f));
}

// bounds[0..2] = ordered min, bounds[3..5] = ordered max of the centroids
__global__ void k_centroid_bounds(const float *pos, uint32_t n, uint32_t *bounds)
{
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float3 c = centroid(pos, i);
        lo[0] = fminf(lo[0], c.x), lo[1] = fminf(lo[1], c.y), lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x), hi[1] = fmaxf(hi[1], c.y), hi[2] = fmaxf(hi[2], c.z);
    }
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_down_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_down_sync(0xffffffffu, hi[a], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(bounds + a, ordered(lo[a]));
            atomicMax(bounds + 3 + a, ordered(hi[a]));
        }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(const float *pos, uint32_t n, const uint32_t *bounds, uint32_t *keys, uint32_t *vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 c = centroid(pos, i);
    float q[3] = {c.x, c.y, c.z};
    uint32_t code = 0;
    for (int a = 0; a < 3; ++a) {
        const float lo = unordered(bounds[a]), hi = unordered(bounds[3 + a]);
        const float ext = hi - lo;
        float u = ext > 0.0f ? (q[a] - lo) / ext : 0.0f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        const uint32_t v = min((uint32_t)(u * 1024.0f), 1023u);
        code |= spread10(v) << (2 - a);
    }
    keys[i] = code;
    vals[i] = i;
}

// ---- radix sort (stable LSD, 8 bits per pass) ---------------------------------

// counts[digit * tiles + tile]
__global__ void __launch_bounds__(kSortBlock) k_sort_count(const uint32_t *keys, uint32_t n, int shift, uint32_t tiles,
                                                         uint32_t *counts)
{
    __shared__ uint32_t c[256];
    c[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t i = base + threadIdx.x; i < min(n, base + kSortTile); i += kSortBlock)
        atomicAdd(&c[(keys[i] >> shift) & 0xffu], 1u);
    __syncthreads();
    counts[threadIdx.x * tiles + blockIdx.x] = c[threadIdx.x];
}

// Exclusive scan of m counts in place (one block).
__global__ void __launch_bounds__(1024) k_sort_scan(uint32_t *counts, uint32_t m)
{
    __shared__ uint32_t part[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += counts[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t v = threadIdx.x >= (uint32_t)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t v = counts[i];
        counts[i] = run;
        run += v;
    }
}

// Stable scatter of one tile: each warp takes a contiguous sub-range; ranks
// within a batch of 32 from __match_any_sync, per-warp digit prefixes from
// shared memory.
__global__ void __launch_bounds__(kSortBlock) k_sort_scatter(const uint32_t *keys, const uint32_t *vals, uint32_t n,
                                                           int shift, uint32_t tiles, const uint32_t *offsets,
                                                           uint32_t *keys_out, uint32_t *vals_out)
{
    __shared__ uint32_t wcount[kSortWarps][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortBlock) (&wcount[0][0])[i] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile + warp * kKeysPerWarp;
    const uint32_t end = min(n, base + kKeysPerWarp);
    // per-warp digit counts
    for (uint32_t i = base + lane; i < end; i += 32) atomicAdd(&wcount[warp][(keys[i] >> shift) & 0xffu], 1u);
    __syncthreads();
    // exclusive prefix across warps, plus the tile's global offset
    for (int d = threadIdx.x; d < 256; d += kSortBlock) {
        uint32_t run = offsets[d * tiles + blockIdx.x];
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t v = wcount[w][d];
            wcount[w][d] = run;
            run += v;
        }
    }
    __syncthreads();
    const unsigned lower = (1u << lane) - 1u;
    for (uint32_t b0 = base; b0 < end; b0 += 32) {
        const uint32_t i = b0 + lane;
        const bool valid = i < end;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 0xffu : 256u + (uint32_t)lane;  // invalid lanes never match
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid) {
            const uint32_t rank = (uint32_t)__popc(peers & lower);
            const uint32_t at = wcount[warp][d] + rank;
            keys_out[at] = key;
            vals_out[at] = vals[i];
        }
        __syncwarp();
        // the first lane of each peer group advances the digit's counter
        if (valid && (peers & lower) == 0) wcount[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
}

// ---- binary radix tree (Karras 2012) -------------------------------------------

__device__ __forceinline__ int delta(const uint32_t *keys, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = keys[i], b = keys[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// child encoding: >= 0 internal node, < 0 leaf ~position
__global__ void k_karras(const uint32_t *keys, int n, int2 *children, int *parent_int, int *parent_leaf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    int2 c;
    if (lo == gamma) {
        c.x = ~gamma;
        parent_leaf[gamma] = i;
    } else {
        c.x = gamma;
        parent_int[gamma] = i;
    }
    if (hi == gamma + 1) {
        c.y = ~(gamma + 1);
        parent_leaf[gamma + 1] = i;
    } else {
        c.y = gamma + 1;
        parent_int[gamma + 1] = i;
    }
    children[i] = c;
}

struct Box6 {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box6 tri_box(const float *pos, uint32_t t)
{
    const float *q = pos + 9 * (size_t)t;
    Box6 b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = fminf(fminf(q[a], q[3 + a]), q[6 + a]);
        b.hi[a] = fmaxf(fmaxf(q[a], q[3 + a]), q[6 + a]);
    }
    return b;
}

// A box and a height written by another thread block: read past L1.
__device__ __forceinline__ Box6 load_box(const Box6 *boxes, int i)
{
    const float *p = reinterpret_cast<const float *>(boxes + i);
    Box6 b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = __ldcg(p + a);
        b.hi[a] = __ldcg(p + 3 + a);
    }
    return b;
}

// Bottom-up boxes and heights: from each leaf towards the root; the second
// arrival at a node unions its children (leaves have height 0).
__global__ void k_boxes(const float *pos, const uint32_t *order, int n, const int2 *children, const int *parent_int,
                        const int *parent_leaf, uint32_t *visits, Box6 *boxes, uint32_t *height)
{
    const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    int node = parent_leaf[leaf];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(visits + node, 1u) == 0) return;  // the other child is not done yet
        __threadfence();
        const int2 c = children[node];
        Box6 a = c.x < 0 ? tri_box(pos, order[~c.x]) : load_box(boxes, c.x);
        const Box6 b = c.y < 0 ? tri_box(pos, order[~c.y]) : load_box(boxes, c.y);
        for (int k = 0; k < 3; ++k) {
            a.lo[k] = fminf(a.lo[k], b.lo[k]);
            a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
        }
        const uint32_t ha = c.x < 0 ? 0u : __ldcg(height + c.x), hb = c.y < 0 ? 0u : __ldcg(height + c.y);
        boxes[node] = a;
        height[node] = 1u + max(ha, hb);
        node = node == 0 ? -1 : parent_int[node];
    }
}

__device__ __forceinline__ float widen_down(float v, float slack) { return nextafterf(v - slack, -INFINITY); }
__device__ __forceinline__ float widen_up(float v, float slack) { return nextafterf(v + slack, INFINITY); }

// Two-box nodes: child boxes widened by the slack and rounded outward.
__global__ void k_emit_nodes(const float *pos, const uint32_t *order, int n, const int2 *children, const Box6 *boxes,
                             float slack, Bvh2Node *nodes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int2 c = children[i];
    Box6 b[2];
    b[0] = c.x < 0 ? tri_box(pos, order[~c.x]) : boxes[c.x];
    b[1] = c.y < 0 ? tri_box(pos, order[~c.y]) : boxes[c.y];
    float lo[2][3], hi[2][3];
    for (int k = 0; k < 2; ++k)
        for (int a = 0; a < 3; ++a) {
            lo[k][a] = widen_down(b[k].lo[a], slack);
            hi[k][a] = widen_up(b[k].hi[a], slack);
        }
    Bvh2Node nd;
    nd.c0xy = make_float4(lo[0][0], hi[0][0], lo[0][1], hi[0][1]);
    nd.c1xy = make_float4(lo[1][0], hi[1][0], lo[1][1], hi[1][1]);
    nd.cz = make_float4(lo[0][2], hi[0][2], lo[1][2], hi[1][2]);
    const auto link = [](int ch) { return ch >= 0 ? ch : ~int32_t(((uint32_t)(~ch) << kLeafCountBits) | 1u); };
    nd.link = make_int4(link(c.x), link(c.y), 0, 0);
    nodes[i] = nd;
}

// One triangle: a root with the leaf and an empty second child.
__global__ void k_emit_single(const float *pos, float slack, Bvh2Node *nodes)
{
    const Box6 b = tri_box(pos, 0);
    Bvh2Node nd;
    nd.c0xy = make_float4(widen_down(b.lo[0], slack), widen_up(b.hi[0], slack), widen_down(b.lo[1], slack),
                          widen_up(b.hi[1], slack));
    nd.c1xy = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    nd.cz = make_float4(widen_down(b.lo[2], slack), widen_up(b.hi[2], slack), INFINITY, -INFINITY);
    nd.link = make_int4(~int32_t((0u << kLeafCountBits) | 1u), ~int32_t(0u), 0, 0);
    nodes[0] = nd;
}

// Triangle records in leaf order, as make_tri_records (same FP32 expressions;
// this file is compiled without contraction).
__global__ void k_records(const float *pos, const uint32_t *order, uint32_t n, float4 *ref, float4 *wt, int32_t *prim)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t t = order[k];
    const float *q = pos + 9 * (size_t)t;
    const float Ax = q[0], Ay = q[1], Az = q[2];
    const float Bx = q[3], By = q[4], Bz = q[5];
    const float Cx = q[6], Cy = q[7], Cz = q[8];
    const float ux = Ax - Bx, uy = Ay - By, uz = Az - Bz;
    const float vx = Ax - Cx, vy = Ay - Cy, vz = Az - Cz;
    const float nfx = uy * vz - uz * vy;
    const float nfy = uz * vx - ux * vz;
    const float nfz = ux * vy - uy * vx;
    const float s = nfx * nfx + nfy * nfy + nfz * nfz;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (!(s < 1e-14f)) {
        const float l = sqrtf(nfx * nfx + nfy * nfy + nfz * nfz);
        nx = nfx / l;
        ny = nfy / l;
        nz = nfz / l;
    }
    const float BAx = Bx - Ax, BAy = By - Ay, BAz = Bz - Az;
    const float CAx = Cx - Ax, CAy = Cy - Ay, CAz = Cz - Az;
    ref[k * 3 + 0] = make_float4(Ax, Ay, Az, nx);
    ref[k * 3 + 1] = make_float4(ny, nz, BAx, BAy);
    ref[k * 3 + 2] = make_float4(BAz, CAx, CAy, CAz);
    wt[k * 3 + 0] = make_float4(Ax, Ay, Az, Bx);
    wt[k * 3 + 1] = make_float4(By, Bz, Cx, Cy);
    wt[k * 3 + 2] = make_float4(Cz, 0.0f, 0.0f, 0.0f);
    prim[k] = (int32_t)t;
}

// ---- compressed 8-wide hierarchy: collapse of the radix tree ---------------------
//
// The collapse of the host build (bvh_build.cpp, WideBuilder), run on the
// device over the radix tree: a bottom-up pass gives every binary node its
// box and, by dynamic programming over (subtree, slots), the least surface-
// area cost of placing the subtree in at most j child slots of a wide node
// (Ylitie, Karras and Laine, HPG 2017); a top-down pass, one kernel pair per
// level of wide nodes, writes the 80-byte nodes breadth first. Each level
// counts its nodes' internal children and leaf triangles, scans the counts
// (so the layout does not depend on thread timing) and then writes the nodes,
// the next level's work list and the triangle order.

constexpr float kWideLeafTriCost = 1.0f;
constexpr uint32_t kWideMaxLeafTris = 3;

struct alignas(16) WideDp {
    float cost[8];     // cost[j - 1]: least cost of the subtree in at most j slots
    int8_t split[8];   // split[j - 1]: the left child's share when the node is opened, 0 = one slot
    uint8_t tris;      // triangles of the subtree, counted up to 4
    uint8_t wide_leaf; // its one slot is a leaf slot (else an internal wide node)
    uint8_t pad[6];
};
static_assert(sizeof(WideDp) == 48, "WideDp is read as three 16-byte words");

__device__ __forceinline__ float box_area(const Box6 &b)
{
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (!(dx >= 0 && dy >= 0 && dz >= 0)) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// The DP entry of a radix-tree leaf (one triangle).
__device__ __forceinline__ WideDp leaf_dp(const Box6 &b)
{
    WideDp d;
    const float c = kWideLeafTriCost * box_area(b);
    for (int j = 0; j < 8; ++j) {
        d.cost[j] = c;
        d.split[j] = 0;
    }
    d.tris = 1;
    d.wide_leaf = 1;
    return d;
}

__device__ __forceinline__ WideDp load_dp(const WideDp *dp, int i)
{
    WideDp d;
    const uint4 *p = reinterpret_cast<const uint4 *>(dp + i);
    uint4 v[3];
    for (int k = 0; k < 3; ++k) v[k] = __ldcg(p + k);
    memcpy(&d, v, sizeof(WideDp));
    return d;
}

// Bottom-up boxes and collapse costs (k_boxes plus the DP of WideBuilder::solve).
__global__ void k_boxes_dp(const float *pos, const uint32_t *order, int n, const int2 *children, const int *parent_int,
                           const int *parent_leaf, uint32_t *visits, Box6 *boxes, uint32_t *height, WideDp *dp)
{
    const int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    int node = parent_leaf[leaf];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(visits + node, 1u) == 0) return;  // the other child is not done yet
        __threadfence();
        const int2 c = children[node];
        const Box6 ba = c.x < 0 ? tri_box(pos, order[~c.x]) : load_box(boxes, c.x);
        const Box6 bb = c.y < 0 ? tri_box(pos, order[~c.y]) : load_box(boxes, c.y);
        const WideDp l = c.x < 0 ? leaf_dp(ba) : load_dp(dp, c.x);
        const WideDp r = c.y < 0 ? leaf_dp(bb) : load_dp(dp, c.y);
        Box6 u = ba;
        for (int k = 0; k < 3; ++k) {
            u.lo[k] = fminf(u.lo[k], bb.lo[k]);
            u.hi[k] = fmaxf(u.hi[k], bb.hi[k]);
        }
        const float A = box_area(u);
        WideDp d;
        d.tris = (uint8_t)min(l.tris + r.tris, 4);
        float open[9];
        int8_t open_split[9];
        for (int j = 2; j <= 8; ++j) {
            open[j] = INFINITY;
            open_split[j] = 1;
            for (int k = 1; k < j; ++k) {
                const float cst = l.cost[k - 1] + r.cost[j - k - 1];
                if (cst < open[j]) {
                    open[j] = cst;
                    open_split[j] = (int8_t)k;
                }
            }
        }
        float one = A + open[8];
        d.wide_leaf = 0;
        if (d.tris <= kWideMaxLeafTris && kWideLeafTriCost * (float)d.tris * A <= one) {
            one = kWideLeafTriCost * (float)d.tris * A;
            d.wide_leaf = 1;
        }
        d.cost[0] = one;
        d.split[0] = 0;
        for (int j = 2; j <= 8; ++j) {
            const bool opened = open[j] < one;
            d.cost[j - 1] = opened ? open[j] : one;
            d.split[j - 1] = opened ? open_split[j] : (int8_t)0;
        }
        for (int k = 0; k < 6; ++k) d.pad[k] = 0;
        const uint32_t ha = c.x < 0 ? 0u : __ldcg(height + c.x), hb = c.y < 0 ? 0u : __ldcg(height + c.y);
        boxes[node] = u;
        dp[node] = d;
        height[node] = 1u + max(ha, hb);
        node = node == 0 ? -1 : parent_int[node];
    }
}

// The child slots of the wide node of internal radix node `node` (WideBuilder::
// collect / expand): up to 8 radix subtrees, internal (>= 0) or leaves (< 0).
__device__ int wide_children(int node, const int2 *children, const WideDp *dp, int out[8])
{
    const int2 c = children[node];
    auto cost = [&](int x, int j) {  // cost of subtree x in j slots
        if (x >= 0) return dp[x].cost[j - 1];
        return 0.0f;  // a radix leaf costs the same for every j: the split does not depend on it
    };
    int k_best = 1;
    float best = INFINITY;
    for (int k = 1; k < 8; ++k) {
        const float v = (c.x >= 0 ? cost(c.x, k) : 0.0f) + (c.y >= 0 ? cost(c.y, 8 - k) : 0.0f);
        if (v < best) {
            best = v;
            k_best = k;
        }
    }
    // explicit stack of (subtree, slots), expanded left first
    int st_node[16], st_j[16], sp = 0, m = 0;
    st_node[sp] = c.y, st_j[sp++] = 8 - k_best;
    st_node[sp] = c.x, st_j[sp++] = k_best;
    while (sp > 0) {
        --sp;
        const int x = st_node[sp], j = st_j[sp];
        const int8_t sp_j = x >= 0 ? dp[x].split[j - 1] : (int8_t)0;
        if (x < 0 || sp_j == 0) {
            out[m++] = x;
            continue;
        }
        const int2 cc = children[x];
        st_node[sp] = cc.y, st_j[sp++] = j - sp_j;
        st_node[sp] = cc.x, st_j[sp++] = sp_j;
    }
    return m;
}

__device__ __forceinline__ bool is_wide_leaf(int x, const WideDp *dp) { return x < 0 || dp[x].wide_leaf; }
__device__ __forceinline__ uint32_t wide_tris(int x, const WideDp *dp) { return x < 0 ? 1u : dp[x].tris; }

// Per task of the level: internal children and leaf triangles of its wide node.
__global__ void k_wide_count(const int *tasks, uint32_t ntasks, const int2 *children, const WideDp *dp,
                             uint32_t *cnt_nodes, uint32_t *cnt_tris, int num_internal)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    if (tasks[t] < 0 || tasks[t] >= num_internal) {  // never by construction; see k_wide_emit
        cnt_nodes[t] = cnt_tris[t] = 0;
        return;
    }
    int ch[8];
    const int m = wide_children(tasks[t], children, dp, ch);
    uint32_t ni = 0, nt = 0;
    for (int k = 0; k < m; ++k) {
        if (is_wide_leaf(ch[k], dp)) nt += wide_tris(ch[k], dp);
        else ++ni;
    }
    cnt_nodes[t] = ni;
    cnt_tris[t] = nt;
}

// Triangles of radix subtree x (at most 3) in leaf order.
__device__ int subtree_tris(int x, const int2 *children, const uint32_t *order, uint32_t out[3])
{
    int stack[8], sp = 0, m = 0;
    stack[sp++] = x;
    while (sp > 0 && m < 3) {
        const int y = stack[--sp];
        if (y < 0) {
            out[m++] = order[~y];
            continue;
        }
        const int2 c = children[y];
        stack[sp++] = c.y;
        stack[sp++] = c.x;
    }
    return m;
}

__device__ __forceinline__ Box6 subtree_box(int x, const float *pos, const uint32_t *order, const Box6 *boxes)
{
    return x < 0 ? tri_box(pos, order[~x]) : boxes[x];
}

// Writes the wide node of each task of the level (the host emit's encoding).
__global__ void k_wide_emit(const float *pos, const uint32_t *order, const int *tasks, const uint32_t *task_node,
                            uint32_t ntasks, const int2 *children, const WideDp *dp, const Box6 *boxes,
                            const uint32_t *scan_nodes, const uint32_t *scan_tris, uint32_t node_base,
                            uint32_t tri_base0, float slack, Bvh8Node *nodes, int *next_tasks,
                            uint32_t *next_task_node, uint32_t *order8, uint32_t max_nodes, uint32_t n)
{
    // every index below stays under max_nodes (wide nodes), n (work-list
    // entries and triangles) by construction; the checks keep a miscount from
    // writing out of bounds (the host then finds the wrong totals)
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks || task_node[t] >= max_nodes || tasks[t] < 0 || tasks[t] >= (int)n - 1) return;
    int ch[8];
    const int m = wide_children(tasks[t], children, dp, ch);
    Box6 cb[8], u;
    for (int a = 0; a < 3; ++a) {
        u.lo[a] = INFINITY;
        u.hi[a] = -INFINITY;
    }
    for (int k = 0; k < m; ++k) {
        const Box6 b = subtree_box(ch[k], pos, order, boxes);
        for (int a = 0; a < 3; ++a) {
            cb[k].lo[a] = widen_down(b.lo[a], slack);
            cb[k].hi[a] = widen_up(b.hi[a], slack);
            u.lo[a] = fminf(u.lo[a], cb[k].lo[a]);
            u.hi[a] = fmaxf(u.hi[a], cb[k].hi[a]);
        }
    }
    // octant slots: greedily the (child, slot) pair whose centroid lies
    // furthest towards the slot's corner, ties to the earlier pair
    int child_in[8];
    bool used[8];
    for (int s = 0; s < 8; ++s) child_in[s] = -1;
    for (int k = 0; k < 8; ++k) used[k] = k >= m;
    float pc[3];
    for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (u.lo[a] + u.hi[a]);
    for (int round = 0; round < m; ++round) {
        float best = -INFINITY;
        int bc = -1, bs = -1;
        for (int k = 0; k < m; ++k) {
            if (used[k]) continue;
            for (int sl = 0; sl < 8; ++sl) {
                if (child_in[sl] >= 0) continue;
                float v = 0.0f;
                for (int a = 0; a < 3; ++a) {
                    const float d = ((sl >> a) & 1) ? 1.0f : -1.0f;
                    v += d * (0.5f * (cb[k].lo[a] + cb[k].hi[a]) - pc[a]);
                }
                if (bc < 0 || v > best) {
                    best = v;
                    bc = k;
                    bs = sl;
                }
            }
        }
        used[bc] = true;
        child_in[bs] = bc;
    }
    // quantisation grid
    uint32_t ebias[3];
    double scale[3];
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)u.hi[a] - (double)u.lo[a];
        int e = -100;
        if (ext > 0.0) e = (int)ceil(log2(ext / 255.0));
        while (ldexp(255.0, e) < ext) ++e;
        e = max(-126, min(127, e));
        ebias[a] = (uint32_t)(e + 127);
        scale[a] = ldexp(1.0, e);
    }
    uint32_t qlo[3][2] = {}, qhi[3][2] = {}, meta[2] = {0u, 0u};
    for (int a = 0; a < 3; ++a) qlo[a][0] = qlo[a][1] = 0xffffffffu;  // empty slots: lo 255, hi 0
    uint32_t imask = 0, tri_off = 0, next_child = 0;
    const uint32_t child_base = node_base + scan_nodes[t];
    const uint32_t tri_base = tri_base0 + scan_tris[t];
    for (int sl = 0; sl < 8; ++sl) {
        const int k = child_in[sl];
        if (k < 0) continue;
        const int w = sl >> 2, sh = 8 * (sl & 3);
        for (int a = 0; a < 3; ++a) {
            const double lo = floor(((double)cb[k].lo[a] - (double)u.lo[a]) / scale[a]);
            const double hi = ceil(((double)cb[k].hi[a] - (double)u.lo[a]) / scale[a]);
            const uint32_t ql = (uint32_t)fmax(0.0, fmin(255.0, lo)), qh = (uint32_t)fmax(0.0, fmin(255.0, hi));
            qlo[a][w] = (qlo[a][w] & ~(0xffu << sh)) | (ql << sh);
            qhi[a][w] |= qh << sh;
        }
        const int x = ch[k];
        uint32_t mt = 0;
        if (!is_wide_leaf(x, dp)) {
            imask |= 1u << sl;
            mt = 0x20u | (24u + (uint32_t)sl);
            const uint32_t slot = scan_nodes[t] + next_child;  // position in the next level's work list
            if (slot < n && child_base + next_child < max_nodes) {
                next_tasks[slot] = x;
                next_task_node[slot] = child_base + next_child;
            }
            ++next_child;
        } else {
            uint32_t tr[3];
            const int nt = subtree_tris(x, children, order, tr);
            for (int q = 0; q < nt; ++q)
                if (tri_base + tri_off + q < n) order8[tri_base + tri_off + q] = tr[q];
            mt = ((((1u << nt) - 1u) << 5) | tri_off);
            tri_off += (uint32_t)nt;
        }
        meta[w] |= mt << sh;
    }
    Bvh8Node nd;
    nd.w[0] = make_uint4(__float_as_uint(u.lo[0]), __float_as_uint(u.lo[1]), __float_as_uint(u.lo[2]),
                         ebias[0] | (ebias[1] << 8) | (ebias[2] << 16) | (imask << 24));
    nd.w[1] = make_uint4(child_base, tri_base, meta[0], meta[1]);
    for (int a = 0; a < 3; ++a) nd.w[2 + a] = make_uint4(qlo[a][0], qlo[a][1], qhi[a][0], qhi[a][1]);
    nodes[task_node[t]] = nd;
}

// A one-triangle scene: a root whose slot 0 is the triangle's leaf.
__global__ void k_wide_single(const float *pos, float slack, Bvh8Node *nodes, uint32_t *order8)
{
    const Box6 b = tri_box(pos, 0);
    Box6 cb;
    for (int a = 0; a < 3; ++a) {
        cb.lo[a] = widen_down(b.lo[a], slack);
        cb.hi[a] = widen_up(b.hi[a], slack);
    }
    uint32_t ebias[3], ql[3], qh[3];
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)cb.hi[a] - (double)cb.lo[a];
        int e = -100;
        if (ext > 0.0) e = (int)ceil(log2(ext / 255.0));
        while (ldexp(255.0, e) < ext) ++e;
        e = max(-126, min(127, e));
        ebias[a] = (uint32_t)(e + 127);
        const double sc = ldexp(1.0, e);
        ql[a] = 0;
        qh[a] = (uint32_t)fmax(0.0, fmin(255.0, ceil(((double)cb.hi[a] - (double)cb.lo[a]) / sc)));
    }
    Bvh8Node nd;
    nd.w[0] = make_uint4(__float_as_uint(cb.lo[0]), __float_as_uint(cb.lo[1]), __float_as_uint(cb.lo[2]),
                         ebias[0] | (ebias[1] << 8) | (ebias[2] << 16));
    nd.w[1] = make_uint4(1u, 0u, 0x20u, 0u);  // slot 0: one triangle at offset 0
    for (int a = 0; a < 3; ++a) nd.w[2 + a] = make_uint4(0xffffff00u | ql[a], 0xffffffffu, qh[a], 0u);
    nodes[0] = nd;
    order8[0] = 0;
}

unsigned grid_for(uint64_t n, unsigned block) { return (unsigned)std::max<uint64_t>(1, (n + block - 1) / block); }

}  // namespace

// Builds nodes, records and the index map of `s` on the device from host
// positions (n >= 1): the radix tree's binary nodes (layout 2) or its collapse
// into compressed 8-wide nodes (layout 8). Sets num_nodes and depth.
dr_status build_lbvh_device(dr_scene *s, const float *positions_host, uint32_t n, float slack, uint32_t layout)
{
    cudaError_t e = cudaSuccess;
    float *pos = nullptr;
    uint32_t *scratch = nullptr;
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    // keys, vals, keys2, vals2, counts, parents (2n), visits, heights, bounds
    const size_t words = (size_t)4 * n + (size_t)256 * tiles + 4 * (size_t)n + 16;
    Box6 *boxes = nullptr;
    int2 *children = nullptr;
    WideDp *dp = nullptr;
    int *tasks = nullptr;         // wide build: two work lists of radix nodes
    uint32_t *wide_tmp = nullptr; // task nodes (2 lists), node and triangle counts, the triangle order
    Bvh8Node *nodes8 = nullptr;   // wide nodes before they are copied to their final size
    const size_t nint = n > 1 ? n - 1 : 1;
    auto done = [&](dr_status st) {
        cudaFree(pos);
        cudaFree(scratch);
        cudaFree(boxes);
        cudaFree(children);
        cudaFree(dp);
        cudaFree(tasks);
        cudaFree(wide_tmp);
        cudaFree(nodes8);
        return st;
    };
    if ((e = dev_malloc(&pos, (size_t)n * 9 * sizeof(float))) != cudaSuccess ||
        (e = dev_malloc(&scratch, words * sizeof(uint32_t))) != cudaSuccess ||
        (e = dev_malloc(&boxes, nint * sizeof(Box6))) != cudaSuccess ||
        (e = dev_malloc(&children, nint * sizeof(int2))) != cudaSuccess ||
        (e = cudaMemcpy(pos, positions_host, (size_t)n * 9 * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
        return done(cuda_fail(e, "device BVH build: allocation"));
    uint32_t *keys = scratch, *vals = keys + n, *keys2 = vals + n, *vals2 = keys2 + n;
    uint32_t *counts = vals2 + n;
    int *parent_int = reinterpret_cast<int *>(counts + (size_t)256 * tiles);
    int *parent_leaf = parent_int + n;
    uint32_t *visits = reinterpret_cast<uint32_t *>(parent_leaf + n);
    uint32_t *heights = visits + n;
    uint32_t *bounds = heights + n;  // 6 words
    const uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    if ((e = cudaMemcpy(bounds, init, sizeof(init), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(visits, 0, (size_t)n * sizeof(uint32_t))) != cudaSuccess)
        return done(cuda_fail(e, "device BVH build: initialisation"));
    const unsigned reduce_blocks = std::min<unsigned>(grid_for(n, 256), (unsigned)s->ctx->num_sms * 8);
    k_centroid_bounds<<<reduce_blocks, 256>>>(pos, n, bounds);
    k_morton<<<grid_for(n, 256), 256>>>(pos, n, bounds, keys, vals);
    for (int shift = 0; shift < 32; shift += 8) {
        k_sort_count<<<tiles, kSortBlock>>>(keys, n, shift, tiles, counts);
        k_sort_scan<<<1, 1024>>>(counts, 256 * tiles);
        k_sort_scatter<<<tiles, kSortBlock>>>(keys, vals, n, shift, tiles, counts, keys2, vals2);
        std::swap(keys, keys2);
        std::swap(vals, vals2);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return done(cuda_fail(e, "device BVH build: sort"));
    uint32_t num_nodes = 1;
    uint32_t depth = 1;
    const uint32_t *tri_order = vals;  // leaf position -> triangle of the records
    if (layout == 8) {
        // the triangle order of the wide leaves, then per level the work lists
        uint32_t *order8 = nullptr;
        if ((e = dev_malloc(&wide_tmp, ((size_t)n * 4 + 2) * sizeof(uint32_t))) != cudaSuccess ||
            (e = dev_malloc(&nodes8, nint * sizeof(Bvh8Node))) != cudaSuccess)
            return done(cuda_fail(e, "device BVH build: wide nodes"));
        order8 = wide_tmp;
        uint32_t *task_node[2] = {wide_tmp + n, wide_tmp + 2 * (size_t)n};
        uint32_t *cnt_nodes = wide_tmp + 3 * (size_t)n;  // n + 1 entries
        if (n == 1) {
            k_wide_single<<<1, 1>>>(pos, slack, nodes8, order8);
        } else {
            uint32_t *cnt2 = nullptr;  // triangle counts, n + 1 entries
            if ((e = dev_malloc(&dp, (n - 1) * sizeof(WideDp))) != cudaSuccess ||
                (e = dev_malloc(&tasks, 2 * (size_t)n * sizeof(int))) != cudaSuccess ||
                (e = dev_malloc(&cnt2, ((size_t)n + 1) * sizeof(uint32_t))) != cudaSuccess) {
                cudaFree(cnt2);
                return done(cuda_fail(e, "device BVH build: wide collapse"));
            }
            uint32_t *cnt_tris = cnt2;
            k_karras<<<grid_for(n - 1, 256), 256>>>(keys, (int)n, children, parent_int, parent_leaf);
            k_boxes_dp<<<grid_for(n, 256), 256>>>(pos, vals, (int)n, children, parent_int, parent_leaf, visits, boxes,
                                                  heights, dp);
            int *list[2] = {tasks, tasks + n};
            if ((e = cudaMemset(tasks, 0, 2 * (size_t)n * sizeof(int))) != cudaSuccess ||
                (e = cudaMemset(task_node[0], 0, 2 * (size_t)n * sizeof(uint32_t))) != cudaSuccess) {
                cudaFree(cnt2);
                return done(cuda_fail(e, "device BVH build: wide collapse"));
            }
            const int root = 0;
            const uint32_t zero = 0;
            if ((e = cudaMemcpy(list[0], &root, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
                (e = cudaMemcpy(task_node[0], &zero, sizeof(uint32_t), cudaMemcpyHostToDevice)) != cudaSuccess) {
                cudaFree(cnt2);
                return done(cuda_fail(e, "device BVH build: wide collapse"));
            }
            uint32_t ntasks = 1, node_base = 1, tri_base = 0, levels = 0;
            while (ntasks > 0 && e == cudaSuccess) {
                const unsigned g = grid_for(ntasks, 128);
                k_wide_count<<<g, 128>>>(list[0], ntasks, children, dp, cnt_nodes, cnt_tris, (int)n - 1);
                // exclusive scans over ntasks + 1 entries: the last one becomes the level's total
                if ((e = cudaMemset(cnt_nodes + ntasks, 0, sizeof(uint32_t))) != cudaSuccess ||
                    (e = cudaMemset(cnt_tris + ntasks, 0, sizeof(uint32_t))) != cudaSuccess)
                    break;
                k_sort_scan<<<1, 1024>>>(cnt_nodes, ntasks + 1);
                k_sort_scan<<<1, 1024>>>(cnt_tris, ntasks + 1);
                k_wide_emit<<<g, 128>>>(pos, vals, list[0], task_node[0], ntasks, children, dp, boxes, cnt_nodes,
                                        cnt_tris, node_base, tri_base, slack, nodes8, list[1], task_node[1], order8,
                                        (uint32_t)nint, n);
                uint32_t totals[2];
                if ((e = cudaMemcpy(&totals[0], cnt_nodes + ntasks, sizeof(uint32_t), cudaMemcpyDeviceToHost)) !=
                        cudaSuccess ||
                    (e = cudaMemcpy(&totals[1], cnt_tris + ntasks, sizeof(uint32_t), cudaMemcpyDeviceToHost)) !=
                        cudaSuccess)
                    break;
                ++levels;
                ntasks = totals[0];
                node_base += totals[0];
                tri_base += totals[1];
                std::swap(list[0], list[1]);
                std::swap(task_node[0], task_node[1]);
                if (levels > (uint32_t)kMaxBuildDepth || node_base > nint) break;
            }
            cudaFree(cnt2);
            if (e != cudaSuccess) return done(cuda_fail(e, "device BVH build: wide collapse"));
            if (levels > (uint32_t)kMaxBuildDepth)
                return done(fail(DR_ERR_TOO_LARGE, "device BVH build: more than %d wide levels", kMaxBuildDepth));
            if (tri_base != n || node_base > nint)
                return done(fail(DR_ERR_CUDA, "device BVH build: wide collapse placed %u of %u triangles", tri_base,
                                 n));
            num_nodes = node_base;
            depth = levels;
        }
        if ((e = dev_malloc(&s->d_nodes8, (size_t)num_nodes * sizeof(Bvh8Node))) != cudaSuccess ||
            (e = cudaMemcpy(s->d_nodes8, nodes8, (size_t)num_nodes * sizeof(Bvh8Node), cudaMemcpyDeviceToDevice)) !=
                cudaSuccess)
            return done(cuda_fail(e, "device BVH build: wide nodes"));
        s->device_bytes += (size_t)num_nodes * sizeof(Bvh8Node);
        tri_order = order8;
    } else if (n == 1) {
        if ((e = dev_malloc(&s->d_nodes, sizeof(Bvh2Node))) != cudaSuccess) return done(cuda_fail(e, "device BVH build"));
        k_emit_single<<<1, 1>>>(pos, slack, s->d_nodes);
        s->device_bytes += sizeof(Bvh2Node);
    } else {
        num_nodes = n - 1;
        k_karras<<<grid_for(n - 1, 256), 256>>>(keys, (int)n, children, parent_int, parent_leaf);
        k_boxes<<<grid_for(n, 256), 256>>>(pos, vals, (int)n, children, parent_int, parent_leaf, visits, boxes, heights);
        if ((e = dev_malloc(&s->d_nodes, (size_t)num_nodes * sizeof(Bvh2Node))) != cudaSuccess)
            return done(cuda_fail(e, "device BVH build: nodes"));
        k_emit_nodes<<<grid_for(n - 1, 256), 256>>>(pos, vals, (int)n, children, boxes, slack, s->d_nodes);
        // root height (edges) + 1 = nodes on the longest root-to-leaf path
        if ((e = cudaMemcpy(&depth, heights, sizeof(uint32_t), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return done(cuda_fail(e, "device BVH build: depth"));
        depth += 1;
        s->device_bytes += (size_t)num_nodes * sizeof(Bvh2Node);
    }
    if ((e = dev_malloc(&s->d_tri_ref, (size_t)n * 3 * sizeof(float4))) != cudaSuccess ||
        (e = dev_malloc(&s->d_tri_wt, (size_t)n * 3 * sizeof(float4))) != cudaSuccess ||
        (e = dev_malloc(&s->d_prim, (size_t)n * sizeof(int32_t))) != cudaSuccess)
        return done(cuda_fail(e, "device BVH build: records"));
    s->device_bytes += (size_t)n * (2 * 3 * sizeof(float4) + sizeof(int32_t));
    k_records<<<grid_for(n, 256), 256>>>(pos, tri_order, n, s->d_tri_ref, s->d_tri_wt, s->d_prim);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return done(cuda_fail(e, "device BVH build"));
    s->num_nodes = num_nodes;
    s->depth = depth;
    if (depth > (uint32_t)kMaxBuildDepth)
        return done(fail(DR_ERR_TOO_LARGE, "device BVH build: depth %u exceeds the traversal stack (%d)", depth,
                         kMaxBuildDepth));
    return done(DR_OK);
}

}  // namespace dr
