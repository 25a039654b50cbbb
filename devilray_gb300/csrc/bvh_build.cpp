// bvh_build.cpp -- host binned-SAH BVH build for the GB300 traversal kernels.
//
// Replaces DevilRay's median-split generateSimpleBBH (src/models/BBH.cpp:38-115:
// one triangle per leaf, split at the median of the max-vertex key along a
// cycling axis) with a binned-SAH build and the two-box node layout that the
// device traversal reads. Unlike the reference it never reorders the caller's
// triangles: the leaf order is returned as a permutation.

#include "dr_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>

namespace dr {
namespace {

struct Box {
    float lo[3], hi[3];
    void reset()
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::numeric_limits<float>::infinity();
            hi[a] = -std::numeric_limits<float>::infinity();
        }
    }
    void grow(const Box &b)
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const float p[3])
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float area() const
    {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0 && dy >= 0 && dz >= 0)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

// A triangle's box and centroid, and its index in the soup. The builder
// partitions these records themselves (not indices to them), so every pass
// over a range reads contiguous memory.
struct Prim {
    Box box;
    float c[3];
    uint32_t id;
};

struct TreeNode {
    Box box;
    std::unique_ptr<TreeNode> child[2];
    uint32_t first = 0, count = 0;  // leaf range in the index array
    int depth = 0;
    bool leaf() const { return !child[0]; }
    // wide collapse (WideBuilder::solve): cost of the subtree in at most j
    // child slots of a wide node, and how it is reached
    float slot_cost[9] = {};
    int8_t slot_split[9] = {};  // left child's share of j slots; 0: one slot
    bool wide_leaf = false;     // its one slot is a leaf slot
    uint8_t tris = 0;           // triangles, counted up to 4
    uint32_t ntris = 0;         // triangles of the subtree
    uint32_t wide_size = 0;     // wide nodes of the subtree when it becomes a wide node
};

struct Builder {
    std::vector<Prim> &prims;  // partitioned in place; ids give the leaf order
    BuildParams params;
    std::atomic<int> spare_threads;
    std::atomic<int> max_depth{0};

    const int threads;  // host threads the build may use

    Builder(std::vector<Prim> &p, const BuildParams &bp, int threads)
        : prims(p), params(bp), spare_threads(threads - 1), threads(threads) {}

    static constexpr float kTraversalCost = 1.0f;
    static constexpr float kTriangleCost = 1.5f;
    static constexpr uint32_t kParallelBinning = 1u << 18;  // ranges binned on several threads
    static constexpr uint32_t kKnownSides = 1u << 12;        // ranges that pass their sides' bounds down

    // Bins of one axis: the primitives' boxes, their centroids' box and count.
    // A bin's entries are written by its first primitive, which also sets its
    // bit of `occupied`; empty bins are never read, so nothing is cleared per
    // range but the mask.
    struct AxisBins {
        Box box[64], cbox[64];
        uint32_t count[64];
        uint64_t occupied;
    };

    // The best SAH split of a range, with the bounds of its two sides.
    struct Split {
        float cost = std::numeric_limits<float>::infinity();
        int axis = -1;
        uint32_t bin = 0;
        bool sides = false;  // the bounds of the two sides are known
        Box left, left_c, right, right_c;
    };

    // Bins [begin, end) on every axis with a centroid extent in one pass over
    // the primitives (large ranges on several threads; boxes and counts merge
    // exactly), then evaluates the SAH at the bin boundaries. Only boundaries
    // after an occupied bin are evaluated: past an empty bin both sides, and
    // so the cost, equal those of the boundary before it, which the strict
    // comparison already preferred. (Not inlined: its 10 KB of bins stay out
    // of the recursion's frames.)
    __attribute__((noinline)) Split best_split(uint32_t begin, uint32_t end, const Box &cbounds, uint32_t B) const
    {
        bool active[3];
        float cmin[3], scale[3];
        for (int a = 0; a < 3; ++a) {
            cmin[a] = cbounds.lo[a];
            active[a] = cbounds.hi[a] > cbounds.lo[a];
            scale[a] = active[a] ? (float)B / (cbounds.hi[a] - cbounds.lo[a]) : 0.0f;
        }
        // centroid boxes per bin only for ranges whose children would
        // otherwise make another pass over many primitives
        const uint32_t n = end - begin;
        const bool sides = n >= kKnownSides;
        auto bin_into = [&](AxisBins *bins, size_t b0, size_t b1) {
            for (int a = 0; a < 3; ++a) bins[a].occupied = 0;
            for (size_t i = b0; i < b1; ++i) {
                const Prim &p = prims[i];
                for (int a = 0; a < 3; ++a) {
                    if (!active[a]) continue;
                    uint32_t b = (uint32_t)((p.c[a] - cmin[a]) * scale[a]);
                    if (b >= B) b = B - 1;
                    AxisBins &ab = bins[a];
                    if (!((ab.occupied >> b) & 1u)) {
                        ab.occupied |= 1ull << b;
                        ab.count[b] = 1;
                        ab.box[b] = p.box;
                        if (sides) {
                            for (int k = 0; k < 3; ++k) ab.cbox[b].lo[k] = ab.cbox[b].hi[k] = p.c[k];
                        }
                    } else {
                        ++ab.count[b];
                        ab.box[b].grow(p.box);
                        if (sides) ab.cbox[b].grow(p.c);
                    }
                }
            }
        };
        AxisBins bins[3];
        if (n >= kParallelBinning && threads > 1) {
            std::vector<AxisBins> parts(3 * (size_t)threads);
            std::atomic<uint32_t> next{0};
            host_parallel_chunks(
                n, kParallelBinning / 4,
                [&](size_t b0, size_t b1) { bin_into(parts.data() + 3 * next.fetch_add(1), begin + b0, begin + b1); },
                (size_t)threads);
            for (int a = 0; a < 3; ++a) bins[a].occupied = 0;
            for (uint32_t k = 0; k < next.load(); ++k)
                for (int a = 0; a < 3; ++a) {
                    const AxisBins &pb = parts[3 * k + a];
                    for (uint64_t m = pb.occupied; m != 0; m &= m - 1) {
                        const int b = __builtin_ctzll(m);
                        if (!((bins[a].occupied >> b) & 1u)) {
                            bins[a].occupied |= 1ull << b;
                            bins[a].count[b] = pb.count[b];
                            bins[a].box[b] = pb.box[b];
                            bins[a].cbox[b] = pb.cbox[b];
                        } else {
                            bins[a].count[b] += pb.count[b];
                            bins[a].box[b].grow(pb.box[b]);
                            bins[a].cbox[b].grow(pb.cbox[b]);
                        }
                    }
                }
        } else {
            bin_into(bins, begin, end);
        }
        Split best;
        for (int axis = 0; axis < 3; ++axis) {
            if (!active[axis]) continue;
            const AxisBins &ab = bins[axis];
            uint32_t occ[64], k = 0;  // occupied bins, ascending
            for (uint64_t m = ab.occupied; m != 0; m &= m - 1) occ[k++] = (uint32_t)__builtin_ctzll(m);
            // right side of the boundary after occupied bin occ[i]: bins occ[i + 1 ..]
            float right_area[64];
            uint32_t right_count[64];
            Box acc;
            acc.reset();
            uint32_t cnt = 0;
            for (uint32_t i = k; i-- > 1;) {
                acc.grow(ab.box[occ[i]]);
                cnt += ab.count[occ[i]];
                right_area[i - 1] = acc.area();
                right_count[i - 1] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (uint32_t i = 0; i + 1 < k; ++i) {
                const uint32_t b = occ[i];
                acc.grow(ab.box[b]);
                cnt += ab.count[b];
                if (b + 1 >= B) break;
                const float cost = acc.area() * cnt + right_area[i] * right_count[i];
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = axis;
                    best.bin = b + 1;
                }
            }
        }
        best.sides = sides && best.axis >= 0;
        if (best.sides) {
            const AxisBins &ab = bins[best.axis];
            best.left.reset();
            best.left_c.reset();
            best.right.reset();
            best.right_c.reset();
            for (uint64_t m = ab.occupied; m != 0; m &= m - 1) {
                const uint32_t b = (uint32_t)__builtin_ctzll(m);
                (b < best.bin ? best.left : best.right).grow(ab.box[b]);
                (b < best.bin ? best.left_c : best.right_c).grow(ab.cbox[b]);
            }
        }
        return best;
    }

    // Builds the subtree of [begin, end); `known` (if given) holds the
    // range's box and centroid box, as the parent's bins found them.
    std::unique_ptr<TreeNode> build(uint32_t begin, uint32_t end, int depth, const Box *known = nullptr)
    {
        auto node = std::make_unique<TreeNode>();
        node->depth = depth;
        int prev = max_depth.load();
        while (depth > prev && !max_depth.compare_exchange_weak(prev, depth)) {}

        Box bounds, cbounds;
        if (known) {
            bounds = known[0];
            cbounds = known[1];
        } else {
            bounds.reset();
            cbounds.reset();
            for (uint32_t i = begin; i < end; ++i) {
                const Prim &p = prims[i];
                bounds.grow(p.box);
                cbounds.grow(p.c);
            }
        }
        node->box = bounds;
        const uint32_t n = end - begin;
        if (n <= 1) {
            node->first = begin;
            node->count = n;
            return node;
        }

        // Binned SAH over the three axes.
        const uint32_t B = std::max<uint32_t>(4, std::min<uint32_t>(params.bins, 64));
        const bool force_median = depth >= 32;  // bounds the depth: <= 32 + log2(n) levels
        Split best;
        if (!force_median) best = best_split(begin, end, cbounds, B);
        const int best_axis = best.axis;
        const float parent_area = bounds.area();
        const float leaf_cost = kTriangleCost * n;
        const float split_cost = best_axis >= 0 && parent_area > 0.0f
                                     ? kTraversalCost + kTriangleCost * best.cost / parent_area
                                     : std::numeric_limits<float>::infinity();
        if (n <= params.max_leaf && (leaf_cost <= split_cost || best_axis < 0)) {
            node->first = begin;
            node->count = n;
            return node;
        }

        uint32_t mid;
        bool sides_known = false;
        if (best_axis >= 0) {
            const float cmin = cbounds.lo[best_axis], cmax = cbounds.hi[best_axis];
            const float scale = (float)B / (cmax - cmin);
            auto it = std::partition(prims.begin() + begin, prims.begin() + end, [&](const Prim &p) {
                uint32_t b = (uint32_t)((p.c[best_axis] - cmin) * scale);
                if (b >= B) b = B - 1;
                return b < best.bin;
            });
            mid = (uint32_t)(it - prims.begin());
            sides_known = best.sides && mid != begin && mid != end;
            if (mid == begin || mid == end) mid = begin + n / 2;
        } else {
            // No useful SAH split (coincident centroids, or the depth cap):
            // split at the median along the largest centroid extent.
            int axis = 0;
            float ext = -1.0f;
            for (int a = 0; a < 3; ++a)
                if (cbounds.hi[a] - cbounds.lo[a] > ext) {
                    ext = cbounds.hi[a] - cbounds.lo[a];
                    axis = a;
                }
            mid = begin + n / 2;
            std::nth_element(prims.begin() + begin, prims.begin() + mid, prims.begin() + end,
                             [&](const Prim &a, const Prim &b) {
                                 if (a.c[axis] != b.c[axis]) return a.c[axis] < b.c[axis];
                                 return a.id < b.id;
                             });
        }
        const Box lk[2] = {best.left, best.left_c}, rk[2] = {best.right, best.right_c};
        const Box *lknown = sides_known ? lk : nullptr, *rknown = sides_known ? rk : nullptr;

        if (n > 65536 && spare_threads.fetch_sub(1) > 0) {
            std::unique_ptr<TreeNode> left;
            std::thread th([&] { left = build(begin, mid, depth + 1, lknown); });
            node->child[1] = build(mid, end, depth + 1, rknown);
            th.join();
            spare_threads.fetch_add(1);
            node->child[0] = std::move(left);
        } else {
            if (n > 65536) spare_threads.fetch_add(1);
            node->child[0] = build(begin, mid, depth + 1, lknown);
            node->child[1] = build(mid, end, depth + 1, rknown);
        }
        return node;
    }
};

// Rounds a widened bound outward so the stored float box contains the exact
// widened box.
inline float lower_bound_out(float v, float slack) { return std::nextafter(v - slack, -INFINITY); }
inline float upper_bound_out(float v, float slack) { return std::nextafter(v + slack, INFINITY); }

struct Flattener {
    std::vector<Bvh2Node> &out;
    float slack;

    void set_child_box(Bvh2Node &n, int which, const Box &b)
    {
        const float lx = lower_bound_out(b.lo[0], slack), hx = upper_bound_out(b.hi[0], slack);
        const float ly = lower_bound_out(b.lo[1], slack), hy = upper_bound_out(b.hi[1], slack);
        const float lz = lower_bound_out(b.lo[2], slack), hz = upper_bound_out(b.hi[2], slack);
        if (which == 0) {
            n.c0xy = make_float4(lx, hx, ly, hy);
            n.cz.x = lz;
            n.cz.y = hz;
        } else {
            n.c1xy = make_float4(lx, hx, ly, hy);
            n.cz.z = lz;
            n.cz.w = hz;
        }
    }

    // Emits `node` (an inner node) at the next index, depth-first with the
    // left child right after its parent. Returns its index.
    int32_t emit(const TreeNode *node)
    {
        const int32_t me = (int32_t)out.size();
        out.push_back(Bvh2Node{});
        for (int c = 0; c < 2; ++c) {
            const TreeNode *ch = node->child[c].get();
            int32_t link;
            if (ch->leaf()) link = leaf_link(ch->first, ch->count);
            else link = emit(ch);
            Bvh2Node &n = out[me];
            set_child_box(n, c, ch->box);
            if (c == 0) n.link.x = link;
            else n.link.y = link;
        }
        return me;
    }
};

}  // namespace

float scene_slack(float mag)
{
    // 2^-14 of the scene magnitude: two orders above the FP32 rounding of
    // hit points, triangle-plane distances and the box-coordinate terms of the
    // slab times. The part of the slab-time error that grows with the distance
    // of the ray origin is covered by the relative margin of the box tests
    // (kBoxFarScale).
    const float m = std::max(mag, 1.0f / 1024.0f);
    return std::ldexp(m, -14);
}

namespace {

// Host threads a build may use: BuildParams::threads, 0 for all cores.
int build_threads(const BuildParams &params)
{
    return params.threads > 0 ? (int)params.threads : (int)std::max(1u, std::thread::hardware_concurrency());
}

// Boxes and centroids of the triangles.
std::vector<Prim> make_prims(const float *pos, uint32_t num_tris, int threads)
{
    std::vector<Prim> prims(num_tris);
    host_parallel_chunks(
        num_tris, size_t(1) << 16,
        [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) {
                Prim &p = prims[i];
                p.box.reset();
                for (int k = 0; k < 3; ++k) p.box.grow(pos + i * 9 + k * 3);
                for (int a = 0; a < 3; ++a) p.c[a] = 0.5f * (p.box.lo[a] + p.box.hi[a]);
                p.id = (uint32_t)i;
            }
        },
        (size_t)threads);
    return prims;
}

// The soup indices of the partitioned records: leaf position -> triangle.
std::vector<uint32_t> leaf_order(const std::vector<Prim> &prims, int threads)
{
    std::vector<uint32_t> idx(prims.size());
    host_parallel_chunks(
        prims.size(), size_t(1) << 16,
        [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) idx[i] = prims[i].id;
        },
        (size_t)threads);
    return idx;
}

// Releases a binary tree, the subtrees of the top `spawn_levels` levels on
// their own threads.
void free_tree(std::unique_ptr<TreeNode> n, int spawn_levels)
{
    if (!n || n->leaf()) return;
    if (spawn_levels > 0) {
        std::thread th([&] { free_tree(std::move(n->child[0]), spawn_levels - 1); });
        free_tree(std::move(n->child[1]), spawn_levels - 1);
        th.join();
    }
}

// The binned-SAH binary tree over the soup; idx receives the leaf order.
std::unique_ptr<TreeNode> build_tree(const float *pos, uint32_t num_tris, const BuildParams &params,
                                     std::vector<uint32_t> &idx, int &depth)
{
    const int threads = build_threads(params);
    std::vector<Prim> prims = make_prims(pos, num_tris, threads);
    Builder builder(prims, params, threads);
    std::unique_ptr<TreeNode> root = builder.build(0, num_tris, 0);
    depth = builder.max_depth.load() + 1;
    idx = leaf_order(prims, threads);
    return root;
}

struct WideBuilder {
    Bvh8 &out;
    const std::vector<uint32_t> &idx;  // binary-tree leaf order
    float slack;
    std::vector<uint32_t> &order;      // wide leaf order (sized to the triangle count)
    std::atomic<int> spare_threads;

    // Collapse of the binary tree into 8-wide nodes by dynamic programming
    // (Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
    // Through Compressed Wide BVHs", HPG 2017): for each binary subtree n and
    // j <= 8 slots, the least surface-area cost of placing n in at most j child
    // slots of one wide node, either as one slot (a leaf slot, or an internal
    // wide node that costs its area plus its own 8-slot distribution) or by
    // opening n and sharing the j slots between its two children. A wide node
    // visit costs 1 x area and a triangle kLeafTriCost x area; subtrees of up
    // to 3 triangles may become one leaf slot. Measured against opening the
    // child of largest area first (2^20 triangles, 16.8 M incoherent rays;
    // 256x256 box room, 16 spp): half the nodes (294 k -> 138 k), 2.5 % fewer
    // node visits, 4.92 -> 4.96 Grays/s, and the box room 2.47 -> 2.24 ms.
    static constexpr float kLeafTriCost = 1.0f;
    static constexpr uint32_t kMaxLeafTris = 3;

    // The subtrees that fill at most 8 child slots (a fixed array: emit runs
    // once per wide node, and per-node heap allocations dominated its time).
    struct Slots {
        const TreeNode *t[8];
        int n = 0;
    };

    // Solves the subtree of n; the subtrees of the top `spawn_levels` levels
    // run on their own threads (every node's result depends only on its
    // children's, so the split changes nothing).
    static void solve(TreeNode *n, int spawn_levels)
    {
        const float A = std::max(n->box.area(), 0.0f);
        if (n->leaf()) {
            n->tris = (uint8_t)std::min<uint32_t>(n->count, 4);
            n->ntris = n->count;
            n->wide_size = 1;
            n->wide_leaf = true;
            for (int j = 1; j <= 8; ++j) {
                n->slot_cost[j] = kLeafTriCost * (float)n->count * A;
                n->slot_split[j] = 0;
            }
            return;
        }
        TreeNode *l = n->child[0].get(), *r = n->child[1].get();
        if (spawn_levels > 0) {
            std::thread th([&] { solve(l, spawn_levels - 1); });
            solve(r, spawn_levels - 1);
            th.join();
        } else {
            solve(l, 0);
            solve(r, 0);
        }
        n->ntris = l->ntris + r->ntris;
        n->tris = (uint8_t)std::min<uint32_t>(l->tris + r->tris, 4);
        float open[9];
        int8_t open_split[9];
        for (int j = 2; j <= 8; ++j) {
            open[j] = INFINITY;
            open_split[j] = 1;
            for (int k = 1; k < j; ++k) {
                const float c = l->slot_cost[k] + r->slot_cost[j - k];
                if (c < open[j]) {
                    open[j] = c;
                    open_split[j] = (int8_t)k;
                }
            }
        }
        float one = A + open[8];  // an internal wide node
        n->wide_leaf = false;
        if (n->tris <= kMaxLeafTris && kLeafTriCost * (float)n->tris * A <= one) {
            one = kLeafTriCost * (float)n->tris * A;
            n->wide_leaf = true;
        }
        n->slot_cost[1] = one;
        n->slot_split[1] = 0;
        for (int j = 2; j <= 8; ++j) {
            const bool opened = open[j] < one;
            n->slot_cost[j] = opened ? open[j] : one;
            n->slot_split[j] = opened ? open_split[j] : (int8_t)0;
        }
        // the wide nodes n would take as a wide node: itself and the subtrees
        // of its internal slots (their children are solved already)
        Slots ch;
        collect(n, ch);
        n->wide_size = 1;
        for (int i = 0; i < ch.n; ++i)
            if (!ch.t[i]->wide_leaf) n->wide_size += ch.t[i]->wide_size;
    }

    static void expand(const TreeNode *n, int j, Slots &ch)
    {
        if (n->leaf() || n->slot_split[j] == 0) {
            ch.t[ch.n++] = n;
            return;
        }
        expand(n->child[0].get(), n->slot_split[j], ch);
        expand(n->child[1].get(), j - n->slot_split[j], ch);
    }

    // The child slots of the wide node of internal subtree n.
    static void collect(const TreeNode *n, Slots &ch)
    {
        ch.n = 0;
        const TreeNode *l = n->child[0].get(), *r = n->child[1].get();
        float best = INFINITY;
        int k_best = 1;
        for (int k = 1; k < 8; ++k) {
            const float c = l->slot_cost[k] + r->slot_cost[8 - k];
            if (c < best) {
                best = c;
                k_best = k;
            }
        }
        expand(l, k_best, ch);
        expand(r, 8 - k_best, ch);
    }

    // Triangles of subtree n in leaf order, written from order[at].
    void gather(const TreeNode *n, uint32_t &at)
    {
        if (n->leaf()) {
            for (uint32_t k = 0; k < n->count; ++k) order[at++] = idx[n->first + k];
            return;
        }
        gather(n->child[0].get(), at);
        gather(n->child[1].get(), at);
    }

    // Writes the node for binary subtree `n` at out.nodes[index]; the wide
    // nodes below it take out.nodes[node_at ...] and its triangles
    // order[tri_at ...], in the depth-first order of a serial emission: each
    // wide node's internal children are contiguous, in slot order, and a
    // child's subtree follows the subtrees of the children before it. The
    // subtree sizes come from solve, so large child subtrees are written by
    // other threads at the same places. Returns the depth of the deepest wide
    // node written.
    int emit(const TreeNode *n, uint32_t index, int depth, uint32_t node_at, uint32_t tri_at)
    {
        int max_depth = depth;
        Slots slots;
        if (n->leaf()) slots.t[slots.n++] = n;  // only the root can be a leaf
        else collect(n, slots);
        const TreeNode *const *ch = slots.t;
        const int nch = slots.n;
        // widened child boxes and their union
        Box cb[8];
        Box u;
        u.reset();
        for (int i = 0; i < nch; ++i) {
            for (int a = 0; a < 3; ++a) {
                cb[i].lo[a] = std::nextafter(ch[i]->box.lo[a] - slack, -INFINITY);
                cb[i].hi[a] = std::nextafter(ch[i]->box.hi[a] + slack, INFINITY);
            }
            u.grow(cb[i]);
        }
        // octant slots: greedy assignment of the child whose centroid lies
        // furthest towards the slot's corner (candidates by descending reach,
        // equal reaches in (child, slot) order)
        int slot_of[8], child_in[8];
        for (int s = 0; s < 8; ++s) child_in[s] = -1;
        {
            float pc[3];
            for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (u.lo[a] + u.hi[a]);
            struct Cand {
                float v;
                int c, s;
            };
            Cand cand[64];
            int nc = 0;
            for (int c = 0; c < nch; ++c)
                for (int s = 0; s < 8; ++s) {
                    float v = 0.0f;
                    for (int a = 0; a < 3; ++a) {
                        const float d = ((s >> a) & 1) ? 1.0f : -1.0f;
                        v += d * (0.5f * (cb[c].lo[a] + cb[c].hi[a]) - pc[a]);
                    }
                    cand[nc++] = Cand{v, c, s};
                }
            std::sort(cand, cand + nc, [](const Cand &x, const Cand &y) {
                return x.v > y.v || (x.v == y.v && 8 * x.c + x.s < 8 * y.c + y.s);
            });
            for (int c = 0; c < 8; ++c) slot_of[c] = -1;
            for (int k = 0; k < nc; ++k)
                if (slot_of[cand[k].c] < 0 && child_in[cand[k].s] < 0) {
                    slot_of[cand[k].c] = cand[k].s;
                    child_in[cand[k].s] = cand[k].c;
                }
        }
        // quantisation grid
        uint32_t ebias[3];
        float scale[3];
        for (int a = 0; a < 3; ++a) {
            const double ext = (double)u.hi[a] - (double)u.lo[a];
            int e = -100;
            if (ext > 0.0) e = (int)std::ceil(std::log2(ext / 255.0));
            while (std::ldexp(255.0, e) < ext) ++e;
            e = std::max(-126, std::min(127, e));
            ebias[a] = (uint32_t)(e + 127);
            scale[a] = std::ldexp(1.0f, e);
        }
        uint8_t qlo[3][8], qhi[3][8], meta[8];
        uint32_t imask = 0;
        for (int s = 0; s < 8; ++s) {
            meta[s] = 0;
            for (int a = 0; a < 3; ++a) {
                qlo[a][s] = 255;
                qhi[a][s] = 0;
            }
        }
        // internal children first (contiguous, slot order), then triangles
        const uint32_t child_base = node_at;
        std::pair<const TreeNode *, uint32_t> todo[8];
        int ntodo = 0;
        uint32_t n_internal = 0;
        for (int s = 0; s < 8; ++s) {
            const int c = child_in[s];
            if (c >= 0 && !ch[c]->wide_leaf) ++n_internal;
        }
        const uint32_t tri_base = tri_at;
        uint32_t next_child = child_base, tri_off = 0;
        for (int s = 0; s < 8; ++s) {
            const int c = child_in[s];
            if (c < 0) continue;
            for (int a = 0; a < 3; ++a) {
                const double lo = std::floor(((double)cb[c].lo[a] - (double)u.lo[a]) / scale[a]);
                const double hi = std::ceil(((double)cb[c].hi[a] - (double)u.lo[a]) / scale[a]);
                qlo[a][s] = (uint8_t)std::max(0.0, std::min(255.0, lo));
                qhi[a][s] = (uint8_t)std::max(0.0, std::min(255.0, hi));
            }
            const TreeNode *t = ch[c];
            if (!t->wide_leaf) {
                imask |= 1u << s;
                meta[s] = (uint8_t)(0x20 | (24 + s));  // hit-mask bit 24 + s
                todo[ntodo++] = {t, next_child++};
            } else if (t->tris > 0) {
                meta[s] = (uint8_t)((((1u << t->tris) - 1u) << 5) | tri_off);
                gather(t, tri_at);
                tri_off += t->tris;
            }
        }
        Bvh8Node &nd = out.nodes[index];
        nd.w[0] = make_uint4(__builtin_bit_cast(uint32_t, u.lo[0]), __builtin_bit_cast(uint32_t, u.lo[1]),
                             __builtin_bit_cast(uint32_t, u.lo[2]),
                             ebias[0] | (ebias[1] << 8) | (ebias[2] << 16) | (imask << 24));
        auto pack = [](const uint8_t *b) {
            return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
        };
        nd.w[1] = make_uint4(child_base, tri_base, pack(meta), pack(meta + 4));
        for (int a = 0; a < 3; ++a)
            nd.w[2 + a] = make_uint4(pack(qlo[a]), pack(qlo[a] + 4), pack(qhi[a]), pack(qhi[a] + 4));
        // the children's subtrees: node and triangle ranges in serial order
        uint32_t sub_node = child_base + n_internal, sub_tri = tri_at;
        std::thread helpers[8];
        int sub_depth[8] = {};
        for (int k = 0; k < ntodo; ++k) {
            const TreeNode *t = todo[k].first;
            const uint32_t at_node = sub_node, at_tri = sub_tri;
            sub_node += t->wide_size - 1;
            sub_tri += t->ntris;
            if (t->wide_size >= kSpawnWideNodes && k + 1 < ntodo && spare_threads.fetch_sub(1) > 0) {
                helpers[k] = std::thread([this, t, k, depth, at_node, at_tri, &todo, &sub_depth] {
                    sub_depth[k] = emit(t, todo[k].second, depth + 1, at_node, at_tri);
                });
            } else {
                if (t->wide_size >= kSpawnWideNodes && k + 1 < ntodo) spare_threads.fetch_add(1);
                sub_depth[k] = emit(t, todo[k].second, depth + 1, at_node, at_tri);
            }
        }
        for (int k = 0; k < ntodo; ++k) {
            if (helpers[k].joinable()) {
                helpers[k].join();
                spare_threads.fetch_add(1);
            }
            max_depth = std::max(max_depth, sub_depth[k]);
        }
        return max_depth;
    }
    static constexpr uint32_t kSpawnWideNodes = 2048;  // smallest subtree given its own thread
};

}  // namespace

Bvh8 build_bvh8(const float *pos, uint32_t num_tris, const BuildParams &params, float slack)
{
    Bvh8 bvh;
    bvh.slack = slack;
    if (num_tris == 0) return bvh;
    BuildParams bp = params;
    bp.max_leaf = std::max<uint32_t>(1, std::min<uint32_t>(bp.max_leaf, 3));
    std::vector<uint32_t> idx;
    int depth2 = 0;
    std::unique_ptr<TreeNode> root = build_tree(pos, num_tris, bp, idx, depth2);
    const int threads = build_threads(params);
    int spawn_levels = 0;
    while ((1 << spawn_levels) < threads && spawn_levels < 6) ++spawn_levels;
    WideBuilder::solve(root.get(), spawn_levels);
    bvh.order.resize(num_tris);
    bvh.nodes.resize(root->wide_size);
    WideBuilder wb{bvh, idx, slack, bvh.order, {threads - 1}};
    bvh.depth = wb.emit(root.get(), 0, 1, 1, 0);
    free_tree(std::move(root), spawn_levels);
    return bvh;
}

Bvh2 build_bvh2(const float *pos, uint32_t num_tris, const BuildParams &params, float slack)
{
    Bvh2 bvh;
    bvh.slack = slack;
    if (num_tris == 0) return bvh;
    const int threads = build_threads(params);
    std::vector<Prim> prims = make_prims(pos, num_tris, threads);
    BuildParams bp = params;
    bp.max_leaf = std::max<uint32_t>(1, std::min(bp.max_leaf, kMaxLeafSize));
    Builder builder(prims, bp, threads);
    std::unique_ptr<TreeNode> root = builder.build(0, num_tris, 0);
    std::vector<uint32_t> idx = leaf_order(prims, threads);

    Flattener fl{bvh.nodes, slack};
    bvh.nodes.reserve(2 * (size_t)num_tris / std::max<uint32_t>(1, bp.max_leaf) + 4);
    if (root->leaf()) {
        // A single leaf: the root record holds it as child 0 and an empty
        // leaf (count 0) with the same box as child 1.
        Bvh2Node n{};
        fl.set_child_box(n, 0, root->box);
        fl.set_child_box(n, 1, root->box);
        n.link = make_int4(leaf_link(root->first, root->count), leaf_link(root->first, 0), 0, 0);
        bvh.nodes.push_back(n);
        bvh.depth = 1;
    } else {
        fl.emit(root.get());
        bvh.depth = builder.max_depth.load() + 1;
    }
    int levels = 0;
    while ((1 << levels) < threads && levels < 6) ++levels;
    free_tree(std::move(root), levels);
    bvh.order = std::move(idx);
    return bvh;
}

void make_tri_records(const float *pos, const std::vector<uint32_t> &order,
                      std::vector<float4> &ref, std::vector<float4> &wt)
{
    const size_t n = order.size();
    ref.resize(n * 3);
    wt.resize(n * 3);
    host_parallel_chunks(n, size_t(1) << 16, [&](size_t k0, size_t k1) {
        for (size_t k = k0; k < k1; ++k) {
            const float *q = pos + (size_t)order[k] * 9;
            const float Ax = q[0], Ay = q[1], Az = q[2];
            const float Bx = q[3], By = q[4], Bz = q[5];
            const float Cx = q[6], Cy = q[7], Cz = q[8];
            // n_f = (A - B) x (A - C), sgn_area2 = n_f . n_f, n = n_f / |n_f|
            // (IntersectionTestsImpl.hpp:261-266; Utils.hpp:88-109), compiled with
            // -ffp-contract=off so it rounds like the reference.
            const float ux = Ax - Bx, uy = Ay - By, uz = Az - Bz;
            const float vx = Ax - Cx, vy = Ay - Cy, vz = Az - Cz;
            const float nfx = uy * vz - uz * vy;
            const float nfy = uz * vx - ux * vz;
            const float nfz = ux * vy - uy * vx;
            const float s = nfx * nfx + nfy * nfy + nfz * nfz;
            float nx = 0.0f, ny = 0.0f, nz = 0.0f;
            if (!(s < 1e-14f)) {
                const float l = std::sqrt(nfx * nfx + nfy * nfy + nfz * nfz);
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
        }
    });
}

}  // namespace dr
