// oracle_trace.cpp -- CPU restatement of DevilRay's ray/triangle test, its
// median-split BBH and its traversal (TEST INFRASTRUCTURE: the oracle the GB300
// kernels are compared against; never linked into the product).
//
// Compiled with -O2 -ffp-contract=off and no fast-math, so every FP32
// expression below rounds exactly like the reference compiled the same way.
// The expression order of every arithmetic line follows the reference line it
// cites (paths relative to the DevilRay tree).

#include "oracle.h"
#include "oracle_common.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

using namespace oracle;

namespace {

// include/tracing/IntersectionTestsImpl.hpp:253-297
bool triTestRef(const V3 &p, const V3 &v, const V3 &A, const V3 &B, const V3 &C,
                float &t_out, V3 &bari)
{
    if (anyNan(p) || anyNan(v)) return false;
    const V3 n_f = cross(sub(A, B), sub(A, C));
    const float sgn_area2 = dot(n_f, n_f);
    if (sgn_area2 < 1e-14f) return false;
    V3 n = normalized(n_f);
    float dp = dot(sub(p, A), n);
    if (dp < 0) {
        n = mul(n, -1.0f);
        dp = -dp;
    }
    const float d = -dot(v, n);
    if (d < 1e-7f) return false;
    const float t = dp / d;
    const V3 hp = add(p, mul(v, t));
    const V3 n_1 = cross(sub(hp, A), sub(C, A));
    const V3 n_2 = cross(sub(B, A), sub(hp, A));
    const float w_B = dot(n_f, n_1) / sgn_area2;
    const float w_C = dot(n_f, n_2) / sgn_area2;
    const float w_A = 1 - w_B - w_C;
    if (w_A < 0 || w_B < 0 || w_C < 0) return false;
    t_out = t;
    bari = V3{w_A, w_B, w_C};
    return true;
}

// Watertight test of Woop, Benthin and Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013, Section 3 (two-sided, no back-face culling,
// FP64 re-evaluation of zero edge functions). FP32 otherwise.
struct WtRay {
    int kx, ky, kz;
    float Sx, Sy, Sz;
    V3 o;
};

WtRay wtSetup(const V3 &o, const V3 &d)
{
    WtRay r;
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dk[3] = {d.x, d.y, d.z};
    if (dk[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = dk[kx] / dk[kz];
    r.Sy = dk[ky] / dk[kz];
    r.Sz = 1.0f / dk[kz];
    r.o = o;
    return r;
}

bool triTestWatertight(const WtRay &r, const V3 &A, const V3 &B, const V3 &C,
                       float &t_out, V3 &bari)
{
    const V3 a = sub(A, r.o), b = sub(B, r.o), c = sub(C, r.o);
    const float ak[3] = {a.x, a.y, a.z}, bk[3] = {b.x, b.y, b.z}, ck[3] = {c.x, c.y, c.z};
    const float Ax = ak[r.kx] - r.Sx * ak[r.kz];
    const float Ay = ak[r.ky] - r.Sy * ak[r.kz];
    const float Bx = bk[r.kx] - r.Sx * bk[r.kz];
    const float By = bk[r.ky] - r.Sy * bk[r.kz];
    const float Cx = ck[r.kx] - r.Sx * ck[r.kz];
    const float Cy = ck[r.ky] - r.Sy * ck[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * ak[r.kz];
    const float Bz = r.Sz * bk[r.kz];
    const float Cz = r.Sz * ck[r.kz];
    const float T = U * Az + V * Bz + W * Cz;
    // two-sided: the sign of T must match the sign of det (t >= 0)
    if (det < 0.0f ? T > 0.0f : T < 0.0f) return false;
    const float rcp = 1.0f / det;
    t_out = T * rcp;
    bari = V3{U * rcp, V * rcp, W * rcp};
    return true;
}

// ---- BBH ---------------------------------------------------------------------

struct Node {           // include/models/BBH.hpp:8-22
    float box[6];       // min xyz, max xyz
    int left = -1, right = -1, parent = -1;
    int begin = 0, end = 0;
    bool isLeaf() const { return left == -1 && right == -1; }
};

struct SortItem {
    float key;
    int32_t tri;        // original triangle index
};

}  // namespace

struct or_bbh {
    std::vector<float> pos;     // original soup, 9 floats per triangle
    std::vector<int32_t> order; // sorted position -> original triangle index
    std::vector<Node> nodes;
    int depth = 0;
};

namespace {

// AABB::extend (include/Utils.hpp:176-188): std::min / std::max semantics.
inline void extendBox(float box[6], const V3 &p)
{
    box[0] = stdMin(box[0], p.x); box[1] = stdMin(box[1], p.y); box[2] = stdMin(box[2], p.z);
    box[3] = stdMax(box[3], p.x); box[4] = stdMax(box[4], p.y); box[5] = stdMax(box[5], p.z);
}

inline V3 vert(const or_bbh &h, int tri, int k)
{
    const float *q = &h.pos[(size_t)tri * 9 + (size_t)k * 3];
    return V3{q[0], q[1], q[2]};
}

// maxExtentAlong (src/models/BBH.cpp:25-36)
inline float maxExtentAlong(const or_bbh &h, int tri, const V3 &dir)
{
    const float a = dot(vert(h, tri, 0), dir);
    const float b = dot(vert(h, tri, 1), dir);
    const float c = dot(vert(h, tri, 2), dir);
    return stdMax(a, stdMax(b, c));
}

// generateBBHLayer (src/models/BBH.cpp:38-79)
int buildLayer(or_bbh &h, std::vector<SortItem> &items, int begin, int end, int depth, int parent)
{
    if (end - begin < 1) return -1;
    Node node;
    const float fmax = std::numeric_limits<float>::max();
    node.box[0] = node.box[1] = node.box[2] = fmax;
    node.box[3] = node.box[4] = node.box[5] = -fmax;
    for (int i = begin; i < end; ++i)
        for (int k = 0; k < 3; ++k) extendBox(node.box, vert(h, items[i].tri, k));
    node.parent = parent;
    node.begin = begin;
    node.end = end;
    const int index = (int)h.nodes.size();
    h.nodes.push_back(node);

    if (end - begin > 1) {
        const V3 dir{(float)(depth % 3 == 0), (float)(depth % 3 == 1), (float)(depth % 3 == 2)};
        for (int i = begin; i < end; ++i) items[i].key = maxExtentAlong(h, items[i].tri, dir);
        // Same comparator results as the reference's lambda on the same
        // sequence, so libstdc++'s introsort performs the same permutation.
        std::sort(items.begin() + begin, items.begin() + end,
                  [](const SortItem &x, const SortItem &y) { return x.key < y.key; });
        const int mid = (begin + end) / 2;
        if (mid - begin >= 1) {
            const int l = buildLayer(h, items, begin, mid, depth + 1, index);
            h.nodes[index].left = l;
        }
        if (end - mid >= 1) {
            const int r = buildLayer(h, items, mid, end, depth + 1, index);
            h.nodes[index].right = r;
        }
    }
    return index;
}

// findBBHDepth (src/models/BBH.cpp:81-98), iterative.
int bbhDepth(const std::vector<Node> &nodes)
{
    if (nodes.empty()) return 0;
    std::vector<std::pair<int, int>> stack{{0, 1}};
    int best = 0;
    while (!stack.empty()) {
        auto [i, d] = stack.back();
        stack.pop_back();
        best = std::max(best, d);
        if (nodes[i].left != -1) stack.push_back({nodes[i].left, d + 1});
        if (nodes[i].right != -1) stack.push_back({nodes[i].right, d + 1});
    }
    return best;
}

// findBoxInterval / testBoxIntersection (IntersectionTestsImpl.hpp:80-105)
inline bool boxTestRef(const float box[6], const V3 &p, const V3 &v, float &t)
{
    const float xt0 = (box[0] - p.x) / v.x, xt1 = (box[3] - p.x) / v.x;
    const float yt0 = (box[1] - p.y) / v.y, yt1 = (box[4] - p.y) / v.y;
    const float zt0 = (box[2] - p.z) / v.z, zt1 = (box[5] - p.z) / v.z;
    const float xe = stdMin(xt0, xt1), xx = stdMax(xt0, xt1);
    const float ye = stdMin(yt0, yt1), yx = stdMax(yt0, yt1);
    const float ze = stdMin(zt0, zt1), zx = stdMax(zt0, zt1);
    const float enter = stdMax(stdMax(xe, ye), ze);
    const float exit = stdMin(stdMin(xx, yx), zx);
    if (exit < 0 || enter > exit) return false;
    t = stdMax(enter, 0.0f);
    return true;
}

// Conservative slab test for the canonical traversal: the box is widened by
// `slack` on every side and NaN slab times (0/0) are treated as unbounded.
inline bool boxTestConservative(const float box[6], const V3 &p, const V3 &v, float slack,
                                float tmax, float &t)
{
    float enter = 0.0f, exit = tmax;
    const float pk[3] = {p.x, p.y, p.z}, vk[3] = {v.x, v.y, v.z};
    for (int a = 0; a < 3; ++a) {
        const float lo = box[a] - slack, hi = box[a + 3] + slack;
        if (vk[a] == 0.0f) {
            if (pk[a] < lo || pk[a] > hi) return false;
            continue;
        }
        float t0 = (lo - pk[a]) / vk[a], t1 = (hi - pk[a]) / vk[a];
        if (t0 > t1) std::swap(t0, t1);
        // widen by a relative 2^-20 to absorb the division rounding
        t0 = t0 - std::fabs(t0) * 0x1p-20f;
        t1 = t1 + std::fabs(t1) * 0x1p-20f;
        enter = std::max(enter, t0);
        exit = std::min(exit, t1);
    }
    if (enter > exit) return false;
    t = enter;
    return true;
}

template <typename F>
void parallelFor(int64_t n, int threads, F &&f)
{
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (n < 1024 || threads == 1) {
        f(0, n);
        return;
    }
    const int64_t chunk = (n + threads - 1) / threads;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto &th : pool) th.join();
}

// One triangle test in the selected mode, on the original soup.
struct TriTester {
    int mode;
    V3 p, v;
    WtRay wt;
    TriTester(int mode_, const V3 &p_, const V3 &v_) : mode(mode_), p(p_), v(v_)
    {
        if (mode == 1) wt = wtSetup(p, v);
    }
    bool test(const V3 &A, const V3 &B, const V3 &C, float &t, V3 &bari) const
    {
        return mode == 1 ? triTestWatertight(wt, A, B, C, t, bari) : triTestRef(p, v, A, B, C, t, bari);
    }
};

// Rays with a non-finite component or a zero direction never hit (the
// reference rejects NaN rays at IntersectionTestsImpl.hpp:255 and zero
// directions at :278; infinite components are outside its domain).
inline bool validRay(const V3 &p, const V3 &v)
{
    return std::isfinite(p.x) && std::isfinite(p.y) && std::isfinite(p.z) &&
           std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z) &&
           !(v.x == 0.0f && v.y == 0.0f && v.z == 0.0f);
}

}  // namespace

extern "C" {

int or_tri_test_ref(const float ray[6], const float tri[9], float out[4])
{
    float t;
    V3 bari;
    if (!triTestRef(V3{ray[0], ray[1], ray[2]}, V3{ray[3], ray[4], ray[5]},
                    V3{tri[0], tri[1], tri[2]}, V3{tri[3], tri[4], tri[5]}, V3{tri[6], tri[7], tri[8]},
                    t, bari))
        return 0;
    out[0] = t; out[1] = bari.x; out[2] = bari.y; out[3] = bari.z;
    return 1;
}

int or_tri_test_watertight(const float ray[6], const float tri[9], float out[4])
{
    const V3 p{ray[0], ray[1], ray[2]}, v{ray[3], ray[4], ray[5]};
    if (!validRay(p, v)) return 0;
    const WtRay r = wtSetup(p, v);
    float t;
    V3 bari;
    if (!triTestWatertight(r, V3{tri[0], tri[1], tri[2]}, V3{tri[3], tri[4], tri[5]},
                           V3{tri[6], tri[7], tri[8]}, t, bari))
        return 0;
    out[0] = t; out[1] = bari.x; out[2] = bari.y; out[3] = bari.z;
    return 1;
}

int or_box_test_ref(const float box[6], const float ray[6], float *t_out)
{
    float t;
    if (!boxTestRef(box, V3{ray[0], ray[1], ray[2]}, V3{ray[3], ray[4], ray[5]}, t)) return 0;
    *t_out = t;
    return 1;
}

or_bbh *or_bbh_create(const float *positions, int32_t num_triangles)
{
    auto *h = new or_bbh;
    h->pos.assign(positions, positions + (size_t)num_triangles * 9);
    std::vector<SortItem> items((size_t)num_triangles);
    for (int32_t i = 0; i < num_triangles; ++i) items[i] = SortItem{0.0f, i};
    h->nodes.reserve((size_t)std::max(1, 2 * num_triangles));
    // generateSimpleBBH (src/models/BBH.cpp:101-115)
    buildLayer(*h, items, 0, num_triangles, 0, -1);
    h->order.resize((size_t)num_triangles);
    for (int32_t i = 0; i < num_triangles; ++i) h->order[i] = items[i].tri;
    h->depth = bbhDepth(h->nodes);
    return h;
}

void or_bbh_destroy(or_bbh *h) { delete h; }
int32_t or_bbh_num_nodes(const or_bbh *h) { return (int32_t)h->nodes.size(); }
int32_t or_bbh_depth(const or_bbh *h) { return h->depth; }

void or_bbh_export(const or_bbh *h, float *boxes, int32_t *links, int32_t *order)
{
    for (size_t i = 0; i < h->nodes.size(); ++i) {
        const Node &n = h->nodes[i];
        if (boxes) std::memcpy(boxes + i * 6, n.box, sizeof(n.box));
        if (links) {
            links[i * 5 + 0] = n.left; links[i * 5 + 1] = n.right; links[i * 5 + 2] = n.parent;
            links[i * 5 + 3] = n.begin; links[i * 5 + 4] = n.end;
        }
    }
    if (order) std::memcpy(order, h->order.data(), h->order.size() * sizeof(int32_t));
}

// getIntersectionImpl (IntersectionTestsImpl.hpp:141-220) with
// getIntersectionTris (:14-72): stackless descent with a parent index and a
// 32-bit trail of visited far children; near child chosen by the sign of the
// ray direction on axis depth % 3 (:107-139).
void or_bbh_trace_reference(const or_bbh *h, const float *rays, int64_t num_rays,
                            float *t_out, int32_t *prim_out,
                            int64_t *box_tests, int64_t *tri_tests,
                            int32_t tri_mode, int32_t threads)
{
    parallelFor(num_rays, threads, [&](int64_t b, int64_t e) {
        for (int64_t r = b; r < e; ++r) {
            const float *q = rays + r * 6;
            const V3 p{q[0], q[1], q[2]}, v{q[3], q[4], q[5]};
            const TriTester tester(tri_mode, p, v);
            bool have = false;
            float best_t = 0.0f;
            int32_t best_prim = -1;
            int64_t nbox = 0, ntri = 0;
            const int nn = (int)h->nodes.size();
            uint32_t trail = 0, depth = 0;
            int cur = nn > 0 ? 0 : -1;
            while (cur >= 0 && cur < nn) {
                const Node &node = h->nodes[cur];
                ++nbox;
                float tb;
                if (boxTestRef(node.box, p, v, tb)) {
                    if (!have || tb < best_t) {
                        if (node.isLeaf()) {
                            for (int i = node.begin; i < node.end; ++i) {
                                const int tri = h->order[i];
                                ++ntri;
                                float t;
                                V3 bari;
                                if (!tester.test(vert(*h, tri, 0), vert(*h, tri, 1), vert(*h, tri, 2), t, bari))
                                    continue;
                                if (!have || best_t > t) {
                                    have = true;
                                    best_t = t;
                                    best_prim = tri;
                                }
                            }
                        } else {
                            const uint32_t axis = depth % 3;
                            const float vk = axis == 0 ? v.x : (axis == 1 ? v.y : v.z);
                            const int near_child = vk > 0.0f ? cur + 1 : node.right;
                            trail &= ~(1u << depth);
                            cur = near_child;
                            ++depth;
                            continue;
                        }
                    }
                }
                while (true) {
                    if (cur == 0) {
                        cur = -1;
                        break;
                    }
                    const int parent_index = h->nodes[cur].parent;
                    const Node &parent = h->nodes[parent_index];
                    --depth;
                    if (!(trail & (1u << depth))) {
                        const uint32_t axis = depth % 3;
                        const float vk = axis == 0 ? v.x : (axis == 1 ? v.y : v.z);
                        const int far_child = vk > 0.0f ? parent.right : parent_index + 1;
                        trail |= (1u << depth);
                        cur = far_child;
                        ++depth;
                        break;
                    }
                    cur = parent_index;
                }
            }
            t_out[r] = have ? best_t : std::numeric_limits<float>::infinity();
            prim_out[r] = have ? best_prim : -1;
            if (box_tests) box_tests[r] = nbox;
            if (tri_tests) tri_tests[r] = ntri;
        }
    });
}

void or_bbh_trace_canonical(const or_bbh *h, const float *rays8, int64_t num_rays,
                            float slack, float *t_out, int32_t *prim_out,
                            int32_t tri_mode, int32_t threads)
{
    parallelFor(num_rays, threads, [&](int64_t b, int64_t e) {
        std::vector<int> stack;
        stack.reserve(128);
        for (int64_t r = b; r < e; ++r) {
            const float *q = rays8 + r * 8;
            const V3 p{q[0], q[1], q[2]}, v{q[4], q[5], q[6]};
            const float tmax = q[3];
            float best_t = std::numeric_limits<float>::infinity();
            int32_t best_prim = -1;
            if (validRay(p, v) && !h->nodes.empty()) {
                const TriTester tester(tri_mode, p, v);
                stack.clear();
                stack.push_back(0);
                while (!stack.empty()) {
                    const Node &node = h->nodes[stack.back()];
                    stack.pop_back();
                    float tb;
                    const float bound = std::min(best_t, tmax);
                    if (!boxTestConservative(node.box, p, v, slack, bound, tb)) continue;
                    if (tb > bound) continue;
                    if (node.isLeaf()) {
                        for (int i = node.begin; i < node.end; ++i) {
                            const int tri = h->order[i];
                            float t;
                            V3 bari;
                            if (!tester.test(vert(*h, tri, 0), vert(*h, tri, 1), vert(*h, tri, 2), t, bari))
                                continue;
                            if (!(t <= tmax)) continue;
                            if (t < best_t || (t == best_t && tri < best_prim)) {
                                best_t = t;
                                best_prim = tri;
                            }
                        }
                    } else {
                        if (node.right != -1) stack.push_back(node.right);
                        if (node.left != -1) stack.push_back(node.left);
                    }
                }
            }
            t_out[r] = best_t;
            prim_out[r] = best_prim;
        }
    });
}

void or_bbh_trace_any(const or_bbh *h, const float *rays8, int64_t num_rays,
                      float slack, uint8_t *occluded, int32_t tri_mode, int32_t threads)
{
    parallelFor(num_rays, threads, [&](int64_t b, int64_t e) {
        std::vector<int> stack;
        stack.reserve(128);
        for (int64_t r = b; r < e; ++r) {
            const float *q = rays8 + r * 8;
            const V3 p{q[0], q[1], q[2]}, v{q[4], q[5], q[6]};
            const float tmax = q[3];
            uint8_t hit = 0;
            if (validRay(p, v) && !h->nodes.empty()) {
                const TriTester tester(tri_mode, p, v);
                stack.clear();
                stack.push_back(0);
                while (!stack.empty() && !hit) {
                    const Node &node = h->nodes[stack.back()];
                    stack.pop_back();
                    float tb;
                    if (!boxTestConservative(node.box, p, v, slack, tmax, tb)) continue;
                    if (node.isLeaf()) {
                        for (int i = node.begin; i < node.end && !hit; ++i) {
                            const int tri = h->order[i];
                            float t;
                            V3 bari;
                            if (tester.test(vert(*h, tri, 0), vert(*h, tri, 1), vert(*h, tri, 2), t, bari) &&
                                t <= tmax)
                                hit = 1;
                        }
                    } else {
                        if (node.right != -1) stack.push_back(node.right);
                        if (node.left != -1) stack.push_back(node.left);
                    }
                }
            }
            occluded[r] = hit;
        }
    });
}

void or_trace_brute(const float *positions, int32_t num_triangles,
                    const float *rays8, int64_t num_rays,
                    float *t_out, int32_t *prim_out, int32_t tri_mode, int32_t threads)
{
    parallelFor(num_rays, threads, [&](int64_t b, int64_t e) {
        for (int64_t r = b; r < e; ++r) {
            const float *q = rays8 + r * 8;
            const V3 p{q[0], q[1], q[2]}, v{q[4], q[5], q[6]};
            const float tmax = q[3];
            float best_t = std::numeric_limits<float>::infinity();
            int32_t best_prim = -1;
            if (validRay(p, v)) {
                const TriTester tester(tri_mode, p, v);
                for (int32_t i = 0; i < num_triangles; ++i) {
                    const float *s = positions + (size_t)i * 9;
                    float t;
                    V3 bari;
                    if (!tester.test(V3{s[0], s[1], s[2]}, V3{s[3], s[4], s[5]}, V3{s[6], s[7], s[8]}, t, bari))
                        continue;
                    if (!(t <= tmax)) continue;
                    if (t < best_t) {  // strict: the first (smallest index) wins ties
                        best_t = t;
                        best_prim = i;
                    }
                }
            }
            t_out[r] = best_t;
            prim_out[r] = best_prim;
        }
    });
}

}  // extern "C"
