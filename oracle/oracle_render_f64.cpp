// oracle_render_f64.cpp -- FP64 restatement of DevilRay's integrator for
// converged reference images (TEST INFRASTRUCTURE: never linked into the
// product).
//
// The same estimator as sampleColor (include/tracing/PathGeneration.hpp:363-515)
// and as the FP32 oracle (oracle_render.cpp), with every quantity in double:
//   * camera ray: cameraRay (include/tracing/CameraRay.hpp:6-34);
//   * closest hit: the reference triangle test (IntersectionTestsImpl.hpp:253-297)
//     evaluated in double over a two-level double-precision BVH of its own
//     (a tree over the objects, a tree over each object's triangles; centroid
//     splits by a binned surface-area heuristic, ordered stack traversal),
//     smallest t, ties to the smaller triangle index;
//   * diffuse bounce: cosineWeightedHemisphereSample (DistributionSamplers.hpp:33-42)
//     with std::sin/std::cos/std::acos in double; dielectric bounce: the IOR
//     stack, total internal reflection, Schlick and Snell of generateNewRay
//     (PathGeneration.hpp:114-211); ray offsets of 1e-5 along the normal;
//   * next-event estimation: an object picked with probability proportional
//     to its emitted power and a triangle of it proportional to area
//     (samplePointOnLights, PathGeneration.hpp:234-272, Renderer.cpp:113-152),
//     drawn from double cumulative sums instead of alias tables so every pdf
//     is exact in double; uniform point on the triangle
//     (uniformTriangleSample, DistributionSamplers.hpp:92-104);
//   * MIS with the power heuristic (PathGeneration.hpp:301-361) and the
//     visibility rule of visible() (:213-224).
// Uniforms come from Philox4x32-10 (53-bit doubles, a stream tag of their own),
// so its samples are independent of the FP32 renderers' at any seed.

#include "oracle.h"
#include "oracle_ptmath.hpp"
#include "oracle_scene.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr double kPiD = 3.14159265358979323846;
constexpr uint32_t kStreamTagF64 = 0x46363421u;

struct D3 {
    double x, y, z;
};
inline D3 operator+(const D3 &a, const D3 &b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(const D3 &a, const D3 &b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(const D3 &a, double f) { return D3{a.x * f, a.y * f, a.z * f}; }
inline D3 operator*(const D3 &a, const D3 &b) { return D3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline double dot(const D3 &a, const D3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(const D3 &a, const D3 &v) { return D3{a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x}; }
inline double length(const D3 &a) { return std::sqrt(dot(a, a)); }
inline D3 normalized(const D3 &a) { return a * (1.0 / length(a)); }
inline double luminance(const D3 &c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }
inline double powerHeuristic(double a, double b) { return a * a / (a * a + b * b); }
inline double get(const D3 &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

double uniform(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim)
{
    uint32_t out[4];
    oracle::ptm::philox(pixel, sample, dim >> 1, kStreamTagF64, (uint32_t)seed, (uint32_t)(seed >> 32), out);
    const uint32_t hi = out[2 * (dim & 1)], lo = out[2 * (dim & 1) + 1];
    const uint64_t bits = (((uint64_t)hi << 32) | lo) >> 11;
    return (double)bits * (1.0 / 9007199254740992.0);  // [0, 1), 53 bits
}

struct Tri {
    D3 a, b, c;
};

// testTriangleIntersection in double; returns t or -1.
double tri_test(const D3 &p, const D3 &v, const Tri &T)
{
    const D3 n_f = cross(T.a - T.b, T.a - T.c);
    const double s2 = dot(n_f, n_f);
    if (s2 < 1e-14) return -1;
    D3 n = normalized(n_f);
    double dp = dot(p - T.a, n);
    if (dp < 0) {
        n = n * -1.0;
        dp = -dp;
    }
    const double d = -dot(v, n);
    if (d < 1e-7) return -1;
    const double t = dp / d;
    const D3 hp = p + v * t;
    const D3 n1 = cross(hp - T.a, T.c - T.a);
    const D3 n2 = cross(T.b - T.a, hp - T.a);
    const double wB = dot(n_f, n1) / s2, wC = dot(n_f, n2) / s2, wA = 1 - wB - wC;
    if (wA < 0 || wB < 0 || wC < 0) return -1;
    return t;
}

// A bounding-volume tree over items with boxes: centroid splits by a binned
// surface-area heuristic, `leaf` items per leaf at most.
struct Node {
    double lo[3], hi[3];
    int32_t left, right;   // children, or -1 for a leaf
    int32_t begin, count;  // leaf range of `order`
};

struct Box {
    double lo[3], hi[3];
};

struct Tree {
    std::vector<Node> nodes;
    std::vector<int32_t> order;
    const std::vector<Box> *boxes = nullptr;
    int leaf = 2;

    int build(int b, int e, const std::vector<D3> &cen)
    {
        constexpr double kInf = std::numeric_limits<double>::infinity();
        Node nd;
        for (int k = 0; k < 3; ++k) {
            nd.lo[k] = kInf;
            nd.hi[k] = -kInf;
        }
        for (int i = b; i < e; ++i)
            for (int k = 0; k < 3; ++k) {
                nd.lo[k] = std::min(nd.lo[k], (*boxes)[order[i]].lo[k]);
                nd.hi[k] = std::max(nd.hi[k], (*boxes)[order[i]].hi[k]);
            }
        const int id = (int)nodes.size();
        nodes.push_back(nd);
        if (e - b <= leaf) {
            nodes[id].left = nodes[id].right = -1;
            nodes[id].begin = b;
            nodes[id].count = e - b;
            return id;
        }
        double clo[3], chi[3];
        for (int k = 0; k < 3; ++k) {
            clo[k] = kInf;
            chi[k] = -kInf;
        }
        for (int i = b; i < e; ++i)
            for (int k = 0; k < 3; ++k) {
                clo[k] = std::min(clo[k], get(cen[order[i]], k));
                chi[k] = std::max(chi[k], get(cen[order[i]], k));
            }
        constexpr int kBins = 16;
        auto area = [](const double *lo, const double *hi) {
            const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
            return dx * dy + dy * dz + dz * dx;
        };
        auto bin_of = [&](int32_t x, int k) {
            return std::min(kBins - 1, (int)((get(cen[x], k) - clo[k]) * (kBins / (chi[k] - clo[k]))));
        };
        double best_cost = kInf;
        int best_axis = -1, best_split = 0;
        for (int k = 0; k < 3; ++k) {
            if (!(chi[k] > clo[k])) continue;
            Box bins[kBins];
            int bcnt[kBins] = {};
            for (int q = 0; q < kBins; ++q)
                for (int c = 0; c < 3; ++c) {
                    bins[q].lo[c] = kInf;
                    bins[q].hi[c] = -kInf;
                }
            for (int i = b; i < e; ++i) {
                const int q = bin_of(order[i], k);
                ++bcnt[q];
                for (int c = 0; c < 3; ++c) {
                    bins[q].lo[c] = std::min(bins[q].lo[c], (*boxes)[order[i]].lo[c]);
                    bins[q].hi[c] = std::max(bins[q].hi[c], (*boxes)[order[i]].hi[c]);
                }
            }
            double rarea[kBins];
            int rcnt[kBins];
            Box acc;
            for (int c = 0; c < 3; ++c) {
                acc.lo[c] = kInf;
                acc.hi[c] = -kInf;
            }
            int cnt = 0;
            for (int q = kBins - 1; q > 0; --q) {
                for (int c = 0; c < 3; ++c) {
                    acc.lo[c] = std::min(acc.lo[c], bins[q].lo[c]);
                    acc.hi[c] = std::max(acc.hi[c], bins[q].hi[c]);
                }
                cnt += bcnt[q];
                rarea[q] = cnt ? area(acc.lo, acc.hi) : 0.0;
                rcnt[q] = cnt;
            }
            for (int c = 0; c < 3; ++c) {
                acc.lo[c] = kInf;
                acc.hi[c] = -kInf;
            }
            cnt = 0;
            for (int q = 0; q < kBins - 1; ++q) {
                for (int c = 0; c < 3; ++c) {
                    acc.lo[c] = std::min(acc.lo[c], bins[q].lo[c]);
                    acc.hi[c] = std::max(acc.hi[c], bins[q].hi[c]);
                }
                cnt += bcnt[q];
                if (cnt == 0 || rcnt[q + 1] == 0) continue;
                const double cost = cnt * area(acc.lo, acc.hi) + rcnt[q + 1] * rarea[q + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = k;
                    best_split = q + 1;
                }
            }
        }
        int mid = (b + e) / 2;  // coincident centroids: split the range
        if (best_axis >= 0)
            mid = (int)(std::partition(order.begin() + b, order.begin() + e,
                                       [&](int32_t x) { return bin_of(x, best_axis) < best_split; }) -
                        order.begin());
        if (mid <= b || mid >= e) mid = (b + e) / 2;
        const int l = build(b, mid, cen);
        const int r = build(mid, e, cen);
        nodes[id].left = l;
        nodes[id].right = r;
        nodes[id].begin = nodes[id].count = 0;
        return id;
    }

    void init(const std::vector<Box> &bx, int leaf_items)
    {
        boxes = &bx;
        leaf = leaf_items;
        order.resize(bx.size());
        for (size_t i = 0; i < bx.size(); ++i) order[i] = (int32_t)i;
        std::vector<D3> cen(bx.size());
        for (size_t i = 0; i < bx.size(); ++i)
            cen[i] = D3{bx[i].lo[0] + bx[i].hi[0], bx[i].lo[1] + bx[i].hi[1], bx[i].lo[2] + bx[i].hi[2]} * 0.5;
        if (!bx.empty()) build(0, (int)bx.size(), cen);
    }

    // slab test with a small relative widening (every box that the exact ray
    // meets is entered); returns the entry distance or +inf
    static double box(const Node &nd, const D3 &p, const D3 &inv)
    {
        double t0 = 0.0, t1 = std::numeric_limits<double>::infinity();
        for (int k = 0; k < 3; ++k) {
            const double pk = get(p, k), ik = get(inv, k);
            const double w = 1e-9 * (std::fabs(nd.lo[k]) + std::fabs(nd.hi[k]) + 1.0);
            double a = (nd.lo[k] - w - pk) * ik, b = (nd.hi[k] + w - pk) * ik;
            if (std::isnan(a)) a = -std::numeric_limits<double>::infinity();
            if (std::isnan(b)) b = std::numeric_limits<double>::infinity();
            if (a > b) std::swap(a, b);
            t0 = std::max(t0, a);
            t1 = std::min(t1, b);
        }
        return t0 <= t1 * (1.0 + 1e-12) ? t0 : std::numeric_limits<double>::infinity();
    }

    // ordered traversal: calls leaf_fn(item) for the items of every leaf whose
    // box starts before the current bound `best` (which leaf_fn may lower)
    template <typename F>
    void traverse(const D3 &p, const D3 &inv, const double &best, F &&leaf_fn) const
    {
        if (nodes.empty()) return;
        int stack[128];
        double entry[128];
        int sp = 0;
        const double t_root = box(nodes[0], p, inv);
        if (t_root == std::numeric_limits<double>::infinity()) return;
        stack[sp] = 0;
        entry[sp++] = t_root;
        while (sp > 0) {
            --sp;
            if (entry[sp] > best) continue;
            const Node &nd = nodes[stack[sp]];
            if (nd.left < 0) {
                for (int i = nd.begin; i < nd.begin + nd.count; ++i) leaf_fn(order[i]);
                continue;
            }
            const double tl = box(nodes[nd.left], p, inv), tr = box(nodes[nd.right], p, inv);
            const int first = tl <= tr ? nd.left : nd.right, second = tl <= tr ? nd.right : nd.left;
            const double tf = std::min(tl, tr), ts = std::max(tl, tr);
            if (ts <= best) {
                stack[sp] = second;
                entry[sp++] = ts;
            }
            if (tf <= best) {
                stack[sp] = first;
                entry[sp++] = tf;
            }
        }
    }
};

Box tri_box(const Tri &t)
{
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min({get(t.a, k), get(t.b, k), get(t.c, k)});
        b.hi[k] = std::max({get(t.a, k), get(t.b, k), get(t.c, k)});
    }
    return b;
}

// Two levels: a tree over the objects (one object per leaf) and a tree over
// each object's triangles, so the large triangles of one object (a wall) do
// not widen the boxes of another's (a sphere).
struct Scene64 {
    const std::vector<Tri> *tris;
    std::vector<Box> obj_boxes;
    std::vector<std::vector<Box>> tri_boxes;
    std::vector<uint32_t> obj_begin;
    Tree top;
    std::vector<Tree> bottom;

    void init(const std::vector<Tri> &t, const std::vector<or_object> &objects)
    {
        tris = &t;
        const size_t N = objects.size();
        tri_boxes.resize(N);
        obj_begin.resize(N);
        bottom.resize(N);
        std::vector<int32_t> keep;
        for (size_t o = 0; o < N; ++o) {
            obj_begin[o] = objects[o].tri_begin;
            for (uint32_t k = 0; k < objects[o].tri_count; ++k) tri_boxes[o].push_back(tri_box(t[objects[o].tri_begin + k]));
            bottom[o].init(tri_boxes[o], 2);
            Box b;
            for (int k = 0; k < 3; ++k) {
                b.lo[k] = std::numeric_limits<double>::infinity();
                b.hi[k] = -b.lo[k];
            }
            if (!bottom[o].nodes.empty())
                for (int k = 0; k < 3; ++k) {
                    b.lo[k] = bottom[o].nodes[0].lo[k];
                    b.hi[k] = bottom[o].nodes[0].hi[k];
                }
            obj_boxes.push_back(b);
        }
        top.init(obj_boxes, 1);
    }

    // closest hit: (t, triangle index), index -1 on a miss
    std::pair<double, int> closest(const D3 &p, const D3 &v) const
    {
        double best = std::numeric_limits<double>::infinity();
        int prim = -1;
        const D3 inv{1.0 / v.x, 1.0 / v.y, 1.0 / v.z};
        top.traverse(p, inv, best, [&](int32_t o) {
            if (bottom[o].nodes.empty()) return;
            bottom[o].traverse(p, inv, best, [&](int32_t local) {
                const int k = (int)obj_begin[o] + local;
                const double t = tri_test(p, v, (*tris)[k]);
                if (t >= 0 && (t < best || (t == best && k < prim))) {
                    best = t;
                    prim = k;
                }
            });
        });
        return {best, prim};
    }
};

struct Vtx {
    D3 p, n;
    int mat;
    D3 thr;
};

}  // namespace

extern "C" void or_render_f64(const or_scene *s, const or_camera *cam, const or_render_cfg *cfg, double *sum_rgb)
{
    const int W = cam->width, H = cam->height;
    const int64_t npix = (int64_t)W * H;
    const size_t ntri = s->pos.size() / 9;
    std::vector<Tri> tris(ntri);
    for (size_t i = 0; i < ntri; ++i) {
        const float *q = &s->pos[i * 9];
        tris[i] = Tri{D3{q[0], q[1], q[2]}, D3{q[3], q[4], q[5]}, D3{q[6], q[7], q[8]}};
    }
    Scene64 bvh;
    bvh.init(tris, s->objects);
    auto emission = [&](int m) { const auto &e = s->mats[m].emission; return D3{e.x, e.y, e.z}; };
    auto albedo = [&](int m) { const auto &a = s->mats[m].albedo; return D3{a.x, a.y, a.z}; };
    // emitted-power weights (area x luminance(pi E), calculateLightWeights) and
    // per-object area cumulative sums, in double
    const size_t N = s->objects.size();
    std::vector<double> obj_area(N, 0.0), obj_w(N, 0.0), obj_cdf(N, 0.0), lum(s->mats.size(), 0.0);
    std::vector<double> tri_cdf(ntri, 0.0);
    for (size_t m = 0; m < s->mats.size(); ++m)
        lum[m] = s->mats[m].kind == 0 ? luminance(emission((int)m) * kPiD) : 0.0;
    double total = 0.0;
    for (size_t o = 0; o < N; ++o) {
        const or_object &ob = s->objects[o];
        double a = 0.0;
        for (uint32_t k = 0; k < ob.tri_count; ++k) {
            const Tri &t = tris[ob.tri_begin + k];
            a += 0.5 * length(cross(t.a - t.b, t.a - t.c));
            tri_cdf[ob.tri_begin + k] = a;
        }
        obj_area[o] = a;
        obj_w[o] = ob.tri_count ? a * lum[ob.material] : 0.0;
        total += obj_w[o];
        obj_cdf[o] = total;
    }
    const bool lights = total > 0.0;

    const int64_t nwork = cfg->pixels ? cfg->num_pixels : npix;
    auto work = [&](int64_t wb, int64_t we) {
        for (int64_t wi = wb; wi < we; ++wi) {
            const int64_t pix = cfg->pixels ? cfg->pixels[wi] : wi;
            if (pix < 0 || pix >= npix) continue;
            const int px = (int)(pix % W), py = (int)(pix / W);
            D3 acc{0, 0, 0};
            for (int si = 0; si < cfg->spp; ++si) {
                const uint32_t sample = (uint32_t)(cfg->sample_offset + si);
                auto rnd = [&](uint32_t dim) { return uniform(cfg->seed, (uint32_t)pix, sample, dim); };
                double subx = 0.5, suby = 0.5;
                if (cfg->pixel_sampling == 1) {
                    subx = rnd(oracle::ptm::dim_camera(0));
                    suby = rnd(oracle::ptm::dim_camera(1));
                }
                const double physx = (px + subx) * cam->psx - cam->cx, physy = (py + suby) * cam->psy - cam->cy;
                const D3 cv = normalized(D3{physx / cam->focal, physy / cam->focal, 1.0});
                const float *m = cam->m;
                D3 rp{m[3], m[7], m[11]};
                D3 rv{m[0] * cv.x + m[1] * cv.y + m[2] * cv.z, m[4] * cv.x + m[5] * cv.y + m[6] * cv.z,
                      m[8] * cv.x + m[9] * cv.y + m[10] * cv.z};
                // path construction
                D3 thr{1, 1, 1};
                int stack[3];
                int ssize = 0;
                Vtx path_buf[64];
                size_t path_len = 0;
                for (int depth = 0; depth < std::min(cfg->max_depth, 64); ++depth) {
                    const auto hit = bvh.closest(rp, rv);
                    if (hit.second < 0) break;
                    const Tri &T = tris[hit.second];
                    D3 n = normalized(cross(T.a - T.b, T.a - T.c));
                    if (dot(n, rv) > 0) n = n * -1.0;
                    const D3 hp = rp + rv * hit.first;
                    const int mat_id = s->tri_material[hit.second];
                    const int obj = s->tri_object[hit.second];
                    path_buf[path_len++] = Vtx{hp, n, mat_id, thr};
                    const oracle::Mat &mat = s->mats[mat_id];
                    D3 normal = n;
                    const uint32_t db = oracle::ptm::dim_bounce(depth, 0);
                    if (mat.kind == 0) {
                        const double theta0 = 2 * kPiD * rnd(db), theta1 = std::acos(1 - 2 * rnd(db + 1));
                        const D3 sph{std::sin(theta1) * std::sin(theta0), std::sin(theta1) * std::cos(theta0),
                                     std::cos(theta1)};
                        rv = normalized(sph + normal);
                        thr = thr * albedo(mat_id);
                        rp = hp;
                    } else {
                        double n1, n2;
                        auto ior_of_object = [&](int o) {
                            const oracle::Mat &tm = s->mats[s->objects[o].material];
                            return tm.kind == 1 ? (double)tm.ior : 1.0;
                        };
                        if (ssize > 0 && stack[ssize - 1] == obj) {
                            n1 = mat.ior;
                            --ssize;
                            if (ssize == 0) n2 = 1;
                            else n2 = ior_of_object(stack[--ssize]);  // Stack::top() pops (:64-67)
                            if (ssize < 3) stack[ssize++] = obj;
                        } else {
                            n2 = mat.ior;
                            if (ssize == 0) n1 = 1;
                            else n1 = ior_of_object(stack[--ssize]);
                        }
                        const double eta = n1 / n2;
                        const double d = dot(rv, normal);
                        const double k = 1 - eta * eta * (1 - d * d);
                        D3 vv;
                        if (n1 > n2 && k < 0) {
                            vv = rv - normal * (2.0 * d);
                        } else {
                            const double r = (n1 - n2) / (n1 + n2);
                            const double R0 = r * r;
                            const double c = 1 - (-d);
                            const double F = R0 + (1 - R0) * c * c * c * c * c;
                            if (rnd(db + 2) < F) {
                                vv = rv - normal * (2.0 * d);
                            } else {
                                if (ssize > 0 && stack[ssize - 1] == obj) --ssize;
                                else if (ssize < 3) stack[ssize++] = obj;
                                normal = normal * -1.0;
                                vv = normal * (std::sqrt(k) - (-d) * eta) + rv * eta;
                            }
                        }
                        rv = vv;
                        rp = hp;
                    }
                    rp = rp + normal * 1e-5;
                }
                // shading
                D3 color{0, 0, 0};
                bool prev_spec = true;
                double pdf_bsdf = 0, pdf_nee = 0;
                for (size_t vi = 0; vi < path_len; ++vi) {
                    const Vtx &v = path_buf[vi];
                    const oracle::Mat &mat = s->mats[v.mat];
                    if (mat.kind != 0) {
                        prev_spec = true;
                        continue;
                    }
                    const D3 E = emission(v.mat);
                    if (prev_spec) color = color + E * v.thr;
                    else if (pdf_bsdf + pdf_nee > 0) color = color + E * v.thr * powerHeuristic(pdf_bsdf, pdf_nee);
                    pdf_bsdf = 0;
                    pdf_nee = 0;
                    if (vi + 1 < path_len) {
                        const Vtx &nx = path_buf[vi + 1];
                        const D3 dir = normalized(nx.p - v.p);
                        const double c = dot(dir, v.n);
                        pdf_bsdf = c > 0 ? c / kPiD : 0.0;
                        const D3 diff = nx.p - v.p;
                        const double cl = std::fabs(dot(normalized(diff), nx.n));
                        pdf_nee = cl < 1e-6 ? 0.0 : lum[nx.mat] / total * dot(diff, diff) / cl;
                    }
                    if (lights) {
                        const uint32_t db = oracle::ptm::dim_bounce((int)vi, 3);
                        const double uo = rnd(db) * total;
                        size_t o = std::upper_bound(obj_cdf.begin(), obj_cdf.end(), uo) - obj_cdf.begin();
                        if (o >= N) o = N - 1;
                        const or_object &ob = s->objects[o];
                        const double ut = rnd(db + 1) * obj_area[o];
                        const double *cb = tri_cdf.data() + ob.tri_begin;
                        size_t k = std::upper_bound(cb, cb + ob.tri_count, ut) - cb;
                        if (k >= ob.tri_count) k = ob.tri_count - 1;
                        const Tri &T = tris[ob.tri_begin + k];
                        double uu = rnd(db + 2), vv = rnd(db + 3);
                        if (uu + vv > 1) {
                            uu = 1 - uu;
                            vv = 1 - vv;
                        }
                        const D3 lp = T.a + (T.b - T.a) * uu + (T.c - T.a) * vv;
                        const D3 perp = cross(T.a - T.b, T.a - T.c);
                        const D3 ln = normalized(perp);
                        // pick probability x triangle probability / triangle area
                        const double lpdf = (obj_w[o] / total) / obj_area[o];
                        const D3 to = lp - v.p;
                        const double dist = length(to);
                        const D3 w = to * (1.0 / dist);
                        const double cs = dot(w, v.n);
                        const double nee_pdf_bsdf = cs > 0 ? cs / kPiD : 0.0;
                        const double cl = std::fabs(dot(w, ln));
                        const double nee_pdf_nee = cl < 1e-6 ? 0.0 : lpdf * dist * dist / cl;
                        D3 Ld{0, 0, 0};
                        const auto sh = bvh.closest(v.p + w * 1e-5, w);
                        const bool visible = sh.second < 0 || sh.first > dist - 2e-5;
                        if (visible && cs > 0) {
                            const double G = cs * cl / (dist * dist);
                            Ld = emission(ob.material) * albedo(v.mat) * (1.0 / kPiD) * (G / lpdf);
                        }
                        if (nee_pdf_nee + nee_pdf_bsdf > 0)
                            color = color + Ld * v.thr * powerHeuristic(nee_pdf_nee, nee_pdf_bsdf);
                    }
                    prev_spec = false;
                }
                acc = acc + color;
            }
            double *o = sum_rgb + pix * 3;
            o[0] += acc.x;
            o[1] += acc.y;
            o[2] += acc.z;
        }
    };
    const int threads = cfg->threads > 0 ? cfg->threads : (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads <= 1 || nwork < 16) {
        work(0, nwork);
        return;
    }
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const int64_t b = next.fetch_add(4);
            if (b >= nwork) break;
            work(b, std::min<int64_t>(nwork, b + 4));
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto &th : pool) th.join();
}
