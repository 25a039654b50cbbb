// oracle_render.cpp -- CPU restatement of DevilRay's integrator (TEST
// INFRASTRUCTURE: the oracle of the GB300 renderer; never linked into the
// product).
//
// Restates sampleColor (include/tracing/PathGeneration.hpp:363-515) with the
// path depth as a parameter, on a flattened scene (world-space triangle soup,
// objects as contiguous triangle ranges with one material each, identity
// transforms). Switches select
//   * the random numbers: the GPU's Philox layout, or a replayed stream
//     consumed in the reference's call order (for pinning against the
//     reference's own sampleColor through the harness);
//   * sin/cos/acos: the portable polynomials (bit-identical to the GPU) or the
//     platform's std functions (the reference's calls);
//   * closest hit: the canonical semantics over one BVH of the soup (the GPU's)
//     or the reference's cast: a loop over objects, each traversed through its
//     own median-split BBH with the reference's first-found rule;
//   * the light-triangle table order: the object's triangles in soup order (the
//     GPU's) or in its BBH-sorted order (the reference's test helper,
//     test/src/TracingTestHelpers.hpp:97-112).
// Every FP32 expression keeps the reference's evaluation order (Vec3/Vec4
// operators of include/Utils.hpp); compiled with -ffp-contract=off.

#include "oracle.h"
#include "oracle_common.hpp"
#include "oracle_ptmath.hpp"
#include "oracle_scene.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

using namespace oracle;

namespace {

constexpr float kPi = 3.14159274f;  // std::numbers::pi_v<float> (include/Utils.hpp:27)

inline V4 add4(const V4 &a, const V4 &b) { return V4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 mul4(const V4 &a, const V4 &b) { return V4{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
inline V4 mul4s(const V4 &a, float f) { return V4{a.x * f, a.y * f, a.z * f, a.w * f}; }
inline V4 div4s(const V4 &a, float f) { return mul4s(a, 1.0f / f); }
inline float luminance(const V4 &c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
inline float powerHeuristic(float a, float b) { return a * a / (a * a + b * b); }

// areaToSolidAngle (include/Utils.hpp:236-247)
inline float areaToSolidAngle(const V3 &from, const V3 &to, const V3 &to_n)
{
    const V3 diff = sub(to, from);
    const float d2 = dot(diff, diff);
    const V3 dir = normalized(diff);
    const float c = std::abs(dot(dir, to_n));
    if (c < 1e-6f) return 0.0f;
    return d2 / c;
}

// cosineWeightedHemispherePdf (include/Utils.hpp:249-254)
inline float cosineHemispherePdf(const V3 &cur, const V3 &next, const V3 &n)
{
    const V3 dir = normalized(sub(next, cur));
    const float c = dot(dir, n);
    return c > 0 ? c / kPi : 0.0f;
}


inline V4 radiantExitance(const Mat &m)  // include/tracing/LightSampling.hpp:7-13
{
    if (m.kind != 0) return V4{0, 0, 0, 0};
    return mul4s(m.emission, kPi);
}

struct Rng {
    int mode = 0;
    const float *stream = nullptr;
    size_t cursor = 0;
    size_t limit = 0;
    uint64_t seed = 0;
    uint32_t pixel = 0, sample = 0;
    float next(uint32_t dim)
    {
        if (mode == 1) {
            const float v = stream[cursor < limit ? cursor : limit - 1];
            ++cursor;
            return v;
        }
        return ptm::uniform(seed, pixel, sample, dim);
    }
};

struct Trig {
    int mode;  // 0 portable, 1 std
    void sincos(float x, float &s, float &c) const
    {
        if (mode == 1) {
            s = std::sin(x);
            c = std::cos(x);
        } else {
            ptm::sincos(x, s, c);
        }
    }
    float acos(float z) const { return mode == 1 ? std::acos(z) : ptm::acos(z); }
};

struct Hit {
    float t;
    int prim;
};


}  // namespace


namespace {

V3 vtx(const or_scene &s, int tri, int k)
{
    const float *q = &s.pos[(size_t)tri * 9 + (size_t)k * 3];
    return V3{q[0], q[1], q[2]};
}

// triangleArea (include/Utils.hpp:218-224)
float triangleArea(const V3 &A, const V3 &B, const V3 &C)
{
    const V3 u = sub(A, B), v = sub(A, C);
    return length(cross(u, v)) / 2;
}

// Closest hit of one ray: returns prim >= 0 on a hit.
Hit castRay(const or_scene &s, int cast_mode, const V3 &p, const V3 &v)
{
    Hit best{std::numeric_limits<float>::infinity(), -1};
    if (cast_mode == 0) {
        const float r8[8] = {p.x, p.y, p.z, std::numeric_limits<float>::infinity(), v.x, v.y, v.z, 0.0f};
        float t;
        int32_t prim;
        if (s.soup_bbh) or_bbh_trace_canonical(s.soup_bbh.get(), r8, 1, s.slack, &t, &prim, 0, 1);
        else prim = -1;
        if (prim >= 0) best = Hit{t, prim};
        return best;
    }
    // reference cast (IntersectionTestsImpl.hpp:234-251): objects in order,
    // replace only on a strictly smaller t.
    bool have = false;
    const float r6[6] = {p.x, p.y, p.z, v.x, v.y, v.z};
    for (size_t o = 0; o < s.objects.size(); ++o) {
        if (!s.obj_bbh[o]) continue;
        float t;
        int32_t local;
        or_bbh_trace_reference(s.obj_bbh[o].get(), r6, 1, &t, &local, nullptr, nullptr, 0, 1);
        if (local < 0) continue;
        if (!have || best.t > t) {
            have = true;
            best = Hit{t, (int)s.objects[o].tri_begin + local};
        }
    }
    return best;
}

struct Vertex {
    V3 p, n;
    int mat;
    V4 thr;
};

struct LightSample {
    V3 p, n;
    int mat;
    float pdf;
};

}  // namespace

extern "C" {

or_scene *or_scene_create(const float *positions, int32_t num_tris, const or_object *objects, int32_t num_objects,
                          const or_material *materials, int32_t num_materials, const int32_t *tri_material,
                          int32_t light_tables)
{
    const auto build_table = light_tables == 1 ? or_alias_build_ref : or_alias_build_sweep;
    auto *s = new or_scene;
    s->pos.assign(positions, positions + (size_t)num_tris * 9);
    if (objects && num_objects > 0) s->objects.assign(objects, objects + num_objects);
    else s->objects.push_back(or_object{0, (uint32_t)num_tris, 0, 0.0f});
    for (int i = 0; i < num_materials; ++i) {
        const or_material &m = materials[i];
        s->mats.push_back(Mat{m.kind, m.ior, V4{m.emission[0], m.emission[1], m.emission[2], m.emission[3]},
                              V4{m.albedo[0], m.albedo[1], m.albedo[2], m.albedo[3]},
                              V4{m.debug_color[0], m.debug_color[1], m.debug_color[2], m.debug_color[3]}});
    }
    if (s->mats.empty()) s->mats.push_back(Mat{0, 1.0f, V4{0, 0, 0, 0}, V4{0.5f, 0.5f, 0.5f, 0}, V4{0, 0, 0, 0}});
    s->tri_object.assign((size_t)num_tris, 0);
    s->tri_material.assign((size_t)num_tris, 0);
    for (size_t o = 0; o < s->objects.size(); ++o)
        for (uint32_t k = 0; k < s->objects[o].tri_count; ++k) {
            s->tri_object[s->objects[o].tri_begin + k] = (int32_t)o;
            s->tri_material[s->objects[o].tri_begin + k] = s->objects[o].material;
        }
    if (tri_material)
        for (int i = 0; i < num_tris; ++i) s->tri_material[i] = tri_material[i];
    float mag = 0.0f;
    for (float x : s->pos) mag = std::max(mag, std::fabs(x));
    s->slack = std::ldexp(std::max(mag, 1.0f / 1024.0f), -14);
    if (num_tris > 0) s->soup_bbh.reset(or_bbh_create(positions, num_tris));

    // Light weights: Renderer::calculateLightWeights (src/Renderer.cpp:113-152).
    const size_t N = s->objects.size();
    std::vector<float> weights(N, 0.0f);
    float total = 0.0f;
    for (size_t i = 0; i < N; ++i) {
        const float A = s->objects[i].surface_area;
        const V4 M = radiantExitance(s->mats[s->objects[i].material]);
        weights[i] = A * luminance(M);
        total += weights[i];
    }
    for (size_t i = 0; i < N; ++i) weights[i] /= total;
    s->light_table.resize(N);
    build_table(weights.data(), (int32_t)N, s->light_table.data());
    s->total_power = total;

    // Per-object BBHs (reference cast) and triangle tables in both orders.
    s->obj_bbh.resize(N);
    s->obj_order.resize(N);
    for (int ord = 0; ord < 2; ++ord) {
        s->tri_table[ord].assign((size_t)num_tris, or_alias_entry{0, 0, 0, 0, 0});
        s->tri_table_map[ord].assign((size_t)num_tris, 0);
    }
    for (size_t o = 0; o < N; ++o) {
        const or_object &ob = s->objects[o];
        if (ob.tri_count == 0) continue;
        s->obj_bbh[o] = BbhPtr(or_bbh_create(positions + (size_t)ob.tri_begin * 9, (int32_t)ob.tri_count));
        std::vector<int32_t> order(ob.tri_count);
        or_bbh_export(s->obj_bbh[o].get(), nullptr, nullptr, order.data());
        s->obj_order[o] = order;
        for (int ord = 0; ord < 2; ++ord) {
            std::vector<float> areas(ob.tri_count);
            for (uint32_t k = 0; k < ob.tri_count; ++k) {
                const int tri = (int)ob.tri_begin + (ord == 0 ? (int)k : order[k]);
                s->tri_table_map[ord][ob.tri_begin + k] = tri;
                areas[k] = triangleArea(vtx(*s, tri, 0), vtx(*s, tri, 1), vtx(*s, tri, 2));
            }
            build_table(areas.data(), (int32_t)ob.tri_count, s->tri_table[ord].data() + ob.tri_begin);
        }
    }
    return s;
}

void or_scene_destroy(or_scene *s) { delete s; }
float or_scene_total_power(const or_scene *s) { return s->total_power; }

void or_scene_light_table(const or_scene *s, or_alias_entry *out)
{
    std::memcpy(out, s->light_table.data(), s->light_table.size() * sizeof(or_alias_entry));
}

void or_render(const or_scene *s, const or_camera *cam, const or_render_cfg *cfg, float *sample_rgb, float *accum,
               uint32_t *casts_out)
{
    const int W = cam->width, H = cam->height;
    const int64_t npix = (int64_t)W * H;
    const int spp = cfg->spp;
    const Trig trig{cfg->trig_mode};
    const int order = cfg->tri_table_order;
    int threads = cfg->threads > 0 ? cfg->threads : (int)std::max(1u, std::thread::hardware_concurrency());
    const int64_t nwork = cfg->pixels ? cfg->num_pixels : npix;
    auto work = [&](int64_t pb, int64_t pe) {
        for (int64_t wi = pb; wi < pe; ++wi) {
            const int64_t pix = cfg->pixels ? cfg->pixels[wi] : wi;
            if (pix < 0 || pix >= npix) continue;
            const int px = (int)(pix % W), py = (int)(pix / W);
            V4 pixel{0, 0, 0, 0};
            uint32_t pixel_casts = 0;
            for (int si = 0; si < spp; ++si) {
                const uint32_t sample = (uint32_t)(cfg->sample_offset + si);
                Rng rng;
                rng.mode = cfg->rng_mode;
                rng.seed = cfg->seed;
                rng.pixel = (uint32_t)pix;
                rng.sample = sample;
                if (rng.mode == 1) {
                    rng.stream = cfg->replay + ((size_t)pix * spp + si) * cfg->replay_stride;
                    rng.limit = (size_t)cfg->replay_stride;
                }
                // cameraRay (include/tracing/CameraRay.hpp:6-34)
                float subx = 0.5f, suby = 0.5f;
                if (cfg->pixel_sampling == 1) {
                    subx = rng.next(ptm::dim_camera(0));
                    suby = rng.next(ptm::dim_camera(1));
                }
                const float pcx = (float)px + subx, pcy = (float)py + suby;
                const float physx = pcx * cam->psx - cam->cx, physy = pcy * cam->psy - cam->cy;
                const float dx = physx / cam->focal, dy = physy / cam->focal;
                const V3 cv = normalized(V3{dx, dy, 1.0f});
                const float *m = cam->m;
                V3 rp{m[3], m[7], m[11]};
                V3 rv{m[0] * cv.x + m[1] * cv.y + m[2] * cv.z, m[4] * cv.x + m[5] * cv.y + m[6] * cv.z,
                      m[8] * cv.x + m[9] * cv.y + m[10] * cv.z};

                if (cfg->debug != 0) {
                    // first-hit debug views (PathGeneration.hpp:274-299, 393-429);
                    // the reference's hit uv is (0, 0), so the UV checkerboard gives its dark colour
                    const Hit hit = castRay(*s, cfg->cast_mode, rp, rv);
                    pixel_casts += 1;
                    V4 color{0, 0, 0, 0};
                    bool counted = true;
                    if (hit.prim >= 0) {
                        const Mat &mat = s->mats[s->tri_material[hit.prim]];
                        if (cfg->debug == 1) {
                            color = mul4(V4{0.5f, 0.5f, 0.5f, 0.0f}, mat.debug);
                        } else {
                            const V3 A = vtx(*s, hit.prim, 0), B = vtx(*s, hit.prim, 1), C = vtx(*s, hit.prim, 2);
                            if (cfg->debug == 2) {
                                // testTriangleIntersection's barycentrics at the hit's t
                                const V3 n_f = cross(sub(A, B), sub(A, C));
                                const float sgn_area2 = dot(n_f, n_f);
                                const V3 hp = add(rp, mul(rv, hit.t));
                                const V3 n_1 = cross(sub(hp, A), sub(C, A));
                                const V3 n_2 = cross(sub(B, A), sub(hp, A));
                                const float w_B = dot(n_f, n_1) / sgn_area2;
                                const float w_C = dot(n_f, n_2) / sgn_area2;
                                const float w_A = 1 - w_B - w_C;
                                color = V4{w_A, w_B, w_C, 0.0f};
                            } else {
                                const bool ccw = dot(cross(sub(A, B), sub(A, C)), rv) > 0;
                                color = ccw ? V4{1.0f, 0.73f, 0.47f, 0.0f} : V4{0.53f, 0.82f, 1.0f, 0.0f};
                            }
                        }
                    } else if (cfg->debug == 1) {
                        counted = false;
                    }
                    if (sample_rgb) {
                        float *o = sample_rgb + ((size_t)si * npix + pix) * 3;
                        o[0] = color.x;
                        o[1] = color.y;
                        o[2] = color.z;
                    }
                    if (counted) {
                        pixel.w += 1;
                        pixel = add4(pixel, color);
                    }
                    continue;
                }

                // path construction (:431-447)
                V4 thr{1, 1, 1, 0};
                int stack[3];
                int ssize = 0;
                std::vector<Vertex> path;
                path.reserve((size_t)cfg->max_depth);
                uint32_t casts = 0;
                for (int depth = 0; depth < cfg->max_depth; ++depth) {
                    const Hit hit = castRay(*s, cfg->cast_mode, rp, rv);
                    ++casts;
                    if (hit.prim < 0) break;
                    // getIntersectionTris (IntersectionTestsImpl.hpp:36-67) with an identity transform
                    const V3 A = vtx(*s, hit.prim, 0), B = vtx(*s, hit.prim, 1), C = vtx(*s, hit.prim, 2);
                    V3 n = normalized(cross(sub(A, B), sub(A, C)));
                    if (dot(n, rv) > 0) n = mul(n, -1.0f);
                    n = normalized(mulv(n, V3{1.0f, 1.0f, 1.0f}));
                    // p = model_to_world.applyToPoint(ray.p + ray.v * t), identity transform
                    const V3 hp = add(mulv(add(rp, mul(rv, hit.t)), V3{1.0f, 1.0f, 1.0f}), V3{0.0f, 0.0f, 0.0f});
                    const int mat_id = s->tri_material[hit.prim];
                    const int obj = s->tri_object[hit.prim];
                    path.push_back(Vertex{hp, n, mat_id, thr});
                    const Mat &mat = s->mats[mat_id];
                    // generateNewRay (PathGeneration.hpp:114-211)
                    V3 normal = n;
                    if (mat.kind == 0) {
                        const float u0 = rng.next(ptm::dim_bounce(depth, 0));
                        const float u1 = rng.next(ptm::dim_bounce(depth, 1));
                        const float theta0 = 2 * kPi * u0;
                        const float theta1 = trig.acos(1 - 2 * u1);
                        float s0, c0, s1, c1;
                        trig.sincos(theta0, s0, c0);
                        trig.sincos(theta1, s1, c1);
                        const V3 sph{s1 * s0, s1 * c0, c1};
                        const V3 w_out = normalized(add(sph, normal));
                        thr = mul4(thr, mat.albedo);
                        rv = w_out;
                        rp = hp;
                    } else {
                        float n1, n2;
                        auto ior_of_object = [&](int o) {
                            const Mat &tm = s->mats[s->objects[o].material];
                            return tm.kind == 1 ? tm.ior : 1.0f;
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
                        const float eta = n1 / n2;
                        const float d = dot(rv, normal);
                        const float k = 1 - eta * eta * (1 - d * d);
                        V3 vv;
                        if (n1 > n2 && k < 0) {
                            vv = sub(rv, mul(mul(normal, 2.0f), d));
                        } else {
                            // schlick (:75-86), evaluated in double as written
                            const float r = (n1 - n2) / (n1 + n2);
                            const float R0 = r * r;
                            const float cosT1 = 1 - (-d);
                            const float c2 = cosT1 * cosT1;
                            const float c4 = c2 * c2;
                            const float c5 = c4 * cosT1;
                            const float F = (float)((double)R0 + (1.0 - (double)R0) * (double)c5);
                            if (rng.next(ptm::dim_bounce(depth, 2)) < F) {
                                vv = sub(rv, mul(mul(normal, 2.0f), d));
                            } else {
                                if (ssize > 0 && stack[ssize - 1] == obj) --ssize;
                                else if (ssize < 3) stack[ssize++] = obj;
                                normal = mul(normal, -1.0f);
                                const float dotp = -d;
                                vv = add(mul(normal, std::sqrt(k) - dotp * eta), mul(rv, eta));
                            }
                        }
                        rv = vv;
                        rp = hp;
                    }
                    rp = add(rp, mul(normal, 1e-5f));
                }

                // shading (:455-510)
                V4 color{0, 0, 0, 0};
                bool prev_spec = true;
                float pdf_bsdf = 0, pdf_nee = 0;
                for (size_t vi = 0; vi < path.size(); ++vi) {
                    const Vertex &v = path[vi];
                    const Mat &mat = s->mats[v.mat];
                    if (mat.kind != 0) {
                        prev_spec = true;
                        continue;
                    }
                    // misWeightedEmission (:306-318)
                    if (prev_spec) color = add4(color, mul4(mat.emission, v.thr));
                    else if (pdf_bsdf + pdf_nee > 0)
                        color = add4(color, mul4s(mul4(mat.emission, v.thr), powerHeuristic(pdf_bsdf, pdf_nee)));
                    pdf_bsdf = 0;
                    pdf_nee = 0;
                    if (vi + 1 < path.size()) {  // computeNextBounceMisPdfs (:320-334)
                        const Vertex &nx = path[vi + 1];
                        pdf_bsdf = cosineHemispherePdf(v.p, nx.p, v.n);
                        const float L = luminance(radiantExitance(s->mats[nx.mat]));
                        const float pdf_area = L / s->total_power;
                        pdf_nee = pdf_area * areaToSolidAngle(v.p, nx.p, nx.n);
                    }
                    if (s->total_power > 0.0f && !s->light_table.empty()) {
                        // samplePointOnLights (:234-272)
                        const int b = (int)vi;
                        int32_t oi, ti;
                        float opdf, tpdf;
                        const float r0 = rng.next(ptm::dim_bounce(b, 3));
                        const float r1 = rng.next(ptm::dim_bounce(b, 4));
                        or_alias_sample(s->light_table.data(), (int32_t)s->light_table.size(), r0, r1, &oi, &opdf);
                        const or_object &ob = s->objects[oi];
                        const float r2 = rng.next(ptm::dim_bounce(b, 5));
                        const float r3 = rng.next(ptm::dim_bounce(b, 6));
                        or_alias_sample(s->tri_table[order].data() + ob.tri_begin, (int32_t)ob.tri_count, r2, r3, &ti,
                                        &tpdf);
                        const int tri = s->tri_table_map[order][ob.tri_begin + ti];
                        const V3 A = vtx(*s, tri, 0), B = vtx(*s, tri, 1), C = vtx(*s, tri, 2);
                        float uu = rng.next(ptm::dim_bounce(b, 7));
                        float vv = rng.next(ptm::dim_bounce(b, 8));
                        if (uu + vv > 1) {
                            uu = 1 - uu;
                            vv = 1 - vv;
                        }
                        const V3 lp = add(add(A, mul(sub(B, A), uu)), mul(sub(C, A), vv));
                        const V3 one{1.0f, 1.0f, 1.0f};
                        const V3 Aw = mulv(A, one), Bw = mulv(B, one), Cw = mulv(C, one);
                        const V3 perp = cross(sub(Aw, Bw), sub(Aw, Cw));
                        const float perp_length = length(perp);
                        const V3 ln = divs(perp, perp_length);
                        const float area = perp_length / 2.0f;
                        LightSample ls{add(mulv(lp, one), V3{0, 0, 0}), ln, ob.material, opdf * tpdf / area};
                        const Mat &lmat = s->mats[ls.mat];
                        const float nee_pdf_bsdf = cosineHemispherePdf(v.p, ls.p, v.n);
                        const float nee_pdf_nee = ls.pdf * areaToSolidAngle(v.p, ls.p, ls.n);
                        // evaluateDirectLighting (:336-361) with visible (:213-224)
                        V4 Ld{0, 0, 0, 0};
                        {
                            const float distance = length(sub(ls.p, v.p));
                            const V3 dirv = divs(sub(ls.p, v.p), distance);
                            const V3 sp = add(v.p, mul(dirv, 1e-5f));
                            const Hit sh = castRay(*s, cfg->cast_mode, sp, dirv);
                            const bool visible = sh.prim < 0 || (double)sh.t > (double)distance - 1e-5 * 2;
                            if (visible) {
                                const float dist2 = length(sub(ls.p, v.p));
                                const V3 w_light = divs(sub(ls.p, v.p), dist2);
                                const V4 brdf = div4s(mat.albedo, kPi);
                                const float cos_s = dot(w_light, v.n);
                                const float cos_l = dot(w_light, ls.n);
                                if (cos_s > 0) {
                                    const float G = cos_s * std::abs(cos_l) / (dist2 * dist2);
                                    Ld = div4s(mul4s(mul4(lmat.emission, brdf), G), ls.pdf);
                                }
                            }
                        }
                        if (nee_pdf_nee + nee_pdf_bsdf > 0)
                            color = add4(color, mul4s(mul4(Ld, v.thr), powerHeuristic(nee_pdf_nee, nee_pdf_bsdf)));
                    }
                    prev_spec = false;
                }
                if (sample_rgb) {
                    float *o = sample_rgb + ((size_t)si * npix + pix) * 3;
                    o[0] = color.x;
                    o[1] = color.y;
                    o[2] = color.z;
                }
                pixel.w += 1;
                pixel = add4(pixel, color);
                pixel_casts += casts;
            }
            if (accum) {
                float *a = accum + pix * 4;
                a[0] = pixel.x;
                a[1] = pixel.y;
                a[2] = pixel.z;
                a[3] = pixel.w;
            }
            if (casts_out) casts_out[pix] = pixel_casts;
        }
    };
    if (threads <= 1 || nwork < 64) {
        work(0, nwork);
        return;
    }
    // interleaved chunks of 64 work items so that expensive regions spread over the threads
    std::vector<std::thread> pool;
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const int64_t b = next.fetch_add(64);
            if (b >= nwork) break;
            work(b, std::min<int64_t>(nwork, b + 64));
        }
    };
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto &th : pool) th.join();
}

void or_create_pixels(const float *accum, int32_t width, int32_t height, int32_t gamma, uint32_t *out)
{
    // toSRGB, to_u32, packPixel and setPixel of src/Renderer.cpp:53-79, in the
    // same mixed float/double arithmetic.
    auto to_srgb = [gamma](float linear) -> float {
        if (!gamma) return linear;
        const float r = std::clamp(linear, 0.f, 1.f);
        if (r < 0.0031308) return r * 12.92;
        return std::pow(r, 1 / 2.4f) * 1.055 - 0.055f;
    };
    auto to_u32 = [](float f) -> uint32_t { return static_cast<uint32_t>(std::round(f)); };
    auto pack = [&](float r, float g, float b, float a) -> uint32_t {
        return (to_u32(to_srgb(r) * 255) << 0) | (to_u32(to_srgb(g) * 255) << 8) |
               (to_u32(to_srgb(b) * 255) << 16) | (to_u32(std::clamp(a, 0.0f, 1.0f) * 255) << 24);
    };
    for (int32_t y = 0; y < height; ++y)
        for (int32_t x = 0; x < width; ++x) {
            const float *p = accum + 4 * ((size_t)x + (size_t)y * width);
            const size_t dst = (size_t)x + (size_t)(height - y - 1) * width;
            if (p[3] == 0)
                out[dst] = pack(0, 0, 0, 1.0f);
            else
                out[dst] = pack(p[0] / p[3], p[1] / p[3], p[2] / p[3], 1.0f);
        }
}

}  // extern "C"
