// ref_harness.cpp -- thin C entry points over DevilRay's OWN host code
// (TEST INFRASTRUCTURE). Compiled by oracle/Makefile directly against the
// reference headers and sources where they lie; its output library goes to
// oracle/_ref/ and is used only to pin the oracle restatement and to write the
// golden fixtures under tests/golden/. Nothing here re-implements the
// reference: every result comes from calling the reference function named.

#include <cstdint>
#include <cstring>
#include <memory>
#include <limits>
#include <numbers>
#include <random>
#include <vector>

#include "tracing/Camera.hpp"  // must precede PathGeneration.hpp (src/device/implementation.cu:6-8)
#include "tracing/PathGeneration.hpp"
#include "tracing/IntersectionTestsImpl.hpp"
#include "tracing/LightSampling.hpp"
#include "tracing/DistributionSamplers.hpp"
#include "models/BBH.hpp"
#include "models/Mesh.hpp"

#include <stdexcept>
#include <string>

// Replays caller-provided uniforms through the `.rnd()` interface the
// reference samplers are templated on (test/src/TracingTestHelpers.hpp:45-57).
struct ReplayRng {
    const float *values;
    size_t count;
    size_t cursor = 0;
    float rnd()
    {
        const float v = values[cursor < count ? cursor : count - 1];
        ++cursor;
        return v;
    }
};

namespace {
struct RefBBH {
    Mesh mesh;
    BBH bbh;
    int ntri;
};

TriangleMesh hostView(RefBBH &h)
{
    // test/src/TracingTestHelpers.hpp:69-83
    TriangleMesh object{};
    object.points = h.mesh.points.data();
    object.normals = h.mesh.normals.data();
    object.triangles = h.mesh.triangles.data();
    object.triangle_count = static_cast<int>(h.mesh.triangles.size());
    object.model_to_world = Transform{};
    object.material = 0;
    object.triangle_sampler = nullptr;
    object.surface_area = 0;
    object.base_surface_area = 0;
    object.bbh = BBHGpuView{std::span<const BBHNode>{h.bbh.nodes.hostPtr(), h.bbh.nodes.size()}};
    return object;
}
}  // namespace

extern "C" {

int refh_tri_test(const float ray[6], const float tri[9], float out[4])
{
    const Ray r{.p = {ray[0], ray[1], ray[2]}, .v = {ray[3], ray[4], ray[5]}};
    const TriangleVertices t{{tri[0], tri[1], tri[2]}, {tri[3], tri[4], tri[5]}, {tri[6], tri[7], tri[8]}};
    const auto hit = testTriangleIntersection(r, t);
    if (!hit.has_value()) return 0;
    out[0] = hit->t;
    out[1] = hit->bari.x;
    out[2] = hit->bari.y;
    out[3] = hit->bari.z;
    return 1;
}

int refh_box_test(const float box[6], const float ray[6], float *t)
{
    const AABB b{.min = {box[0], box[1], box[2]}, .max = {box[3], box[4], box[5]}};
    const Ray r{.p = {ray[0], ray[1], ray[2]}, .v = {ray[3], ray[4], ray[5]}};
    const auto hit = testBoxIntersection(b, r);
    if (!hit.has_value()) return 0;
    *t = *hit;
    return 1;
}

// Soup -> Mesh with triangle k owning points 3k..3k+2 and normal index k (the
// traversal never reads normal indices, so ni carries the original id through
// generateSimpleBBH's in-place sort).
void *refh_bbh_create(const float *pos, int ntri)
{
    auto *h = new RefBBH{Mesh{}, BBH{0, DeviceVector<BBHNode>{{}}}, ntri};
    h->mesh.name = "soup";
    for (int k = 0; k < ntri; ++k) {
        for (int j = 0; j < 3; ++j)
            h->mesh.points.push_back(Vec3{pos[k * 9 + j * 3], pos[k * 9 + j * 3 + 1], pos[k * 9 + j * 3 + 2]});
        h->mesh.normals.push_back(Vec3{0, 0, 1});
        const uint32_t b = 3u * k;
        h->mesh.triangles.push_back(Triangle{.a = {b, (uint32_t)k}, .b = {b + 1, (uint32_t)k}, .c = {b + 2, (uint32_t)k}});
    }
    h->bbh = generateSimpleBBH(h->mesh);
    return h;
}

void refh_bbh_destroy(void *p) { delete static_cast<RefBBH *>(p); }

int refh_bbh_num_nodes(void *p) { return (int)static_cast<RefBBH *>(p)->bbh.nodes.size(); }
int refh_bbh_depth(void *p) { return static_cast<RefBBH *>(p)->bbh.depth; }

void refh_bbh_export(void *p, float *boxes, int *links, int *order)
{
    auto *h = static_cast<RefBBH *>(p);
    const BBHNode *nodes = h->bbh.nodes.hostPtr();
    for (size_t i = 0; i < h->bbh.nodes.size(); ++i) {
        const auto &n = nodes[i];
        const float b[6] = {n.box.min.x, n.box.min.y, n.box.min.z, n.box.max.x, n.box.max.y, n.box.max.z};
        std::memcpy(boxes + i * 6, b, sizeof(b));
        links[i * 5 + 0] = n.left_child;
        links[i * 5 + 1] = n.right_child;
        links[i * 5 + 2] = n.parent_index;
        links[i * 5 + 3] = n.tris_begin;
        links[i * 5 + 4] = n.tris_end;
    }
    for (int i = 0; i < h->ntri; ++i) order[i] = (int)h->mesh.triangles[i].a.ni;
}

// getIntersectionBenchmark on every ray. The original triangle index of a hit
// is recovered as the unique triangle whose reference test reproduces the hit's
// t and barycentrics bit for bit; -2 marks an ambiguous (tied) recovery.
void refh_bbh_trace(void *p, const float *rays, int nray, float *t_out, int *id_out,
                    float *n_out, float *area_out, int64_t *box_tests, int64_t *tri_tests)
{
    auto *h = static_cast<RefBBH *>(p);
    const TriangleMesh view = hostView(*h);
    for (int r = 0; r < nray; ++r) {
        const Ray ray{.p = {rays[r * 6], rays[r * 6 + 1], rays[r * 6 + 2]},
                      .v = {rays[r * 6 + 3], rays[r * 6 + 4], rays[r * 6 + 5]}};
        benchmark::HitTests counts;
        const auto hit = getIntersectionBenchmark(ray, view, counts);
        box_tests[r] = counts.bbox_tests;
        tri_tests[r] = counts.triangle_tests;
        if (!hit.has_value()) {
            t_out[r] = std::numeric_limits<float>::infinity();
            id_out[r] = -1;
            continue;
        }
        t_out[r] = hit->t;
        if (n_out) {
            n_out[r * 3] = hit->n.x;
            n_out[r * 3 + 1] = hit->n.y;
            n_out[r * 3 + 2] = hit->n.z;
        }
        if (area_out) area_out[r] = hit->triangle.area;
        int found = -1;
        for (int i = 0; i < h->ntri; ++i) {
            const auto &tri = h->mesh.triangles[i];
            const TriangleVertices tv{h->mesh.points[tri.a.pi], h->mesh.points[tri.b.pi], h->mesh.points[tri.c.pi]};
            const auto c = testTriangleIntersection(ray, tv);
            if (!c.has_value()) continue;
            if (std::memcmp(&c->t, &hit->t, 4) == 0 && std::memcmp(&c->bari, &hit->triangle.bari, 12) == 0) {
                found = found == -1 ? (int)tri.a.ni : -2;
            }
        }
        id_out[r] = found;
    }
}

// generateAliasTable on the given weights.
void refh_alias_build(const float *w, int n, float *pA, float *pdfA, float *pdfB, int *A, int *B)
{
    const AliasTable table = generateAliasTable(std::span<const float>{w, static_cast<size_t>(n)});
    const AliasEntry *e = table.entries.hostPtr();
    for (int i = 0; i < n; ++i) {
        pA[i] = e[i].p_A;
        pdfA[i] = e[i].pdf_A;
        pdfB[i] = e[i].pdf_B;
        A[i] = e[i].A;
        B[i] = e[i].B;
    }
}

// sample() over a table given as struct-of-arrays, with replayed uniforms.
void refh_alias_sample(const float *pA, const float *pdfA, const float *pdfB, const int *A, const int *B,
                       int n, const float *uniforms, int ndraw, int *idx_out, float *pdf_out)
{
    std::vector<AliasEntry> t(n);
    for (int i = 0; i < n; ++i) t[i] = AliasEntry{pA[i], pdfA[i], pdfB[i], A[i], B[i]};
    ReplayRng rng{uniforms, (size_t)ndraw * 2};
    for (int d = 0; d < ndraw; ++d) {
        const auto s = sample(std::span<const AliasEntry>{t}, rng);
        idx_out[d] = s.index;
        pdf_out[d] = s.pdf;
    }
}

// The 200,000-weight lognormal input of test/src/test_alias.cpp:193-229.
void refh_lognormal(int n, unsigned seed, float *out)
{
    std::mt19937 rng(seed);
    std::lognormal_distribution<float> dist(0.0f, 1.0f);
    for (int i = 0; i < n; ++i) out[i] = dist(rng);
}

// uniformSphereSample / cosineWeightedHemisphereSample / uniformTriangleSample
// (DistributionSamplers.hpp:8-42, 92-104) with replayed uniforms.
void refh_sphere_sample(const float *u, int n, float *out)
{
    ReplayRng rng{u, (size_t)n * 2};
    for (int i = 0; i < n; ++i) {
        const Vec3 v = uniformSphereSample(rng);
        out[i * 3] = v.x; out[i * 3 + 1] = v.y; out[i * 3 + 2] = v.z;
    }
}

void refh_cosine_sample(const float *normal, const float *u, int n, float *out)
{
    ReplayRng rng{u, (size_t)n * 2};
    const Vec3 nn{normal[0], normal[1], normal[2]};
    for (int i = 0; i < n; ++i) {
        const Vec3 v = cosineWeightedHemisphereSample(nn, rng);
        out[i * 3] = v.x; out[i * 3 + 1] = v.y; out[i * 3 + 2] = v.z;
    }
}

// cameraRay (include/tracing/CameraRay.hpp:6-34) for a row-major 4x4 transform.
void refh_camera_ray(const float *m16, float focal, float cx, float cy, float psx, float psy,
                     float px, float py, int sampling, const float *u, float *ray_out)
{
    Camera cam{};
    std::memcpy(cam.transform.values, m16, sizeof(float) * 16);
    cam.intrinsics = Intrinsics{.focal_length = focal, .center = Vec2f{cx, cy}};
    cam.physical_pixel_size = Size2f{psx, psy};
    ReplayRng rng{u, 2};
    const Ray r = cameraRay(cam, Vec2f{px, py}, static_cast<PixelSampling>(sampling), 0, rng);
    ray_out[0] = r.p.x; ray_out[1] = r.p.y; ray_out[2] = r.p.z;
    ray_out[3] = r.v.x; ray_out[4] = r.v.y; ray_out[5] = r.v.z;
}

// sampleColor (include/tracing/PathGeneration.hpp:363-515, max_depth 10) on a
// flattened scene: each object becomes a Mesh of its triangles (triangle k
// owning points 3k..3k+2) with an identity transform, its BBH from
// generateSimpleBBH and its triangle sampler built after the sort
// (test/src/TracingTestHelpers.hpp:97-112); the light table follows
// Renderer::calculateLightWeights (src/Renderer.cpp:113-152) with the
// reference's radiantExitance and luminance. Uniforms are replayed from
// `replay` ([pixel][sample][stride]); out_rgb receives each sample's colour
// and out_w (may be NULL) its sample count (0 or 1). debug: DebugOptions.
void refh_render_samples(const float *pos, const int *obj_begin, const int *obj_count, const int *obj_mat,
                         const float *obj_area, int nobj, const float *mats, int nmat, const float *m16, float focal,
                         float cx, float cy, int width, int height, float psx, float psy, int sampling, int spp,
                         const float *replay, int stride, float *out_rgb, unsigned *casts_out, int debug,
                         float *out_w)
{
    std::vector<Material> materials;
    for (int i = 0; i < nmat; ++i) {
        const float *m = mats + i * 16;
        int32_t kind;  // dr_material::kind is an int32 in the first word
        std::memcpy(&kind, m, sizeof(kind));
        if (kind == 1) {
            TransparentMaterial t{};
            t.debug_color = Vec4{m[12], m[13], m[14], m[15]};
            t.inside_medium = Medium{.ior = m[1]};
            materials.push_back(t);
        } else {
            DiffuseMaterial d{};
            d.debug_color = Vec4{m[12], m[13], m[14], m[15]};
            d.emission = Vec4{m[4], m[5], m[6], m[7]};
            d.diffuse_reflectance = Vec4{m[8], m[9], m[10], m[11]};
            materials.push_back(d);
        }
    }
    struct Obj {
        Mesh mesh;
        BBH bbh{0, DeviceVector<BBHNode>{{}}};
        AliasTable sampler;
    };
    std::vector<std::unique_ptr<Obj>> store;
    std::vector<TriangleMesh> objects;
    for (int o = 0; o < nobj; ++o) {
        auto ob = std::make_unique<Obj>();
        ob->mesh.name = "object";
        for (int k = 0; k < obj_count[o]; ++k) {
            const float *q = pos + (size_t)(obj_begin[o] + k) * 9;
            for (int j = 0; j < 3; ++j) ob->mesh.points.push_back(Vec3{q[j * 3], q[j * 3 + 1], q[j * 3 + 2]});
            ob->mesh.normals.push_back(Vec3{0, 0, 1});
            const uint32_t b = 3u * k;
            ob->mesh.triangles.push_back(Triangle{.a = {b, (uint32_t)k}, .b = {b + 1, (uint32_t)k}, .c = {b + 2, (uint32_t)k}});
        }
        ob->bbh = generateSimpleBBH(ob->mesh);
        std::vector<float> areas;
        for (const auto &t : ob->mesh.triangles)
            areas.push_back(triangleArea(ob->mesh.points[t.a.pi], ob->mesh.points[t.b.pi], ob->mesh.points[t.c.pi]));
        ob->sampler = generateAliasTable(areas);
        TriangleMesh view{};
        view.points = ob->mesh.points.data();
        view.normals = ob->mesh.normals.data();
        view.triangles = ob->mesh.triangles.data();
        view.triangle_count = (int)ob->mesh.triangles.size();
        view.model_to_world = Transform{};
        view.material = obj_mat[o];
        view.triangle_sampler = ob->sampler.entries.hostPtr();
        view.surface_area = obj_area[o];
        view.base_surface_area = obj_area[o];
        view.bbh = BBHGpuView{std::span<const BBHNode>{ob->bbh.nodes.hostPtr(), ob->bbh.nodes.size()}};
        objects.push_back(view);
        store.push_back(std::move(ob));
    }
    std::vector<float> weights(objects.size(), 0.0f);
    float total = 0.0f;
    for (size_t i = 0; i < objects.size(); ++i) {
        const auto A = objects[i].surface_area;
        const auto M = radiantExitance(materials[objects[i].material]);
        weights[i] = A * luminance(M);
        total += weights[i];
    }
    for (size_t i = 0; i < objects.size(); ++i) weights[i] /= total;
    const AliasTable light = generateAliasTable(weights);
    const ObjectsInfo info{.total_radiant_power = total};
    Camera cam{};
    std::memcpy(cam.transform.values, m16, sizeof(float) * 16);
    cam.intrinsics = Intrinsics{.focal_length = focal, .center = Vec2f{cx, cy}};
    cam.resolution = Size2i{width, height};
    cam.physical_pixel_size = Size2f{psx, psy};
    const size_t npix = (size_t)width * height;
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            const size_t pix = (size_t)y * width + x;
            unsigned casts = 0;
            for (int s2 = 0; s2 < spp; ++s2) {
                Vec4 pixel{0, 0, 0, 0};
                SampleStats stats{.ray_casts = 0};
                ReplayRng rng{replay + (pix * spp + s2) * stride, (size_t)stride};
                sampleColor(Vec2f{(float)x, (float)y}, pixel, stats, cam, static_cast<PixelSampling>(sampling),
                            std::span<const TriangleMesh>{objects}, info, std::span<const Material>{materials},
                            std::span<const AliasEntry>{light.entries.hostPtr(), light.entries.size()},
                            static_cast<DebugOptions>(debug), rng);
                float *o = out_rgb + ((size_t)s2 * npix + pix) * 3;
                o[0] = pixel.x;
                o[1] = pixel.y;
                o[2] = pixel.z;
                if (out_w) out_w[(size_t)s2 * npix + pix] = pixel.w;
                casts += stats.ray_casts;
            }
            casts_out[pix] = casts;
        }
}

// ---- OBJ loading (src/models/Mesh.cpp) ------------------------------------------

// loadMesh on `path`; NULL when it throws, with the message in `err`.
void *refh_mesh_load(const char *path, char *err, int err_cap)
{
    try {
        return new Mesh(loadMesh(path));
    } catch (const std::exception &e) {
        if (err && err_cap > 0) {
            std::strncpy(err, e.what(), (size_t)err_cap - 1);
            err[err_cap - 1] = 0;
        }
        return nullptr;
    }
}

void refh_mesh_free(void *m) { delete static_cast<Mesh *>(m); }

void refh_mesh_sizes(void *m, int *np, int *nn, int *nt)
{
    const Mesh &mesh = *static_cast<Mesh *>(m);
    *np = (int)mesh.points.size();
    *nn = (int)mesh.normals.size();
    *nt = (int)mesh.triangles.size();
}

// points [np][3], normals [nn][3], triangles [nt][6] (a.pi, a.ni, b.pi, b.ni,
// c.pi, c.ni), the name into name (capacity name_cap).
void refh_mesh_export(void *m, float *points, float *normals, uint32_t *tris, char *name, int name_cap)
{
    const Mesh &mesh = *static_cast<Mesh *>(m);
    for (size_t i = 0; i < mesh.points.size(); ++i) {
        points[3 * i] = mesh.points[i].x;
        points[3 * i + 1] = mesh.points[i].y;
        points[3 * i + 2] = mesh.points[i].z;
    }
    for (size_t i = 0; i < mesh.normals.size(); ++i) {
        normals[3 * i] = mesh.normals[i].x;
        normals[3 * i + 1] = mesh.normals[i].y;
        normals[3 * i + 2] = mesh.normals[i].z;
    }
    for (size_t i = 0; i < mesh.triangles.size(); ++i) {
        const Triangle &t = mesh.triangles[i];
        const uint32_t v[6] = {t.a.pi, t.a.ni, t.b.pi, t.b.ni, t.c.pi, t.c.ni};
        std::memcpy(tris + 6 * i, v, sizeof(v));
    }
    std::strncpy(name, mesh.name.c_str(), (size_t)name_cap - 1);
    name[name_cap - 1] = 0;
}

// normalizeMeshSize then generateCoarseNormals on the loaded mesh.
void refh_mesh_normalize_and_coarse_normals(void *m)
{
    Mesh &mesh = *static_cast<Mesh *>(m);
    normalizeMeshSize(mesh);
    generateCoarseNormals(mesh);
}

}  // extern "C"
