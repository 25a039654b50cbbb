// test_devilray_cxx.cpp -- tests of the C++ interface (Renderer, Scene, GpuTris,
// DistributionSamplers, Mesh, Image) written against the reference's header
// names. Usage: test_devilray_cxx <cpu|gpu|all> <scratch dir>. Prints one line
// per check group and exits non-zero on any failed check.
#include "Renderer.hpp"
#include "Image.hpp"
#include "models/Mesh.hpp"
#include "tracing/DistributionSamplers.hpp"
#include "tracing/GpuTris.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <random>
#include <string>
#include <vector>

namespace {

int g_failed = 0;
int g_checks = 0;

#define CHECK(cond)                                                                    \
    do {                                                                               \
        ++g_checks;                                                                    \
        if (!(cond)) {                                                                 \
            ++g_failed;                                                                \
            std::fprintf(stderr, "  FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);   \
        }                                                                              \
    } while (0)

#define CHECK_NEAR(a, b, tol) CHECK(std::fabs((double)(a) - (double)(b)) <= (double)(tol))

template <class F>
bool throws(F &&f)
{
    try {
        f();
    } catch (const std::exception &) {
        return true;
    }
    return false;
}

std::filesystem::path g_dir;

// ---- CPU: mesh loading, mesh utilities, PNG output ---------------------------

void writeFile(const std::filesystem::path &p, const std::string &text)
{
    std::ofstream f(p);
    f << text;
}

void test_obj_loader()
{
    const auto p = g_dir / "tetra.obj";
    writeFile(p, "# tetra\nmtllib x.mtl\no tetra\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvt 0 0\nvn 0 0 1\ns off\n"
                 "f 1 2 3\nf 1//1 2//1 4//1\nf 1/1/1 3/1/1 4/1/1\nf 2/1 3/1 4/1\n");
    const Mesh m = loadMesh(p.string());
    CHECK(m.name == "tetra");
    CHECK(m.points.size() == 4 && m.normals.size() == 1 && m.triangles.size() == 4);
    CHECK(m.triangles[0].a.pi == 0 && m.triangles[0].b.pi == 1 && m.triangles[0].c.pi == 2);
    CHECK(m.triangles[3].c.pi == 3 && m.triangles[3].a.ni == 0);

    writeFile(g_dir / "quad.obj", "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n");
    CHECK(throws([] { loadMesh((g_dir / "quad.obj").string()); }));
    writeFile(g_dir / "tag.obj", "v 0 0 0\nusemtl foo\n");
    CHECK(throws([] { loadMesh((g_dir / "tag.obj").string()); }));
    writeFile(g_dir / "range.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n");
    CHECK(throws([] { loadMesh((g_dir / "range.obj").string()); }));
    writeFile(g_dir / "neg.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf -1 -2 -3\n");
    CHECK(throws([] { loadMesh((g_dir / "neg.obj").string()); }));
    CHECK(throws([] { loadMesh((g_dir / "missing.obj").string()); }));
    writeFile(g_dir / "nonorm.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n");
    const Mesh n = loadMesh((g_dir / "nonorm.obj").string());
    CHECK(n.normals.size() == 1 && n.normals[0].x == 0 && n.normals[0].z == 0);
}

void test_mesh_utilities()
{
    Mesh m;
    m.points = {{1, 1, 1}, {3, 1, 1}, {1, 3, 1}, {1, 1, 3}};
    m.triangles = {Triangle{{0, 0}, {1, 0}, {2, 0}}, Triangle{{0, 0}, {2, 0}, {3, 0}}};
    generateCoarseNormals(m);
    CHECK(m.normals.size() == 2 && m.triangles[1].a.ni == 1);
    CHECK_NEAR(m.normals[0].length(), 1.0, 1e-6);
    CHECK_NEAR(std::fabs(m.normals[0].z), 1.0, 1e-6);
    const MeshBounds b = calculateMeshBounds(m);
    CHECK_NEAR(b.center.x, 1.5, 1e-6);
    normalizeMeshSize(m);
    CHECK_NEAR(calculateMeshBounds(m).extent, 1.0, 1e-5);
    CHECK_NEAR(triangleArea({0, 0, 0}, {2, 0, 0}, {0, 2, 0}), 2.0, 1e-6);
    Transform t{Vec3{2, 2, 2}, Vec3{1, 0, 0}};
    const Vec3 q = t.applyToPoint({1, 1, 1});
    CHECK(q.x == 3 && q.y == 2 && q.z == 2);
    const Matrix4x4f r = Matrix4x4f::rotation(Vec3{0, 0, 1}, pi / 2);
    const Vec3 d = r.applyToDirection({1, 0, 0});
    CHECK_NEAR(d.y, 1.0, 1e-6);
    CHECK(Matrix4x4f::translation({1, 2, 3}).getOffset().z == 3);
}

uint32_t be32(const std::vector<uint8_t> &b, size_t o)
{
    return (uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | b[o + 3];
}

void test_png_writer()
{
    const Size2i size{300, 250};  // > 64 KiB of rows: several stored blocks
    std::vector<uint32_t> px((size_t)size.area());
    for (size_t i = 0; i < px.size(); ++i) px[i] = (uint32_t)(i * 2654435761u);
    const auto path = g_dir / "img.png";
    savePNG(path.string(), px, size);
    std::ifstream f(path, std::ios::binary);
    std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    CHECK(b.size() > 8 && b[0] == 0x89 && b[1] == 'P' && b[3] == 'G');
    // IHDR
    CHECK(be32(b, 8) == 13 && std::memcmp(&b[12], "IHDR", 4) == 0);
    CHECK(be32(b, 16) == 300 && be32(b, 20) == 250 && b[24] == 8 && b[25] == 6);
    // IDAT: zlib header, stored blocks, rows with filter byte 0
    size_t o = 8 + 12 + 13;
    CHECK(std::memcmp(&b[o + 4], "IDAT", 4) == 0);
    const uint32_t len = be32(b, o);
    std::vector<uint8_t> raw;
    size_t z = o + 8 + 2;
    while (true) {
        const bool last = b[z] & 1;
        const size_t n = b[z + 1] | (size_t)b[z + 2] << 8;
        const size_t nn = b[z + 3] | (size_t)b[z + 4] << 8;
        CHECK((n ^ nn) == 0xffff);
        raw.insert(raw.end(), b.begin() + (std::ptrdiff_t)(z + 5), b.begin() + (std::ptrdiff_t)(z + 5 + n));
        z += 5 + n;
        if (last) break;
    }
    CHECK(z + 4 == o + 8 + len);
    CHECK(raw.size() == (size_t)size.height * (1 + 4 * size.width));
    bool same = true;
    for (int y = 0; y < size.height; ++y) {
        same = same && raw[(size_t)y * (1 + 4 * size.width)] == 0;
        for (int x = 0; x < size.width; ++x) {
            const uint32_t p = px[(size_t)y * size.width + x];
            const uint8_t *q = &raw[(size_t)y * (1 + 4 * size.width) + 1 + 4 * x];
            same = same && q[0] == (uint8_t)p && q[1] == (uint8_t)(p >> 8) && q[2] == (uint8_t)(p >> 16) &&
                   q[3] == (uint8_t)(p >> 24);
        }
    }
    CHECK(same);
}

// ---- GPU: alias tables --------------------------------------------------------

struct ScriptedRng {
    std::vector<float> values;
    size_t cursor = 0;
    float rnd() { return values[std::min(cursor++, values.size() - 1)]; }
};

// Probability of each index implied by a table (1/n per slot, split p_A : 1 - p_A).
std::vector<double> impliedProbabilities(const AliasTable &t)
{
    const size_t n = t.entries.size();
    std::vector<double> p(n, 0.0);
    const AliasEntry *e = t.entries.hostPtr();
    for (size_t j = 0; j < n; ++j) {
        if (e[j].A >= 0 && (size_t)e[j].A < n) p[e[j].A] += e[j].p_A / (double)n;
        if (e[j].p_A < 1.0f && e[j].B >= 0 && (size_t)e[j].B < n) p[e[j].B] += (1.0f - e[j].p_A) / (double)n;
    }
    return p;
}

void checkFidelity(const std::vector<float> &w, double tol)
{
    const AliasTable t = generateAliasTable(w);
    CHECK(t.entries.size() == w.size());
    double total = 0;
    for (float x : w) total += x;
    const auto p = impliedProbabilities(t);
    double worst = 0;
    for (size_t i = 0; i < w.size(); ++i) worst = std::max(worst, std::fabs(p[i] - w[i] / total));
    CHECK(worst <= tol);
}

void test_alias_tables()
{
    CHECK(generateAliasTable(std::vector<float>{}).entries.size() == 0);
    const AliasTable one = generateAliasTable(std::vector<float>{3.0f});
    CHECK(one.entries.size() == 1 && one.entries.hostPtr()[0].p_A == 1.0f && one.entries.hostPtr()[0].A == 0);
    const AliasTable uni = generateAliasTable(std::vector<float>(8, 2.0f));
    for (size_t i = 0; i < 8; ++i) CHECK(uni.entries.hostPtr()[i].p_A == 1.0f);
    const AliasTable zero = generateAliasTable(std::vector<float>(5, 0.0f));
    for (double p : impliedProbabilities(zero)) CHECK_NEAR(p, 0.2, 1e-6);
    checkFidelity({1, 2, 3, 4, 10}, 1e-4);
    std::mt19937 g(5);
    std::uniform_real_distribution<float> u(0, 1);
    std::vector<float> w(1000);
    for (float &x : w) x = u(g);
    checkFidelity(w, 1e-4);
    std::lognormal_distribution<float> ln(0.0f, 1.0f);
    std::vector<float> big(200000);
    for (float &x : big) x = ln(g);
    checkFidelity(big, 1e-3);
    // sample(): slot floor(r0 n), then A when r1 <= p_A
    const AliasTable t = generateAliasTable(std::vector<float>{1, 3});
    const std::span<const AliasEntry> s{t.entries.hostPtr(), t.entries.size()};
    ScriptedRng r0{{0.0f, 0.0f}}, r1{{1.0f, 1.0f}};
    const AliasSample a = sample(s, r0), b = sample(s, r1);
    CHECK(a.index == s[0].A && a.pdf == s[0].pdf_A);
    CHECK(b.index == (1.0f <= s[1].p_A ? s[1].A : s[1].B));
}

// ---- GPU: GpuTris -----------------------------------------------------------

Mesh tetra()
{
    Mesh m;
    m.name = "tetra";
    m.points = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    m.triangles = {Triangle{{0, 0}, {1, 0}, {2, 0}}, Triangle{{0, 0}, {1, 0}, {3, 0}}, Triangle{{0, 0}, {2, 0}, {3, 0}},
                   Triangle{{1, 0}, {2, 0}, {3, 0}}};
    return m;
}

void test_gpu_tris()
{
    Mesh m = tetra();
    GpuTris t = convertMeshToTris(m);
    CHECK(t.points.size() == 4 && t.triangles.size() == 4);
    CHECK(t.bbh.nodes.size() > 0);
    CHECK(t.triangle_sampler.entries.size() == 4);
    GpuTris ns = convertMeshToTris(m, false);
    CHECK(ns.triangle_sampler.entries.size() == 0);

    GpuTris quad = createQuadMesh(Vec3{0, 0, 0}, Vec3{0, 0, 1}, Vec3{1, 0, 0}, 2.0f);
    CHECK(quad.points.size() == 4 && quad.triangles.size() == 2);
    for (size_t i = 0; i < 4; ++i) {
        CHECK_NEAR(std::fabs(quad.points[i].x), 1.0, 1e-5);
        CHECK_NEAR(std::fabs(quad.points[i].y), 1.0, 1e-5);
        CHECK_NEAR(quad.points[i].z, 0.0, 1e-5);
    }
    TriangleMesh v = viewGpuTris(quad);
    CHECK(v.triangle_count == 2 && v.points && v.normals && v.triangles && v.triangle_sampler);
    CHECK(!v.bbh.isEmpty());
    CHECK_NEAR(v.base_surface_area, 4.0, 1e-5);
    CHECK(v.surface_area == v.base_surface_area);
    v.setScale(Vec3{2, 2, 2});
    CHECK_NEAR(v.surface_area, 16.0, 1e-4);
    v.setPosition(Vec3{1, 2, 3});
    CHECK(v.model_to_world.p.y == 2);
}

// ---- GPU: Renderer ----------------------------------------------------------

Camera makeCamera(Size2i res, float focal, float pixel)
{
    Camera cam{};
    cam.transform = Matrix4x4f::identity();
    cam.intrinsics = Intrinsics{focal, Vec2f{res.width / 2.f * pixel, res.height / 2.f * pixel}};
    cam.resolution = res;
    cam.physical_pixel_size = Size2f{pixel, pixel};
    return cam;
}

int addDiffuse(Scene &s, Vec4 emission, Vec4 reflectance, Vec4 debug = Vec4{0.5f, 0.5f, 0.5f, 0})
{
    DiffuseMaterial m{};
    m.debug_color = debug;
    m.emission = emission;
    m.diffuse_reflectance = reflectance;
    s.materials.push_back(m);
    return (int)s.materials.size() - 1;
}

void addQuad(Scene &s, Vec3 c, Vec3 n, Vec3 r, float size, int mat)
{
    s.mesh_storage.push_back(createQuadMesh(c, n, r, size));
    TriangleMesh v = viewGpuTris(s.mesh_storage.back());
    v.material = mat;
    s.objects.push_back(v);
}

void test_renderer_analytic_planes()
{
    // A white receiver facing a large emitter of radiance 0.55 behind the
    // camera: every camera pixel converges to 0.55.
    const Size2i res{256, 256};
    Renderer r(res);
    r.setCamera(makeCamera(res, 50.0f, 0.1f));
    Scene scene;
    const int white = addDiffuse(scene, Vec4{0, 0, 0, 0}, Vec4{1, 1, 1, 0}, Vec4{0.9f, 0.7f, 0.5f, 0});
    const int light = addDiffuse(scene, Vec4{0.55f, 0.55f, 0.55f, 0}, Vec4{0, 0, 0, 0});
    addQuad(scene, Vec3{0, 0, 1}, Vec3{0, 0, -1}, Vec3{1, 0, 0}, 1000.0f, white);
    addQuad(scene, Vec3{0, 0, -1}, Vec3{0, 0, 1}, Vec3{1, 0, 0}, 1000.0f, light);
    r.setScene(std::move(scene));
    r.setOutputOptions(OutputOptions{OutputLinearity::Linear});
    r.setDebug(DebugOptions::Off);
    for (int i = 0; i < 100; ++i) r.render();
    r.createPixels();
    const Vec4 *px = r.getRawPixels();
    double sum = 0, sum2 = 0;
    const int n = res.area();
    for (int i = 0; i < n; ++i) {
        const double v = px[i].x / px[i].w;
        sum += v;
        sum2 += v * v;
    }
    const double mean = sum / n, sd = std::sqrt(std::max(0.0, sum2 / n - mean * mean));
    std::printf("  analytic planes: mean %.5f sd %.5f casts %llu mean time %.3f ms\n", mean, sd,
                (unsigned long long)r.getTotalCasts(), r.getMeanRenderTimes());
    CHECK_NEAR(mean, 0.55, 0.01);
    CHECK(sd <= 0.04);
    CHECK(px[0].w == 100.0f);
    CHECK(r.getTotalCasts() >= (uint64_t)n * 100);
    CHECK(r.getMeanRenderTimes() > 0);
    CHECK_NEAR(r.scene().info.total_radiant_power, 1e6 * 0.55 * pi, 1e6 * 0.55 * pi * 1e-5);
}

void test_renderer_debug_square()
{
    const Size2i res{512, 512};
    Renderer r(res);
    r.setCamera(makeCamera(res, 50.0f, 0.1f));
    Scene scene;
    const int white = addDiffuse(scene, Vec4{0, 0, 0, 0}, Vec4{1, 1, 1, 0}, Vec4{0.9f, 0.7f, 0.5f, 0});
    addQuad(scene, Vec3{0, 0, 1}, Vec3{0, 0, -1}, Vec3{1, 0, 0}, 1.0f, white);
    r.setScene(std::move(scene));
    r.setOutputOptions(OutputOptions{OutputLinearity::GammaCorrected});
    r.setDebug(DebugOptions::UVChecker);
    r.render();
    r.createPixels();
    const uint32_t *px = r.getPixels();
    int bad_rim = 0, bad_inside = 0;
    for (int i = 0; i < res.height; ++i)
        for (int j = 0; j < res.width; ++j) {
            const uint32_t p = px[i * res.width + j];
            const float cr = (p & 0xff) / 255.0f, cg = ((p >> 8) & 0xff) / 255.0f, cb = ((p >> 16) & 0xff) / 255.0f;
            const bool rim = i < 6 || j < 6 || i >= res.height - 6 || j >= res.width - 6;
            if (rim && (cr != 0 || cg != 0 || cb != 0)) ++bad_rim;
            if (!rim && (cr < 0.65f || cg < 0.6f || cb < 0.5f)) ++bad_inside;
        }
    CHECK(bad_rim == 0);
    CHECK(bad_inside == 0);
    r.saveImage(g_dir / "debug_square.png");
    CHECK(std::filesystem::file_size(g_dir / "debug_square.png") > (uintmax_t)res.area() * 4);
}

// N progressive render() calls equal one dr_render call of N samples.
void test_renderer_progressive_equals_one_call()
{
    const Size2i res{64, 48};
    Renderer r(res);
    const Camera cam = makeCamera(res, 2.0f, 0.05f);
    r.setCamera(cam);
    Scene scene;
    const int white = addDiffuse(scene, Vec4{0, 0, 0, 0}, Vec4{0.75f, 0.75f, 0.75f, 0});
    const int red = addDiffuse(scene, Vec4{0, 0, 0, 0}, Vec4{0.6f, 0.1f, 0.1f, 0});
    const int light = addDiffuse(scene, Vec4{15, 15, 15, 0}, Vec4{0, 0, 0, 0});
    TransparentMaterial glass{};
    glass.inside_medium = Medium{1.5f};
    scene.materials.push_back(glass);
    const int glass_id = (int)scene.materials.size() - 1;
    addQuad(scene, Vec3{0, 0, 3}, Vec3{0, 0, -1}, Vec3{1, 0, 0}, 4.0f, white);
    addQuad(scene, Vec3{-1, 0, 2}, Vec3{1, 0, 0}, Vec3{0, 0, 1}, 4.0f, red);
    addQuad(scene, Vec3{0, 0.99f, 2}, Vec3{0, -1, 0}, Vec3{1, 0, 0}, 0.5f, light);
    Mesh m = tetra();
    scene.mesh_storage.push_back(convertMeshToTris(m));
    TriangleMesh tv = viewGpuTris(scene.mesh_storage.back());
    tv.material = glass_id;
    tv.setScale(Vec3{0.5f, 0.5f, 0.5f});
    tv.setPosition(Vec3{0.2f, -0.3f, 2.0f});
    scene.objects.push_back(tv);
    r.setScene(std::move(scene));
    const int N = 6;
    r.render();          // this sample is discarded by the camera change below
    r.setCamera(cam);
    for (int i = 0; i < N; ++i) r.render();
    const Vec4 *px = r.getRawPixels();
    std::vector<Vec4> got(px, px + res.area());

    // the same through the C ABI on the renderer's device scene
    dr_context *ctx = devilray::context();
    void *acc = nullptr;
    const size_t bytes = (size_t)res.area() * sizeof(Vec4);
    devilray::check(dr_device_allocate(ctx, bytes, &acc), "alloc");
    devilray::check(dr_device_zero(ctx, acc, bytes, nullptr), "zero");
    dr_camera c{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) c.transform[i * 4 + j] = cam.transform.values[i][j];
    c.focal_length = cam.intrinsics.focal_length;
    c.center[0] = cam.intrinsics.center.x;
    c.center[1] = cam.intrinsics.center.y;
    c.width = res.width;
    c.height = res.height;
    c.pixel_size[0] = c.pixel_size[1] = 0.05f;
    dr_render_config cfg{};
    cfg.max_depth = 10;
    cfg.spp = N;
    cfg.pixel_sampling = DR_PIXEL_UNIFORM_RANDOM;
    devilray::check(dr_render(r.deviceScene(), &c, &cfg, static_cast<float *>(acc), nullptr, nullptr), "render");
    std::vector<Vec4> want((size_t)res.area());
    devilray::check(dr_device_copy_to_host(ctx, want.data(), acc, bytes), "copy");
    dr_device_free(ctx, acc);
    CHECK(std::memcmp(got.data(), want.data(), bytes) == 0);
    double energy = 0;
    for (const Vec4 &v : got) energy += v.x + v.y + v.z;
    CHECK(energy > 0);
    CHECK(got[0].w == (float)N);

    // the object light table equals generateAliasTable of the reference's
    // weights A * luminance(pi E) / total
    const Scene &s = r.scene();
    std::vector<float> w(s.objects.size());
    float total = 0;
    for (size_t i = 0; i < w.size(); ++i) {
        w[i] = s.objects[i].surface_area * luminance(radiantExitance(s.materials[s.objects[i].material]));
        total += w[i];
    }
    for (float &x : w) x /= total;
    const AliasTable expect = generateAliasTable(w);
    CHECK(r.lightSampler().entries.size() == w.size());
    CHECK(std::memcmp(expect.entries.hostPtr(), r.lightSampler().entries.hostPtr(), w.size() * sizeof(AliasEntry)) == 0);
    CHECK(s.info.total_radiant_power == total);

    // clear(): the next render starts a new accumulation
    r.clear();
    r.render();
    CHECK(r.getRawPixels()[0].w == 1.0f);
    CHECK(throws([] { Renderer bad(Size2i{0, 4}); }));
    CHECK(throws([&] { r.setMaxDepth(0); }));
}

}  // namespace

// dump-mesh <obj> <out>: loadMesh, then normalizeMeshSize + generateCoarseNormals,
// written as int32 ok, then per stage int32 np, nn, nt, the float points,
// the float normals, the uint32 triangles (a.pi, a.ni, b.pi, b.ni, c.pi, c.ni)
// and the name (int32 length + bytes); ok = 0 when loadMesh throws.
int dump_mesh(const char *obj, const char *out_path)
{
    std::ofstream out(out_path, std::ios::binary);
    auto i32 = [&](int32_t v) { out.write(reinterpret_cast<const char *>(&v), 4); };
    auto stage = [&](const Mesh &m) {
        i32((int32_t)m.points.size());
        i32((int32_t)m.normals.size());
        i32((int32_t)m.triangles.size());
        out.write(reinterpret_cast<const char *>(m.points.data()), (std::streamsize)(m.points.size() * sizeof(Vec3)));
        out.write(reinterpret_cast<const char *>(m.normals.data()), (std::streamsize)(m.normals.size() * sizeof(Vec3)));
        for (const Triangle &t : m.triangles)
            for (const Vertex &v : {t.a, t.b, t.c}) {
                i32((int32_t)v.pi);
                i32((int32_t)v.ni);
            }
        i32((int32_t)m.name.size());
        out.write(m.name.data(), (std::streamsize)m.name.size());
    };
    Mesh m;
    try {
        m = loadMesh(obj);
    } catch (const std::exception &) {
        i32(0);
        return 0;
    }
    i32(1);
    stage(m);
    if (!m.points.empty()) {
        normalizeMeshSize(m);
        generateCoarseNormals(m);
        stage(m);
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 4 && std::string(argv[1]) == "dump-mesh") return dump_mesh(argv[2], argv[3]);
    const std::string which = argc > 1 ? argv[1] : "all";
    g_dir = argc > 2 ? std::filesystem::path(argv[2]) : std::filesystem::path(".");
    std::filesystem::create_directories(g_dir);
    struct Case {
        const char *name;
        bool gpu;
        std::function<void()> fn;
    };
    const std::vector<Case> cases = {
        {"obj_loader", false, test_obj_loader},
        {"mesh_utilities", false, test_mesh_utilities},
        {"png_writer", false, test_png_writer},
        {"alias_tables", true, test_alias_tables},
        {"gpu_tris", true, test_gpu_tris},
        {"renderer_analytic_planes", true, test_renderer_analytic_planes},
        {"renderer_debug_square", true, test_renderer_debug_square},
        {"renderer_progressive_equals_one_call", true, test_renderer_progressive_equals_one_call},
    };
    for (const Case &c : cases) {
        if ((which == "cpu" && c.gpu) || (which == "gpu" && !c.gpu)) continue;
        const int before = g_failed;
        try {
            c.fn();
        } catch (const std::exception &e) {
            ++g_failed;
            std::fprintf(stderr, "  FAILED %s: exception: %s\n", c.name, e.what());
        }
        std::printf("%s %s\n", g_failed == before ? "ok  " : "FAIL", c.name);
    }
    std::printf("%d checks, %d failed\n", g_checks, g_failed);
    return g_failed == 0 ? 0 : 1;
}
