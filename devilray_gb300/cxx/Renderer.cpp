// Renderer.cpp -- the reference's Renderer (src/Renderer.cpp) over the C ABI.
#include "Renderer.hpp"
#include "Image.hpp"

#include <cstring>
#include <numeric>
#include <stdexcept>
#include <variant>

using devilray::check;
using devilray::context;

Buffers::Buffers(Size2i resolution) : color(resolution.area(), Vec4{0, 0, 0, 0}), casts(resolution.area(), 0) {}

void Buffers::reset()
{
    std::fill(color.hostSpan().begin(), color.hostSpan().end(), Vec4{0, 0, 0, 0});
    std::fill(casts.hostSpan().begin(), casts.hostSpan().end(), 0u);
    if (color.devicePtr())
        check(dr_device_zero(context(), color.devicePtr(), color.size() * sizeof(Vec4), nullptr), "Buffers::reset");
    if (casts.devicePtr())
        check(dr_device_zero(context(), casts.devicePtr(), casts.size() * sizeof(uint32_t), nullptr), "Buffers::reset");
}

void Buffers::ensureDeviceAllocation()
{
    color.ensureDeviceAllocation();
    casts.ensureDeviceAllocation();
}

uint64_t Buffers::totalCasts() const
{
    const uint32_t *p = casts.hostPtr();
    return std::accumulate(p, p + casts.size(), uint64_t{0});
}

Renderer::Renderer(Size2i resolution)
    : m_buffers(resolution),
      m_resolution(resolution),
      m_pixels((size_t)std::max(resolution.area(), 0)),
      m_displayPixels((size_t)std::max(resolution.area(), 0), 0),
      m_devicePixels(std::max(resolution.area(), 0), 0u)
{
    if (resolution.width <= 0 || resolution.height <= 0) throw std::runtime_error("Renderer: empty resolution");
}

Renderer::~Renderer()
{
    if (m_deviceScene) dr_scene_destroy(m_deviceScene);
}

void Renderer::setDebug(DebugOptions dbg)
{
    std::scoped_lock guard{m_renderMutex};
    m_debug = dbg;
    m_needsToBeCleared = true;
}

void Renderer::setCamera(Camera cam)
{
    std::scoped_lock guard{m_renderMutex};
    m_camera = std::move(cam);
    m_needsToBeCleared = true;
}

void Renderer::clear()
{
    std::scoped_lock guard{m_renderMutex};
    m_needsToBeCleared = true;
}

void Renderer::setPixelSampling(PixelSampling sampling)
{
    std::scoped_lock guard{m_renderMutex};
    m_pixel_sampling = sampling;
    m_needsToBeCleared = true;
}

void Renderer::setOutputOptions(OutputOptions options)
{
    std::scoped_lock guard{m_renderMutex};
    m_output_options = options;
}

void Renderer::setMaxDepth(int depth)
{
    if (depth < 1 || depth > 63) throw std::runtime_error("Renderer::setMaxDepth: depth must be in [1, 63]");
    std::scoped_lock guard{m_renderMutex};
    m_maxDepth = depth;
    m_needsToBeCleared = true;
}

void Renderer::setSeed(uint64_t seed)
{
    std::scoped_lock guard{m_renderMutex};
    m_seed = seed;
    m_needsToBeCleared = true;
}

void Renderer::calculateLightWeights()
{
    // Flatten the object views into one world-space soup: object o owns a
    // contiguous triangle range; its points go through model_to_world.
    const size_t nobj = m_scene.objects.size();
    std::vector<float> positions;
    std::vector<float> tri_weight;
    std::vector<dr_object> objects(nobj);
    uint32_t begin = 0;
    for (size_t o = 0; o < nobj; ++o) {
        const TriangleMesh &m = m_scene.objects[o];
        if (m.triangle_count > 0 && (!m.points || !m.triangles))
            throw std::runtime_error("Renderer::setScene: object without geometry");
        for (int k = 0; k < m.triangle_count; ++k) {
            const Triangle &t = m.triangles[k];
            for (const Vertex *v : {&t.a, &t.b, &t.c}) {
                const Vec3 p = m.model_to_world.applyToPoint(m.points[v->pi]);
                positions.insert(positions.end(), {p.x, p.y, p.z});
            }
            // the triangle sampler's weight: the model-space area
            tri_weight.push_back(triangleArea(m.points[t.a.pi], m.points[t.b.pi], m.points[t.c.pi]));
        }
        objects[o] = dr_object{begin, (uint32_t)m.triangle_count, m.material, m.surface_area};
        begin += (uint32_t)m.triangle_count;
    }
    std::vector<dr_material> materials(m_scene.materials.size());
    for (size_t i = 0; i < materials.size(); ++i) {
        dr_material d{};
        const Material &mat = m_scene.materials[i];
        const Vec4 dc = getDebugColor(mat);
        std::memcpy(d.debug_color, &dc, sizeof(Vec4));
        if (const auto *t = std::get_if<TransparentMaterial>(&mat)) {
            d.kind = DR_MAT_DIELECTRIC;
            d.ior = t->inside_medium.ior;
        } else {
            const auto &f = std::get<DiffuseMaterial>(mat);
            d.kind = DR_MAT_DIFFUSE;
            d.ior = 1.0f;
            std::memcpy(d.emission, &f.emission, sizeof(Vec4));
            std::memcpy(d.albedo, &f.diffuse_reflectance, sizeof(Vec4));
        }
        materials[i] = d;
    }
    dr_scene_desc desc{};
    desc.positions_host = positions.data();
    desc.num_triangles = begin;
    desc.objects_host = objects.data();
    desc.num_objects = (uint32_t)nobj;
    desc.materials_host = materials.data();
    desc.num_materials = (uint32_t)materials.size();
    desc.tri_weight_host = tri_weight.data();
    // Renderer::calculateLightWeights and convertMeshToTris build their tables
    // with generateAliasTable: keep the reference's pairing (bit-identical tables)
    desc.light_tables = DR_LIGHT_TABLES_REFERENCE;
    dr_scene *scene = nullptr;
    check(dr_scene_create(context(), &desc, nullptr, &scene), "Renderer::setScene");
    if (m_deviceScene) dr_scene_destroy(m_deviceScene);
    m_deviceScene = scene;

    dr_scene_info info{};
    check(dr_scene_get_info(scene, &info), "Renderer::setScene");
    m_scene.info.total_radiant_power = info.total_radiant_power;
    uint32_t count = 0;
    check(dr_scene_get_light_table(scene, nullptr, 0, &count), "Renderer::setScene");
    m_light_sampler = AliasTable{DeviceArray<AliasEntry>((int)count, AliasEntry{})};
    if (count)
        check(dr_scene_get_light_table(scene, reinterpret_cast<dr_alias_entry *>(m_light_sampler.entries.hostPtr()),
                                       count, &count),
              "Renderer::setScene");
    std::scoped_lock guard{m_renderMutex};
    m_needsToBeCleared = true;
}

void Renderer::render()
{
    Camera camera;
    DebugOptions debug;
    PixelSampling sampling;
    int depth;
    uint64_t seed;
    {
        std::scoped_lock guard{m_renderMutex};
        if (m_needsToBeCleared) {
            m_renderTimes.reset();
            m_buffers.reset();
            m_sampleIndex = 0;
            m_needsToBeCleared = false;
        }
        camera = m_camera;
        debug = m_debug;
        sampling = m_pixel_sampling;
        depth = m_maxDepth;
        seed = m_seed;
    }
    m_buffers.ensureDeviceAllocation();
    if (!m_deviceScene) calculateLightWeights();

    Timer t;
    dr_camera cam{};
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) cam.transform[r * 4 + c] = camera.transform.values[r][c];
    cam.focal_length = camera.intrinsics.focal_length;
    cam.center[0] = camera.intrinsics.center.x;
    cam.center[1] = camera.intrinsics.center.y;
    cam.width = m_resolution.width;
    cam.height = m_resolution.height;
    cam.pixel_size[0] = camera.physical_pixel_size.width;
    cam.pixel_size[1] = camera.physical_pixel_size.height;
    dr_render_config cfg{};
    cfg.max_depth = (uint32_t)depth;
    cfg.spp = 1;
    cfg.sample_offset = m_sampleIndex;
    cfg.pixel_sampling = (int32_t)sampling;
    cfg.seed = seed;
    cfg.tri_mode = DR_TRI_REFERENCE;
    cfg.debug = (int32_t)debug;
    check(dr_render(m_deviceScene, &cam, &cfg, reinterpret_cast<float *>(m_buffers.color.devicePtr()),
                    m_buffers.casts.devicePtr(), nullptr),
          "Renderer::render");
    ++m_sampleIndex;

    createPixels();
    {
        std::scoped_lock guard{m_displayMutex};
        std::memcpy(m_displayPixels.data(), m_pixels.data(), m_pixels.size() * sizeof(uint32_t));
    }
    m_renderTimes.add(t.elapsedSeconds() * 1000.0);

    m_buffers.casts.updateHostData();
    m_totalCasts = m_buffers.totalCasts();
}

void Renderer::createPixels()
{
    m_buffers.ensureDeviceAllocation();
    m_devicePixels.ensureDeviceAllocation();
    const bool gamma = m_output_options.linearity == OutputLinearity::GammaCorrected;
    check(dr_tonemap(reinterpret_cast<const float *>(m_buffers.color.devicePtr()), m_resolution.width,
                     m_resolution.height, gamma ? 1 : 0, m_devicePixels.devicePtr(), nullptr),
          "Renderer::createPixels");
    check(dr_device_copy_to_host(context(), m_pixels.data(), m_devicePixels.devicePtr(),
                                 m_pixels.size() * sizeof(uint32_t)),
          "Renderer::createPixels");
}

void Renderer::saveImage(const std::filesystem::path &path)
{
    std::scoped_lock guard{m_displayMutex};
    savePNG(path.string(), m_displayPixels, m_resolution);
}

const uint32_t *Renderer::getPixels()
{
    std::scoped_lock guard{m_displayMutex};
    return m_displayPixels.data();
}

const Vec4 *Renderer::getRawPixels()
{
    m_buffers.ensureDeviceAllocation();
    m_buffers.color.updateHostData();
    return m_buffers.color.hostPtr();
}
