// Renderer.hpp -- progressive path-tracing renderer (include/Renderer.hpp of the
// reference) over the GB300 library: each render() adds one sample per pixel
// through dr_render (wavefront path tracer, Philox random numbers indexed by
// pixel and sample), tonemaps on the device (dr_tonemap) and copies the 8-bit
// pixels to the host. Setters that change the image (camera, debug view, pixel
// sampling, depth, seed) restart the accumulation on the next render().
#pragma once

#include "Buffers.hpp"
#include "DebugOptions.hpp"
#include "RunningAverage.hpp"
#include "tracing/Camera.hpp"
#include "tracing/DistributionSamplers.hpp"
#include "tracing/OutputOptions.hpp"
#include "tracing/PixelSampling.hpp"
#include "tracing/Scene.hpp"
#include "tracing/TriangleMesh.hpp"
#include "devilray_gb300.h"

#include <cstdint>
#include <filesystem>
#include <mutex>
#include <vector>

class Renderer
{
public:
    explicit Renderer(Size2i resolution);
    ~Renderer();
    Renderer(const Renderer &) = delete;
    Renderer &operator=(const Renderer &) = delete;

    const Buffers &getBuffers() const { return m_buffers; }
    float getMeanRenderTimes() const { return (float)m_renderTimes.mean(); }
    uint64_t getTotalCasts() const { return m_totalCasts; }

    void setDebug(DebugOptions dbg);
    void setCamera(Camera cam);
    void setScene(Scene scn)
    {
        m_scene = std::move(scn);
        calculateLightWeights();
    }
    void setPixelSampling(PixelSampling sampling);
    void setOutputOptions(OutputOptions options);

    void render();
    void clear();

    void createPixels();
    void saveImage(const std::filesystem::path &path);

    const uint32_t *getPixels();
    const Vec4 *getRawPixels();

    // Builds the device scene of the current objects (world-space soup,
    // hierarchy, light tables) and reads its object light table back.
    void calculateLightWeights();

    // Extensions: path vertices per sample (the reference fixes 10), the
    // Philox key, and the device scene.
    void setMaxDepth(int depth);
    void setSeed(uint64_t seed);
    dr_scene *deviceScene() const { return m_deviceScene; }
    const AliasTable &lightSampler() const { return m_light_sampler; }
    const Scene &scene() const { return m_scene; }

private:
    Buffers m_buffers;
    uint64_t m_totalCasts = 0;

    Camera m_camera{};
    DebugOptions m_debug = DebugOptions::Off;
    OutputOptions m_output_options{OutputLinearity::GammaCorrected};
    PixelSampling m_pixel_sampling = PixelSampling::UniformRandom;
    Size2i m_resolution;
    AliasTable m_light_sampler;

    std::vector<uint32_t> m_pixels;
    std::vector<uint32_t> m_displayPixels;
    DeviceArray<uint32_t> m_devicePixels;

    Scene m_scene;
    dr_scene *m_deviceScene = nullptr;

    RunningAverage m_renderTimes{20};
    uint32_t m_sampleIndex = 0;
    int m_maxDepth = Buffers::maxPathLength;
    uint64_t m_seed = 0;

    std::mutex m_renderMutex;
    std::mutex m_displayMutex;
    bool m_needsToBeCleared = false;
};
