// render_internal.h -- the wavefront renderer shared by dr_render (one image)
// and dr_batch (many images of many scenes in one schedule).
//
// A render is a list of jobs (an image, its camera, its hierarchy root in the
// scene arrays, its light tables, its sample range and output buffers) and a
// plan that packs the jobs' samples into waves of path slots. A wave holds whole
// samples: segment (job, first sample, count) covers count x npix consecutive
// slots. Waves run on up to kMaxWaveStreams streams; each wave's colours are
// added to its jobs' images by one ordered pass, chained from wave to wave, so
// every pixel receives its samples in sample order.
#pragma once

#include "dr_internal.h"
#include "trace_kernels.cuh"

#include <vector>

namespace dr {

constexpr int kMaxWaveStreams = 3;
constexpr int kMaxRenderDepth = 63;

// One image of a render (device resident; 16-byte aligned fields first).
struct RenderJob {
    float4 *accum;             // float4 per pixel: rgb sums, sample count in w
    uint32_t *pix_casts;       // path-ray casts per pixel, may be NULL
    float m[12];               // camera-to-world rows 0..2
    float focal, cx, cy, psx, psy;
    int32_t width, height, pixel_sampling;
    uint32_t npix;
    uint32_t root;             // hierarchy root in the scene arrays, kNoRoot when empty
    uint32_t obj_base;         // first object (and first light-table entry) of the job
    uint32_t num_objects;
    float total_power;
    int32_t lights;
    uint32_t seed_lo, seed_hi;
    uint32_t sample_offset;    // absolute index of the job's sample 0 in this call
    uint32_t max_depth;
    uint32_t spp;              // samples of this call
};

struct WaveSegment {
    uint32_t job;
    uint32_t slot_begin;       // first slot in the wave
    uint32_t pix_begin;        // first accumulation thread of the segment in the wave
    uint32_t npix;
    uint32_t sample_rel;       // first sample, relative to the job's sample_offset
    uint32_t nsamples;
};

struct WavePlan {
    std::vector<WaveSegment> segs;     // segments of all waves, wave by wave
    std::vector<uint32_t> wave_first;  // first segment of wave w; size nwaves + 1
    std::vector<uint32_t> wave_slots;  // path slots of wave w
    std::vector<uint32_t> wave_pix;    // accumulation threads of wave w
    uint32_t max_slots = 0;
    uint32_t max_depth = 0;
};

// Scene arrays the kernels read (one scene, or the concatenation of a batch).
struct SceneArrays {
    TraceArgs trace;
    const float4 *shade;
    const dr_object *objects;
    const dr_material *materials;
    const dr_alias_entry *light_table;
    const dr_alias_entry *tri_tables;
};

// Tunables of the wave schedule.
struct WaveConfig {
    // target slots per wave (at least one sample of the largest job); many-light
    // 1080p, 64 spp: 2^21 -> 188 ms, 2^22 -> 163 ms
    uint32_t wave_paths = 1u << 22;
    uint32_t streams = kMaxWaveStreams;
    uint32_t chunk = 0;              // rays per warp fetch of the persistent traversal, 0 = adaptive
    uint32_t stack = 8;              // shared-memory stack entries per lane: 4, 8 or 16
};

// Path guiding of a render: the network, the mixture probability, and online
// training after every wave (steps x batch rows of the newest samples).
struct GuideRun {
    dr_guide *guide = nullptr;
    float alpha = 0.5f;
    bool train = true;
    uint32_t batch = 16384;
    uint32_t steps = 4;
    uint32_t budget = 0;  // total Adam steps of the network after which training stops, 0 = none
    uint32_t streams = 1; // concurrent waves; training of the waves runs one after another
    uint32_t target = 0;  // training target: 0 radiance, 1 log(1 + radiance)
    uint32_t bounces = 64;  // bounces b < bounces are guided
    uint32_t alpha_ramp = 0;  // alpha rises linearly over the network's first alpha_ramp steps, 0 = none
};

// Packs the samples of `jobs` (their npix and spp) into waves.
WavePlan plan_waves(const std::vector<RenderJob> &jobs, uint32_t wave_paths);

// Device state of a wave schedule: per-stream slot buffers, streams, events,
// the job table and the segment table. Grown on demand (outside any capture).
struct WaveRunner {
    dr_context *ctx = nullptr;
    void *d_wave[kMaxWaveStreams] = {};
    size_t wave_bytes[kMaxWaveStreams] = {};
    cudaStream_t stream[kMaxWaveStreams] = {};
    cudaEvent_t acc_done[kMaxWaveStreams] = {};
    cudaEvent_t fork = nullptr;
    RenderJob *d_jobs = nullptr;
    size_t jobs_capacity = 0;
    WaveSegment *d_segs = nullptr;
    size_t segs_capacity = 0;
    bool guided = false;              // slot buffers carry the guiding state
    void *d_train = nullptr;          // training ring (guided renders)
    uint32_t train_cap = 0;
    unsigned long long *d_totals = nullptr;  // rays of the last schedule: path, shadow

    ~WaveRunner();
    // Allocates buffers for `plan` and uploads jobs and segments (on `st`).
    dr_status prepare(const std::vector<RenderJob> &jobs, const WavePlan &plan, const WaveConfig &cfg,
                      cudaStream_t st, const GuideRun *guide = nullptr);
    // Enqueues the whole schedule on `st` (forks to the wave streams and joins
    // back). Capturable into a CUDA graph: no allocation, no host sync.
    dr_status enqueue(const SceneArrays &scene, const WavePlan &plan, const WaveConfig &cfg, int tri_mode,
                      cudaStream_t st, const GuideRun *guide = nullptr);
};

SceneArrays scene_arrays(const dr_scene *s);

// Job of one image of scene `s` (root 0, objects from 0).
RenderJob make_job(const dr_scene *s, const dr_camera *cam, const dr_render_config *cfg, float *accum,
                   uint32_t *casts);

}  // namespace dr
