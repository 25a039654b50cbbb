// autotune.cpp -- picks the hierarchy width and the wavefront schedule
// (paths per wave, concurrent waves, traversal fetch size, shared-memory
// stack depth) by timing short probe renders on the device.
//
// The search is coordinate descent from the defaults (8-wide, 2^22 paths per
// wave, 3 streams, adaptive fetch, 8 stack entries): each knob in turn is set
// to the fastest of its candidates with the others fixed, where a candidate
// must beat the incumbent by more than 2 %. Every candidate renders the same
// samples, and the images do not depend on the schedule, so the probes differ
// only in time. Timing: CUDA events on the probe stream, one warm-up render,
// then the minimum over `reps` renders.

#include "dr_internal.h"

#include <algorithm>
#include <vector>

namespace dr {
namespace {

struct Knobs {
    uint32_t layout, wave_paths, streams, chunk, stack;
};

struct Probe {
    cudaStream_t stream = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    ~Probe()
    {
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (stream) cudaStreamDestroy(stream);
    }
};

void record(dr_autotune_result *out, const Knobs &k, float ms)
{
    if (out->num_candidates < sizeof(out->candidates) / sizeof(out->candidates[0]))
        out->candidates[out->num_candidates++] =
            dr_autotune_candidate{k.layout, k.wave_paths, k.streams, k.chunk, k.stack, ms};
}

// Times `run` (one render enqueued on the probe stream): warm-up, then min over reps.
template <class F>
dr_status time_probe(Probe &p, uint32_t reps, F &&run, float &ms)
{
    dr_status st = run();
    if (st != DR_OK) return st;
    DR_CUDA(cudaStreamSynchronize(p.stream));
    ms = 1e30f;
    for (uint32_t r = 0; r < reps; ++r) {
        DR_CUDA(cudaEventRecord(p.t0, p.stream));
        st = run();
        if (st != DR_OK) return st;
        DR_CUDA(cudaEventRecord(p.t1, p.stream));
        DR_CUDA(cudaEventSynchronize(p.t1));
        float t = 0.0f;
        DR_CUDA(cudaEventElapsedTime(&t, p.t0, p.t1));
        ms = std::min(ms, t);
    }
    return DR_OK;
}

const uint32_t kWaveCandidates[] = {1u << 19, 1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24};
const uint32_t kStreamCandidates[] = {1, 2, 3};
const uint32_t kChunkCandidates[] = {0, 32, 64, 128};
const uint32_t kStackCandidates[] = {8, 4, 16};

// A candidate replaces the incumbent only when its probe is faster by more
// than this fraction: probes of nearly equal schedules differ by about 1 %
// from run to run, and a near tie once moved a 64-scene batch from 3 to 2
// streams and 8 to 16 stack entries (probe 5.96 -> 5.97 ms) and its full
// render from 0.135 to 0.150 s.
constexpr float kSwitchMargin = 0.02f;
inline bool clearly_faster(float ms, float incumbent_ms) { return ms < incumbent_ms * (1.0f - kSwitchMargin); }

uint32_t &knob_ref(Knobs &k, int knob)
{
    return knob == 0 ? k.wave_paths : knob == 1 ? k.streams : knob == 2 ? k.chunk : k.stack;
}

// Coordinate descent over wave size, streams, fetch size and stack depth for
// a fixed layout.
template <class Measure>
dr_status descend(Knobs &best, float &best_ms, Measure &&measure)
{
    for (int knob = 0; knob < 4; ++knob) {
        const uint32_t *cand = knob == 0   ? kWaveCandidates
                               : knob == 1 ? kStreamCandidates
                               : knob == 2 ? kChunkCandidates
                                           : kStackCandidates;
        const int n = knob == 0 ? 6 : knob == 1 ? 3 : knob == 2 ? 4 : 3;
        if (knob >= 2 && best.layout != 8) break;  // fetch size and stack belong to the persistent 8-wide kernels
        Knobs winner = best;
        for (int i = 0; i < n; ++i) {
            Knobs k = best;
            knob_ref(k, knob) = cand[i];
            if (knob_ref(k, knob) == knob_ref(best, knob)) continue;
            float ms = 0.0f;
            const dr_status st = measure(k, ms);
            if (st != DR_OK) return st;
            if (clearly_faster(ms, best_ms)) {
                best_ms = ms;
                winner = k;
            }
        }
        best = winner;
    }
    return DR_OK;
}

}  // namespace
}  // namespace dr

using namespace dr;

extern "C" {

dr_status dr_autotune(dr_context *ctx, const dr_scene_desc *desc, const dr_camera *cam, const dr_render_config *cfg,
                      const dr_autotune_config *tc, dr_autotune_result *out)
{
    DR_CHECK_ARG(ctx && desc && cam && cfg && out, "dr_autotune: NULL argument");
    DR_CHECK_ARG(cfg->debug == DR_DEBUG_OFF, "dr_autotune: debug views are not tuned");
    DR_CHECK_ARG(cam->width > 0 && cam->height > 0, "dr_autotune: empty image");
    DR_CUDA(cudaSetDevice(ctx->device));
    *out = dr_autotune_result{};
    const uint32_t probe_spp = tc && tc->probe_spp ? tc->probe_spp : std::max<uint32_t>(1, std::min<uint32_t>(cfg->spp, 2));
    const uint32_t reps = tc && tc->reps ? tc->reps : 2;
    std::vector<uint32_t> layouts = {8};
    if (!tc || tc->try_layouts) layouts.push_back(2);

    Probe p;
    DR_CUDA(cudaStreamCreateWithFlags(&p.stream, cudaStreamNonBlocking));
    DR_CUDA(cudaEventCreate(&p.t0));
    DR_CUDA(cudaEventCreate(&p.t1));
    const size_t npix = (size_t)cam->width * (size_t)cam->height;
    void *accum = nullptr;
    dr_status st = dr_device_allocate(ctx, npix * 16, &accum);
    if (st != DR_OK) return st;

    Knobs best{8, 1u << 22, 3, 0, 8};
    float best_ms = 1e30f;
    dr_scene *scenes[2] = {nullptr, nullptr};
    auto measure_on = [&](dr_scene *s, const Knobs &k, float &ms) -> dr_status {
        dr_render_config c = *cfg;
        c.spp = probe_spp;
        c.sample_offset = 0;
        c.wave_paths = k.wave_paths;
        c.streams = k.streams;
        c.chunk = k.chunk;
        c.stack = k.stack;
        const dr_status r = time_probe(p, reps, [&] { return dr_render(s, cam, &c, static_cast<float *>(accum), nullptr, p.stream); }, ms);
        if (r == DR_OK) record(out, k, ms);
        return r;
    };
    for (size_t li = 0; li < layouts.size() && st == DR_OK; ++li) {
        dr_build_config bc{};
        bc.layout = layouts[li];
        if (tc) bc.max_leaf_size = tc->max_leaf_size;
        st = dr_scene_create(ctx, desc, &bc, &scenes[li]);
        if (st != DR_OK) break;
        Knobs k = best;
        k.layout = layouts[li];
        float ms = 0.0f;
        st = measure_on(scenes[li], k, ms);
        if (st == DR_OK && (li == 0 || clearly_faster(ms, best_ms))) {
            best_ms = ms;
            best = k;
        }
    }
    if (st == DR_OK) {
        dr_scene *s = scenes[best.layout == 8 ? 0 : 1];
        st = descend(best, best_ms, [&](const Knobs &k, float &ms) { return measure_on(s, k, ms); });
    }
    for (dr_scene *s : scenes) dr_scene_destroy(s);
    dr_device_free(ctx, accum);
    if (st != DR_OK) return st;
    out->layout = best.layout;
    out->wave_paths = best.wave_paths;
    out->streams = best.streams;
    out->chunk = best.chunk;
    out->stack = best.stack;
    out->best_ms = best_ms;
    return DR_OK;
}

dr_status dr_autotune_batch(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_autotune_config *tc,
                            dr_autotune_result *out)
{
    DR_CHECK_ARG(ctx && jobs && njobs && out, "dr_autotune_batch: NULL argument");
    DR_CUDA(cudaSetDevice(ctx->device));
    *out = dr_autotune_result{};
    const uint32_t reps = tc && tc->reps ? tc->reps : 2;
    const uint32_t probe_spp = tc && tc->probe_spp ? tc->probe_spp : 1;
    Probe p;
    DR_CUDA(cudaStreamCreateWithFlags(&p.stream, cudaStreamNonBlocking));
    DR_CUDA(cudaEventCreate(&p.t0));
    DR_CUDA(cudaEventCreate(&p.t1));
    // probe jobs: the same images into scratch buffers, probe_spp samples each
    std::vector<dr_job> probe(jobs, jobs + njobs);
    std::vector<void *> scratch(njobs, nullptr);
    dr_status st = DR_OK;
    for (uint32_t j = 0; j < njobs && st == DR_OK; ++j) {
        const size_t npix = (size_t)jobs[j].camera.width * (size_t)jobs[j].camera.height;
        st = dr_device_allocate(ctx, npix * 16, &scratch[j]);
        probe[j].accum_dev = static_cast<float *>(scratch[j]);
        probe[j].casts_dev = nullptr;
        probe[j].config.spp = probe_spp;
    }
    Knobs best{jobs[0].scene->layout, 1u << 22, 3, 0, 8};
    float best_ms = 1e30f;
    auto measure = [&](const Knobs &k, float &ms) -> dr_status {
        dr_batch_config bc{k.wave_paths, k.streams, k.chunk, 0, k.stack};
        dr_batch *b = nullptr;
        dr_status r = dr_batch_create(ctx, probe.data(), njobs, &bc, &b);
        if (r != DR_OK) return r;
        r = time_probe(p, reps, [&] { return dr_batch_render(b, nullptr, p.stream); }, ms);
        dr_batch_destroy(b);
        if (r == DR_OK) record(out, k, ms);
        return r;
    };
    if (st == DR_OK) st = measure(best, best_ms);
    if (st == DR_OK) st = descend(best, best_ms, measure);
    for (void *q : scratch) dr_device_free(ctx, q);
    if (st != DR_OK) return st;
    out->layout = best.layout;
    out->wave_paths = best.wave_paths;
    out->streams = best.streams;
    out->chunk = best.chunk;
    out->stack = best.stack;
    out->best_ms = best_ms;
    return DR_OK;
}

}  // extern "C"
