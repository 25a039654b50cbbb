// batch.cu -- many images of many scenes in one wavefront schedule.
//
// The scenes of a batch are concatenated into one set of device arrays
// (hierarchies, triangle records, shading records, objects, materials, light
// tables), with node, triangle, object and material indices rebased by each
// scene's offsets; each image (job) names its hierarchy root and its first
// object. One persistent traversal launch per bounce then serves the rays of
// every scene in the wave. The schedule of a batch is fixed at creation, so the
// first dr_batch_render captures it into a CUDA graph and later calls replay
// the graph after updating the jobs' sample offsets.

#include "dr_internal.h"
#include "render_internal.h"
#include "trace_device.cuh"

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <vector>

struct dr_batch {
    dr_context *ctx = nullptr;
    uint32_t layout = 8;
    int tri_mode = DR_TRI_REFERENCE;
    uint64_t device_bytes = 0;
    // concatenated scene arrays
    dr::Bvh2Node *nodes = nullptr;
    dr::Bvh8Node *nodes8 = nullptr;
    float4 *tri_ref = nullptr, *tri_wt = nullptr;
    int32_t *prim = nullptr;
    float4 *shade = nullptr;
    dr_object *objects = nullptr;
    dr_material *materials = nullptr;
    dr_alias_entry *light_table = nullptr, *tri_tables = nullptr;
    uint32_t num_nodes = 0, num_tris = 0;
    // schedule
    std::vector<dr::RenderJob> jobs;
    std::vector<uint32_t> next_offset;
    dr::WavePlan plan;
    dr::WaveConfig wave;
    dr::WaveRunner runner;
    bool use_graph = true;
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t graph_nodes = 0;
    dr::RenderJob *h_jobs = nullptr;  // pinned staging of the job table
    cudaEvent_t done = nullptr;       // end of the last render
};

namespace dr {
namespace {

__global__ void k_rebase_nodes8(Bvh8Node *n, uint32_t count, uint32_t node_off, uint32_t tri_off)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint4 w1 = n[i].w[1];
    w1.x += node_off;
    w1.y += tri_off;
    n[i].w[1] = w1;
}

__global__ void k_rebase_nodes2(Bvh2Node *n, uint32_t count, uint32_t node_off, uint32_t tri_off)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int4 l = n[i].link;
    auto fix = [&](int32_t c) -> int32_t {
        if (c >= 0) return c + (int32_t)node_off;
        const uint32_t code = ~(uint32_t)c;
        const uint32_t first = (code >> kLeafCountBits) + tri_off, cnt = code & kMaxLeafSize;
        return ~int32_t((first << kLeafCountBits) | cnt);
    };
    l.x = fix(l.x);
    l.y = fix(l.y);
    n[i].link = l;
}

__global__ void k_rebase_prim(int32_t *prim, uint32_t count, uint32_t off)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) prim[i] += (int32_t)off;
}

// shading record 3 of a triangle holds (C.z, object, material, -) as int bits
__global__ void k_rebase_shade(float4 *shade, uint32_t count, uint32_t obj_off, uint32_t mat_off)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float4 r = shade[3 * (size_t)i + 2];
    r.y = __int_as_float(__float_as_int(r.y) + (int32_t)obj_off);
    r.z = __int_as_float(__float_as_int(r.z) + (int32_t)mat_off);
    shade[3 * (size_t)i + 2] = r;
}

__global__ void k_rebase_objects(dr_object *o, uint32_t count, uint32_t tri_off, uint32_t mat_off)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    o[i].tri_begin += tri_off;
    o[i].material += (int32_t)mat_off;
}

unsigned blocks_for(uint32_t n) { return (n + 255) / 256; }

template <typename T>
cudaError_t copy_d2d(T *dst, const T *src, size_t count, cudaStream_t st)
{
    if (count == 0 || !src) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToDevice, st);
}

void release(dr_batch *b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    if (b->done) cudaEventDestroy(b->done);
    cudaFreeHost(b->h_jobs);
    cudaFree(b->nodes);
    cudaFree(b->nodes8);
    cudaFree(b->tri_ref);
    cudaFree(b->tri_wt);
    cudaFree(b->prim);
    cudaFree(b->shade);
    cudaFree(b->objects);
    cudaFree(b->materials);
    cudaFree(b->light_table);
    cudaFree(b->tri_tables);
    delete b;
}

struct SceneSlot {
    uint32_t node_off, tri_off, obj_off, mat_off;
};

}  // namespace
}  // namespace dr

using namespace dr;

extern "C" {

dr_status dr_batch_create(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_batch_config *cfg,
                          dr_batch **out)
{
    DR_CHECK_ARG(ctx && out && (njobs == 0 || jobs), "dr_batch_create: NULL argument");
    *out = nullptr;
    DR_CHECK_ARG(njobs > 0, "dr_batch_create: no jobs");
    DR_CHECK_ARGF(!cfg || cfg->stack == 0 || cfg->stack == 4 || cfg->stack == 8 || cfg->stack == 16,
                  "dr_batch_create: stack must be 0, 4, 8 or 16 (got %u)", cfg ? cfg->stack : 0u);
    DR_CUDA(cudaSetDevice(ctx->device));
    // distinct scenes in first-use order
    std::vector<const dr_scene *> scenes;
    std::map<const dr_scene *, uint32_t> index;
    for (uint32_t j = 0; j < njobs; ++j) {
        const dr_job &J = jobs[j];
        DR_CHECK_ARGF(J.scene && J.accum_dev, "dr_batch_create: job %u without scene or accumulation buffer", j);
        DR_CHECK_ARGF(J.scene->ctx == ctx, "dr_batch_create: job %u scene belongs to another context", j);
        DR_CHECK_ARGF(J.camera.width > 0 && J.camera.height > 0 &&
                         (uint64_t)J.camera.width * (uint64_t)J.camera.height < (1ull << 27),
                     "dr_batch_create: job %u image size", j);
        DR_CHECK_ARGF(J.config.max_depth >= 1 && J.config.max_depth <= (uint32_t)kMaxRenderDepth,
                     "dr_batch_create: job %u max_depth must be in [1, 63]", j);
        DR_CHECK_ARGF(J.config.debug == DR_DEBUG_OFF, "dr_batch_create: job %u: debug views are not batched", j);
        DR_CHECK_ARG(J.config.tri_mode == jobs[0].config.tri_mode, "dr_batch_create: jobs differ in tri_mode");
        DR_CHECK_ARGF((reinterpret_cast<uintptr_t>(J.accum_dev) & 15) == 0,
                     "dr_batch_create: job %u accum must be 16-byte aligned", j);
        if (!index.count(J.scene)) {
            index[J.scene] = (uint32_t)scenes.size();
            scenes.push_back(J.scene);
        }
    }
    const uint32_t layout = scenes[0]->layout;
    for (const dr_scene *s : scenes)
        DR_CHECK_ARG(s->layout == layout, "dr_batch_create: scenes differ in hierarchy layout");

    auto *b = new (std::nothrow) dr_batch;
    if (!b) return fail(DR_ERR_OUT_OF_MEMORY, "dr_batch_create: host allocation failed");
    b->ctx = ctx;
    b->layout = layout;
    b->tri_mode = jobs[0].config.tri_mode;
    b->runner.ctx = ctx;
    if (cfg) {
        if (cfg->wave_paths) b->wave.wave_paths = cfg->wave_paths;
        if (cfg->streams) b->wave.streams = cfg->streams;
        b->wave.chunk = cfg->chunk;
        b->use_graph = cfg->use_graph != 0;
        if (cfg->stack) b->wave.stack = cfg->stack;
    }

    // offsets
    std::vector<SceneSlot> slots(scenes.size());
    uint64_t nodes = 0, tris = 0, objs = 0, mats = 0;
    for (size_t i = 0; i < scenes.size(); ++i) {
        slots[i] = SceneSlot{(uint32_t)nodes, (uint32_t)tris, (uint32_t)objs, (uint32_t)mats};
        nodes += scenes[i]->num_nodes;
        tris += scenes[i]->num_tris;
        objs += scenes[i]->num_objects;
        mats += scenes[i]->num_materials;
    }
    const uint64_t max_tris = layout == 2 ? kMaxTriangles : 0xffffffffull;
    if (tris > max_tris || nodes > 0x7fffffffull || objs > 0x7fffffffull) {
        release(b);
        return fail(DR_ERR_TOO_LARGE, "dr_batch_create: batch too large (%llu triangles)", (unsigned long long)tris);
    }
    b->num_nodes = (uint32_t)nodes;
    b->num_tris = (uint32_t)tris;

    auto alloc = [&](auto **p, uint64_t count) -> cudaError_t {
        if (count == 0) return cudaSuccess;
        const size_t bytes = count * sizeof(**p);
        b->device_bytes += bytes;
        return dev_malloc(reinterpret_cast<void **>(p), bytes);
    };
    cudaError_t e = cudaSuccess;
    if (layout == 8) e = alloc(&b->nodes8, nodes);
    else e = alloc(&b->nodes, nodes);
    if (e == cudaSuccess) e = alloc(&b->tri_ref, tris * 3);
    if (e == cudaSuccess) e = alloc(&b->tri_wt, tris * 3);
    if (e == cudaSuccess) e = alloc(&b->prim, tris);
    if (e == cudaSuccess) e = alloc(&b->shade, tris * 3);
    if (e == cudaSuccess) e = alloc(&b->objects, objs);
    if (e == cudaSuccess) e = alloc(&b->materials, std::max<uint64_t>(mats, 1));
    if (e == cudaSuccess) e = alloc(&b->light_table, std::max<uint64_t>(objs, 1));
    if (e == cudaSuccess) e = alloc(&b->tri_tables, std::max<uint64_t>(tris, 1));
    if (e == cudaSuccess) e = cudaMemset(b->light_table, 0, std::max<uint64_t>(objs, 1) * sizeof(dr_alias_entry));
    if (e == cudaSuccess) e = cudaMemset(b->tri_tables, 0, std::max<uint64_t>(tris, 1) * sizeof(dr_alias_entry));
    if (e != cudaSuccess) {
        release(b);
        return cuda_fail(e, "dr_batch_create: allocation");
    }
    cudaStream_t st = nullptr;
    for (size_t i = 0; i < scenes.size() && e == cudaSuccess; ++i) {
        const dr_scene *s = scenes[i];
        const SceneSlot &o = slots[i];
        if (layout == 8) e = copy_d2d(b->nodes8 + o.node_off, s->d_nodes8, s->num_nodes, st);
        else e = copy_d2d(b->nodes + o.node_off, s->d_nodes, s->num_nodes, st);
        if (e == cudaSuccess) e = copy_d2d(b->tri_ref + 3 * (size_t)o.tri_off, s->d_tri_ref, 3 * (size_t)s->num_tris, st);
        if (e == cudaSuccess) e = copy_d2d(b->tri_wt + 3 * (size_t)o.tri_off, s->d_tri_wt, 3 * (size_t)s->num_tris, st);
        if (e == cudaSuccess) e = copy_d2d(b->prim + o.tri_off, s->d_prim, s->num_tris, st);
        if (e == cudaSuccess) e = copy_d2d(b->shade + 3 * (size_t)o.tri_off, s->d_shade, 3 * (size_t)s->num_tris, st);
        if (e == cudaSuccess) e = copy_d2d(b->objects + o.obj_off, s->d_objects, s->num_objects, st);
        if (e == cudaSuccess) e = copy_d2d(b->materials + o.mat_off, s->d_materials, s->num_materials, st);
        if (e == cudaSuccess && s->d_light_table)
            e = copy_d2d(b->light_table + o.obj_off, s->d_light_table, s->num_objects, st);
        if (e == cudaSuccess && s->d_tri_tables)
            e = copy_d2d(b->tri_tables + o.tri_off, s->d_tri_tables, s->num_tris, st);
        if (e != cudaSuccess) break;
        if (s->num_nodes) {
            if (layout == 8) k_rebase_nodes8<<<blocks_for(s->num_nodes), 256, 0, st>>>(b->nodes8 + o.node_off, s->num_nodes, o.node_off, o.tri_off);
            else k_rebase_nodes2<<<blocks_for(s->num_nodes), 256, 0, st>>>(b->nodes + o.node_off, s->num_nodes, o.node_off, o.tri_off);
        }
        if (s->num_tris) {
            k_rebase_prim<<<blocks_for(s->num_tris), 256, 0, st>>>(b->prim + o.tri_off, s->num_tris, o.tri_off);
            k_rebase_shade<<<blocks_for(s->num_tris), 256, 0, st>>>(b->shade + 3 * (size_t)o.tri_off, s->num_tris, o.obj_off, o.mat_off);
        }
        if (s->num_objects)
            k_rebase_objects<<<blocks_for(s->num_objects), 256, 0, st>>>(b->objects + o.obj_off, s->num_objects, o.tri_off, o.mat_off);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        release(b);
        return cuda_fail(e, "dr_batch_create: merge");
    }

    // jobs
    b->jobs.resize(njobs);
    b->next_offset.resize(njobs);
    for (uint32_t j = 0; j < njobs; ++j) {
        const dr_job &J = jobs[j];
        const dr_scene *s = J.scene;
        const SceneSlot &o = slots[index[s]];
        RenderJob rj = make_job(s, &J.camera, &J.config, J.accum_dev, J.casts_dev);
        rj.root = s->num_nodes ? o.node_off : kNoRoot;
        rj.obj_base = o.obj_off;
        b->jobs[j] = rj;
        b->next_offset[j] = J.config.sample_offset;
    }
    b->plan = plan_waves(b->jobs, b->wave.wave_paths);
    if ((e = cudaMallocHost(&b->h_jobs, njobs * sizeof(RenderJob))) != cudaSuccess) {
        release(b);
        return cuda_fail(e, "dr_batch_create: pinned job table");
    }
    if ((e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming)) != cudaSuccess) {
        release(b);
        return cuda_fail(e, "dr_batch_create: stream");
    }
    dr_status r = b->runner.prepare(b->jobs, b->plan, b->wave, b->capture_stream);
    if (r == DR_OK && cudaStreamSynchronize(b->capture_stream) != cudaSuccess) r = cuda_fail(cudaGetLastError(), "dr_batch_create");
    if (r != DR_OK) {
        release(b);
        return r;
    }
    *out = b;
    return DR_OK;
}

dr_status dr_batch_render(dr_batch *b, const uint32_t *sample_offsets, void *stream)
{
    DR_CHECK_ARG(b != nullptr, "dr_batch_render: batch is NULL");
    DR_CUDA(cudaSetDevice(b->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    const uint32_t njobs = (uint32_t)b->jobs.size();
    for (uint32_t j = 0; j < njobs; ++j) {
        b->jobs[j].sample_offset = sample_offsets ? sample_offsets[j] : b->next_offset[j];
        b->next_offset[j] = b->jobs[j].sample_offset + b->jobs[j].spp;
    }
    const SceneArrays sc = [&] {
        SceneArrays a{};
        a.trace.nodes = b->nodes;
        a.trace.nodes8 = b->nodes8;
        a.trace.layout = (int)b->layout;
        a.trace.tri_ref = b->tri_ref;
        a.trace.tri_wt = b->tri_wt;
        a.trace.prim = b->prim;
        a.trace.num_nodes = b->num_nodes;
        a.trace.error = b->ctx->d_error;
        a.trace.stack_limit = b->ctx->stack_limit;
        a.shade = b->shade;
        a.objects = b->objects;
        a.materials = b->materials;
        a.light_table = b->light_table;
        a.tri_tables = b->tri_tables;
        return a;
    }();
    // the previous render of this batch has finished reading the job table and
    // its pinned staging (renders of one batch are serialised)
    DR_CUDA(cudaEventSynchronize(b->done));
    std::memcpy(b->h_jobs, b->jobs.data(), njobs * sizeof(RenderJob));
    DR_CUDA(cudaMemcpyAsync(b->runner.d_jobs, b->h_jobs, njobs * sizeof(RenderJob), cudaMemcpyHostToDevice, st));
    if (!b->use_graph) {
        const dr_status r = b->runner.enqueue(sc, b->plan, b->wave, b->tri_mode, st);
        if (r == DR_OK) DR_CUDA(cudaEventRecord(b->done, st));
        return r;
    }
    if (!b->exec) {
        // capture the schedule once on the batch's own stream
        DR_CUDA(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
        const dr_status r = b->runner.enqueue(sc, b->plan, b->wave, b->tri_mode, b->capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b->capture_stream, &g);
        if (r != DR_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "dr_batch_render: capture");
        b->graph = g;
        DR_CUDA(cudaGraphGetNodes(g, nullptr, &b->graph_nodes));
        DR_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    }
    DR_CUDA(cudaGraphLaunch(b->exec, st));
    DR_CUDA(cudaEventRecord(b->done, st));
    return DR_OK;
}

dr_status dr_batch_get_info(const dr_batch *b, dr_batch_info *info)
{
    DR_CHECK_ARG(b && info, "dr_batch_get_info: NULL argument");
    info->num_jobs = (uint32_t)b->jobs.size();
    info->num_waves = (uint32_t)b->plan.wave_slots.size();
    info->max_wave_paths = b->plan.max_slots;
    info->layout = b->layout;
    info->graph_nodes = (uint64_t)b->graph_nodes;
    uint64_t paths = 0;
    for (const RenderJob &j : b->jobs) paths += (uint64_t)j.npix * j.spp;
    info->paths_per_render = paths;
    info->device_bytes = b->device_bytes;
    info->streams = std::min<uint32_t>(b->wave.streams, (uint32_t)kMaxWaveStreams);
    info->chunk = b->wave.chunk;
    return DR_OK;
}

dr_status dr_batch_destroy(dr_batch *b)
{
    if (!b) return DR_OK;
    cudaSetDevice(b->ctx->device);
    cudaDeviceSynchronize();
    release(b);
    return DR_OK;
}

dr_status dr_render_batch(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_batch_config *cfg,
                          void *stream)
{
    dr_batch *b = nullptr;
    dr_batch_config c = cfg ? *cfg : dr_batch_config{};
    c.use_graph = 0;  // a single render gains nothing from a graph
    dr_status r = dr_batch_create(ctx, jobs, njobs, &c, &b);
    if (r != DR_OK) return r;
    r = dr_batch_render(b, nullptr, stream);
    if (r == DR_OK) DR_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    dr_batch_destroy(b);
    return r;
}

}  // extern "C"
