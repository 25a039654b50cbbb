// capi.cu -- the C ABI entry points: context, scene and traversal.

#include "dr_internal.h"
#include "render_internal.h"
#include "trace_kernels.cuh"
#include "alias_kernels.cuh"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace dr {

namespace {
thread_local char g_error[1024] = "";
}

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

dr_status fail(dr_status code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    return code;
}

dr_status cuda_fail(cudaError_t e, const char *what)
{
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    if (e == cudaErrorMemoryAllocation) return DR_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return DR_ERR_NO_DEVICE;
    return DR_ERR_CUDA;
}

namespace {

template <typename T>
cudaError_t upload(T **dst, const T *src, size_t count, uint64_t &bytes)
{
    *dst = nullptr;
    if (count == 0) return cudaSuccess;
    cudaError_t e = dev_malloc(reinterpret_cast<void **>(dst), sizeof(T) * count);
    if (e != cudaSuccess) return e;
    bytes += sizeof(T) * count;
    return cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
}

// Maps the context's device error word to a status and clears it.
dr_status check_error_word(dr_context *ctx, cudaStream_t s)
{
    uint32_t word = 0;
    DR_CUDA(cudaMemcpyAsync(&word, ctx->d_error, sizeof(word), cudaMemcpyDeviceToHost, s));
    DR_CUDA(cudaStreamSynchronize(s));
    if (word == 0) return DR_OK;
    DR_CUDA(cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), s));
    if (word & ERR_STACK_OVERFLOW) return fail(DR_ERR_STACK_OVERFLOW, "traversal stack overflow");
    if (word & ERR_TIMEOUT) return fail(DR_ERR_TIMEOUT, "a bounded device loop gave up");
    return fail(DR_ERR_CUDA, "device error word 0x%x", word);
}

TraceArgs trace_args(dr_scene *s)
{
    TraceArgs a{};
    a.nodes = s->d_nodes;
    a.nodes8 = s->d_nodes8;
    a.layout = (int)s->layout;
    a.tri_ref = s->d_tri_ref;
    a.tri_wt = s->d_tri_wt;
    a.prim = s->d_prim;
    a.num_nodes = s->num_nodes;
    a.error = s->ctx->d_error;
    // each launch takes its own work counter and traversal counters, so that
    // launches on different streams can overlap
    const uint32_t slot = s->ctx->work_next.fetch_add(1) % kWorkCounters;
    a.work = s->ctx->d_work + slot;
    a.counters = s->ctx->d_counters + 8 * (size_t)slot;
    a.num_sms = s->ctx->num_sms;
    a.stack_limit = s->ctx->stack_limit;
    return a;
}

}  // namespace

// Countdown of dr_debug_fail_allocation: 0 = off, k = the k-th next allocation fails.
static std::atomic<uint32_t> g_fail_alloc_after{0};

}  // namespace dr

extern "C" dr_status dr_debug_fail_allocation(uint32_t after)
{
    dr::g_fail_alloc_after.store(after, std::memory_order_relaxed);
    return DR_OK;
}

namespace dr {

cudaError_t dev_malloc_raw(void **p, size_t bytes)
{
    uint32_t k = g_fail_alloc_after.load(std::memory_order_relaxed);
    while (k != 0) {
        if (g_fail_alloc_after.compare_exchange_weak(k, k - 1, std::memory_order_relaxed)) {
            if (k == 1) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(p, bytes);
}

dr_status ensure_scratch(dr_context *ctx, size_t bytes)
{
    if (ctx->scratch_bytes >= bytes) return DR_OK;
    // Grow geometrically; the old contents need not survive.
    size_t want = std::max(bytes, ctx->scratch_bytes * 2);
    cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    DR_CUDA(dev_malloc(&ctx->scratch, want));
    ctx->scratch_bytes = want;
    return DR_OK;
}

}  // namespace dr

using namespace dr;

extern "C" {

uint32_t dr_abi_version(void) { return DR_ABI_VERSION; }

const char *dr_last_error_string(void) { return g_error; }

dr_status dr_context_create(const dr_context_config *cfg, dr_context **out)
{
    DR_CHECK_ARG(out != nullptr, "dr_context_create: out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(DR_ERR_NO_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    const int dev = cfg ? cfg->device : 0;
    DR_CHECK_ARG(dev >= 0 && dev < count, "dr_context_create: bad device ordinal");
    DR_CUDA(cudaSetDevice(dev));
    auto *ctx = new (std::nothrow) dr_context;
    if (!ctx) return fail(DR_ERR_OUT_OF_MEMORY, "host allocation failed");
    ctx->device = dev;
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess) {
        delete ctx;
        return cuda_fail(e, "cudaGetDeviceProperties");
    }
    ctx->num_sms = prop.multiProcessorCount;
    // [0, 64) error word, [128, 132) probe sink, [256, +512) work counters,
    // then 8 traversal counters per work counter
    const size_t words = 256 + kWorkCounters * sizeof(unsigned long long) * 9;
    if ((e = dev_malloc(&ctx->d_error, words)) != cudaSuccess || (e = cudaMemset(ctx->d_error, 0, words)) != cudaSuccess) {
        delete ctx;
        return cuda_fail(e, "allocation of the error word");
    }
    ctx->d_work = reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(ctx->d_error) + 256);
    ctx->d_counters = ctx->d_work + kWorkCounters;
    *out = ctx;
    return DR_OK;
}

dr_status dr_context_destroy(dr_context *ctx)
{
    if (!ctx) return DR_OK;
    cudaSetDevice(ctx->device);
    cudaFree(ctx->d_error);
    cudaFree(ctx->scratch);
    delete ctx;
    return DR_OK;
}

dr_status dr_context_check(dr_context *ctx)
{
    DR_CHECK_ARG(ctx != nullptr, "dr_context_check: ctx is NULL");
    DR_CUDA(cudaSetDevice(ctx->device));
    return check_error_word(ctx, nullptr);
}

dr_status dr_scene_create(dr_context *ctx, const dr_scene_desc *desc, const dr_build_config *cfg, dr_scene **out)
{
    DR_CHECK_ARG(ctx && desc && out, "dr_scene_create: NULL argument");
    *out = nullptr;
    const uint32_t n = desc->num_triangles;
    DR_CHECK_ARG(n == 0 || desc->positions_host, "dr_scene_create: positions_host is NULL");
    if (n >= kMaxTriangles) return fail(DR_ERR_TOO_LARGE, "dr_scene_create: %u triangles (max %u)", n, kMaxTriangles - 1);
    DR_CHECK_ARG(desc->light_tables == DR_LIGHT_TABLES_SWEEP || desc->light_tables == DR_LIGHT_TABLES_REFERENCE,
                 "dr_scene_create: unknown light_tables value");
    // largest coordinate magnitude, and whether any coordinate is not finite
    std::vector<float> part_mag(std::max(1u, std::thread::hardware_concurrency()) + 1, 0.0f);
    std::atomic<bool> non_finite{false};
    std::atomic<uint32_t> next_part{0};
    host_parallel_chunks((size_t)n * 9, size_t(1) << 20, [&](size_t b, size_t e) {
        float m = 0.0f;
        bool bad = false;
        for (size_t i = b; i < e; ++i) {
            const float a = std::fabs(desc->positions_host[i]);
            bad |= !(a <= FLT_MAX);  // NaN or infinity
            m = std::max(m, a);
        }
        part_mag[next_part.fetch_add(1)] = m;
        if (bad) non_finite = true;
    });
    if (non_finite) return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: non-finite vertex coordinate");
    float mag = 0.0f;
    for (float m : part_mag) mag = std::max(mag, m);
    if (desc->objects_host) {
        for (uint32_t o = 0; o < desc->num_objects; ++o) {
            const dr_object &ob = desc->objects_host[o];
            if ((uint64_t)ob.tri_begin + ob.tri_count > n)
                return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: object %u range out of bounds", o);
            if (ob.material < 0 || (uint32_t)ob.material >= std::max(1u, desc->num_materials))
                return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: object %u material out of range", o);
        }
    }
    DR_CUDA(cudaSetDevice(ctx->device));

    const auto t_start = std::chrono::steady_clock::now();
    BuildParams bp;
    if (cfg) {
        if (cfg->max_leaf_size) bp.max_leaf = cfg->max_leaf_size;
        if (cfg->sah_bins) bp.bins = cfg->sah_bins;
        bp.threads = cfg->threads;
    }
    const float slack = scene_slack(mag);
    const bool device_build = cfg && cfg->builder == DR_BUILD_DEVICE_LBVH;
    if (cfg && cfg->builder != DR_BUILD_HOST_SAH && cfg->builder != DR_BUILD_DEVICE_LBVH)
        return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: unknown builder");
    // the device build makes the binary layout unless the 8-wide one is asked for
    const uint32_t layout = (device_build && cfg->layout != 8) || (cfg && cfg->layout == 2) ? 2u : 8u;
    if (cfg && cfg->layout != 0 && cfg->layout != 2 && cfg->layout != 8)
        return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: layout must be 0, 2 or 8");
    if (device_build && n > 0) {
        auto *s = new (std::nothrow) dr_scene;
        if (!s) return fail(DR_ERR_OUT_OF_MEMORY, "host allocation failed");
        s->ctx = ctx;
        s->num_tris = n;
        s->layout = layout;
        s->slack = slack;
        dr_status r = build_lbvh_device(s, desc->positions_host, n, slack, layout);
        cudaError_t e = cudaSuccess;
        if (r == DR_OK && desc->materials_host && desc->num_materials) {
            if ((e = upload(&s->d_materials, desc->materials_host, desc->num_materials, s->device_bytes)) != cudaSuccess)
                r = cuda_fail(e, "dr_scene_create upload materials");
            s->num_materials = desc->num_materials;
        }
        if (r == DR_OK) r = build_render_data(s, desc);
        if (r != DR_OK) {
            dr_scene_destroy(s);
            return r;
        }
        s->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        *out = s;
        return DR_OK;
    }
    Bvh2 bvh2;
    Bvh8 bvh8;
    const std::vector<uint32_t> *order;
    if (layout == 8) {
        bvh8 = build_bvh8(desc->positions_host, n, bp, slack);
        order = &bvh8.order;
    } else {
        bvh2 = build_bvh2(desc->positions_host, n, bp, slack);
        order = &bvh2.order;
    }
    std::vector<float4> ref_rec, wt_rec;
    make_tri_records(desc->positions_host, *order, ref_rec, wt_rec);
    std::vector<int32_t> prim(order->begin(), order->end());

    auto *s = new (std::nothrow) dr_scene;
    if (!s) return fail(DR_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->ctx = ctx;
    s->num_tris = n;
    s->layout = layout;
    s->num_nodes = (uint32_t)(layout == 8 ? bvh8.nodes.size() : bvh2.nodes.size());
    s->depth = (uint32_t)(layout == 8 ? bvh8.depth : bvh2.depth);
    s->slack = slack;
    cudaError_t e = cudaSuccess;
    if ((e = (layout == 8 ? upload(&s->d_nodes8, bvh8.nodes.data(), bvh8.nodes.size(), s->device_bytes)
                          : upload(&s->d_nodes, bvh2.nodes.data(), bvh2.nodes.size(), s->device_bytes))) != cudaSuccess ||
        (e = upload(&s->d_tri_ref, ref_rec.data(), ref_rec.size(), s->device_bytes)) != cudaSuccess ||
        (e = upload(&s->d_tri_wt, wt_rec.data(), wt_rec.size(), s->device_bytes)) != cudaSuccess ||
        (e = upload(&s->d_prim, prim.data(), prim.size(), s->device_bytes)) != cudaSuccess) {
        dr_scene_destroy(s);
        return cuda_fail(e, "dr_scene_create upload");
    }
    if (desc->materials_host && desc->num_materials) {
        if ((e = upload(&s->d_materials, desc->materials_host, desc->num_materials, s->device_bytes)) != cudaSuccess) {
            dr_scene_destroy(s);
            return cuda_fail(e, "dr_scene_create upload materials");
        }
        s->num_materials = desc->num_materials;
    }
    const dr_status rs = build_render_data(s, desc);
    if (rs != DR_OK) {
        dr_scene_destroy(s);
        return rs;
    }
    s->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    *out = s;
    return DR_OK;
}

dr_status dr_scene_destroy(dr_scene *s)
{
    if (!s) return DR_OK;
    cudaSetDevice(s->ctx->device);
    cudaFree(s->d_nodes);
    cudaFree(s->d_nodes8);
    cudaFree(s->d_tri_ref);
    cudaFree(s->d_tri_wt);
    cudaFree(s->d_prim);
    cudaFree(s->d_materials);
    cudaFree(s->d_objects);
    cudaFree(s->d_shade);
    cudaFree(s->d_light_table);
    cudaFree(s->d_tri_tables);
    delete s->runner;
    cudaFree(s->d_stage_rays);
    cudaFree(s->d_stage_hits);
    for (cudaStream_t h : s->stage_streams)
        if (h) cudaStreamDestroy(h);
    delete s;
    return DR_OK;
}

dr_status dr_scene_get_info(const dr_scene *s, dr_scene_info *info)
{
    DR_CHECK_ARG(s && info, "dr_scene_get_info: NULL argument");
    info->num_triangles = s->num_tris;
    info->num_nodes = s->num_nodes;
    info->depth = s->depth;
    info->layout = s->layout;
    info->slack = s->slack;
    info->total_radiant_power = s->total_radiant_power;
    info->device_bytes = s->device_bytes;
    info->build_seconds = s->build_seconds;
    return DR_OK;
}

dr_status dr_scene_get_render_stats(const dr_scene *s, dr_render_stats *stats)
{
    DR_CHECK_ARG(s && stats, "dr_scene_get_render_stats: NULL argument");
    *stats = dr_render_stats{};
    if (!s->runner || !s->runner->d_totals) return DR_OK;
    DR_CUDA(cudaSetDevice(s->ctx->device));
    DR_CUDA(cudaDeviceSynchronize());  // the render's streams do not synchronise with the legacy stream
    unsigned long long t[2];
    DR_CUDA(cudaMemcpy(t, s->runner->d_totals, sizeof t, cudaMemcpyDeviceToHost));
    stats->path_rays = t[0];
    stats->shadow_rays = t[1];
    return DR_OK;
}

dr_status dr_scene_get_light_table(const dr_scene *s, dr_alias_entry *table_host, uint32_t capacity,
                                   uint32_t *count)
{
    DR_CHECK_ARG(s && count, "dr_scene_get_light_table: NULL argument");
    *count = s->num_objects;
    if (!table_host || capacity == 0) return DR_OK;
    DR_CHECK_ARG(capacity >= s->num_objects, "dr_scene_get_light_table: capacity below the object count");
    if (s->num_objects == 0 || !s->d_light_table) return DR_OK;
    DR_CUDA(cudaSetDevice(s->ctx->device));
    DR_CUDA(cudaMemcpy(table_host, s->d_light_table, (size_t)s->num_objects * sizeof(dr_alias_entry),
                       cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_device_allocate(dr_context *ctx, uint64_t bytes, void **dev)
{
    DR_CHECK_ARG(ctx && dev, "dr_device_allocate: NULL argument");
    *dev = nullptr;
    if (bytes == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    const cudaError_t e = dev_malloc(dev, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(DR_ERR_OUT_OF_MEMORY, "dr_device_allocate: %llu bytes", (unsigned long long)bytes);
    }
    if (e != cudaSuccess) return cuda_fail(e, "dr_device_allocate");
    return DR_OK;
}

dr_status dr_device_free(dr_context *ctx, void *dev)
{
    DR_CHECK_ARG(ctx != nullptr, "dr_device_free: ctx is NULL");
    if (!dev) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    DR_CUDA(cudaFree(dev));
    return DR_OK;
}

dr_status dr_device_copy_from_host(dr_context *ctx, void *dev, const void *host, uint64_t bytes)
{
    DR_CHECK_ARG(ctx && (bytes == 0 || (dev && host)), "dr_device_copy_from_host: NULL argument");
    if (bytes == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    DR_CUDA(cudaMemcpy(dev, host, bytes, cudaMemcpyHostToDevice));
    return DR_OK;
}

dr_status dr_device_copy_to_host(dr_context *ctx, void *host, const void *dev, uint64_t bytes)
{
    DR_CHECK_ARG(ctx && (bytes == 0 || (dev && host)), "dr_device_copy_to_host: NULL argument");
    if (bytes == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    DR_CUDA(cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost));
    return DR_OK;
}

dr_status dr_device_zero(dr_context *ctx, void *dev, uint64_t bytes, void *stream)
{
    DR_CHECK_ARG(ctx && (bytes == 0 || dev), "dr_device_zero: NULL argument");
    if (bytes == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    DR_CUDA(cudaMemsetAsync(dev, 0, bytes, static_cast<cudaStream_t>(stream)));
    return DR_OK;
}

dr_status dr_synchronize(dr_context *ctx, void *stream)
{
    DR_CHECK_ARG(ctx != nullptr, "dr_synchronize: ctx is NULL");
    DR_CUDA(cudaSetDevice(ctx->device));
    if (stream) DR_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    else DR_CUDA(cudaDeviceSynchronize());
    return check_error_word(ctx, static_cast<cudaStream_t>(stream));
}

dr_status dr_trace_closest(dr_scene *s, const dr_ray *rays, uint64_t n, dr_hit *hits, int32_t tri_mode,
                           dr_trace_counters *counters, void *stream)
{
    DR_CHECK_ARG(s != nullptr, "dr_trace_closest: scene is NULL");
    DR_CHECK_ARG(n == 0 || (rays && hits), "dr_trace_closest: NULL buffer");
    DR_CHECK_ARG(tri_mode == DR_TRI_REFERENCE || tri_mode == DR_TRI_WATERTIGHT, "dr_trace_closest: bad tri_mode");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(rays) & 15) == 0 && (reinterpret_cast<uintptr_t>(hits) & 7) == 0,
                 "dr_trace_closest: rays must be 16-byte and hits 8-byte aligned");
    DR_CUDA(cudaSetDevice(s->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    TraceArgs a = trace_args(s);
    a.rays = rays;
    a.n = n;
    a.hits = hits;
    if (counters) DR_CUDA(cudaMemsetAsync(a.counters, 0, 8 * sizeof(unsigned long long), st));
    DR_CUDA(launch_trace_closest(a, tri_mode, counters != nullptr, st));
    if (counters) {
        unsigned long long c[8];
        DR_CUDA(cudaMemcpyAsync(c, a.counters, sizeof(c), cudaMemcpyDeviceToHost, st));
        DR_CUDA(cudaStreamSynchronize(st));
        counters->rays = n;
        counters->node_visits = c[0];
        counters->box_tests = c[1];
        counters->tri_tests = c[2];
        counters->hits = c[3];
        return check_error_word(s->ctx, st);
    }
    return DR_OK;
}

dr_status dr_trace_any(dr_scene *s, const dr_ray *rays, uint64_t n, uint8_t *occluded, int32_t tri_mode, void *stream)
{
    DR_CHECK_ARG(s != nullptr, "dr_trace_any: scene is NULL");
    DR_CHECK_ARG(n == 0 || (rays && occluded), "dr_trace_any: NULL buffer");
    DR_CHECK_ARG(tri_mode == DR_TRI_REFERENCE || tri_mode == DR_TRI_WATERTIGHT, "dr_trace_any: bad tri_mode");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(rays) & 15) == 0, "dr_trace_any: rays must be 16-byte aligned");
    DR_CUDA(cudaSetDevice(s->ctx->device));
    TraceArgs a = trace_args(s);
    a.rays = rays;
    a.n = n;
    a.occluded = occluded;
    DR_CUDA(launch_trace_any(a, tri_mode, static_cast<cudaStream_t>(stream)));
    return DR_OK;
}

// Chunk sizes of dr_trace_closest_host in relative units (see there).
// Compute streams the chunks of dr_trace_closest_host rotate over (2 or 3;
// measured the same: 3.778 and 3.779 ms per 16.8 M-ray step).
#ifndef DR_HOST_COMPUTE_STREAMS
#define DR_HOST_COMPUTE_STREAMS 2
#endif
#ifndef DR_HOST_CHUNKS
#define DR_HOST_CHUNKS 1, 1, 2, 2, 4, 4, 4, 4, 4, 4, 2
#endif

dr_status dr_trace_closest_host(dr_scene *s, const dr_ray *rays_host, uint64_t n, dr_hit *hits_host,
                                int32_t tri_mode, void *stream)
{
    DR_CHECK_ARG(s != nullptr, "dr_trace_closest_host: scene is NULL");
    DR_CHECK_ARG(n == 0 || (rays_host && hits_host), "dr_trace_closest_host: NULL buffer");
    DR_CHECK_ARG(tri_mode == DR_TRI_REFERENCE || tri_mode == DR_TRI_WATERTIGHT, "dr_trace_closest_host: bad tri_mode");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(s->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    if (s->stage_capacity < n) {
        cudaFree(s->d_stage_rays);
        cudaFree(s->d_stage_hits);
        s->d_stage_rays = s->d_stage_hits = nullptr;
        s->stage_capacity = 0;
        DR_CUDA(dev_malloc(&s->d_stage_rays, n * sizeof(dr_ray)));
        DR_CUDA(dev_malloc(&s->d_stage_hits, n * sizeof(dr_hit)));
        s->stage_capacity = n;
    }
    // Pipeline in chunks: the copy-in of chunk k+1 and the copy-out of chunk
    // k-1 overlap the traversal of chunk k. Chunks alternate between two
    // compute streams, so the tail of one persistent launch overlaps the start
    // of the next (each launch has its own work counter). Measured (16.8 M
    // rays, 2^20 triangles): one compute stream 5.11 / 5.21 / 5.87 ms for 4 /
    // 8 / 16 chunks; two streams 4.76 / 4.52 / 4.55 / 4.63 / 4.89 ms for
    // 4 / 8 / 12 / 16 / 24 chunks. With the faster traversal: 8 equal chunks
    // 4.13 ms; a first chunk of 1/32 and a second of 1/16 of the rays (the
    // traversal starts sooner) 4.01 ms; short chunks at the end as well
    // 4.07 ms. Reading the rays and writing the hits in place in mapped
    // page-locked memory, in one launch: 4.82 ms; copying the chunks in on
    // two alternating streams: 4.43 ms. With the 3.19 ms traversal (chunks
    // in 32nds): 1,2,4,4,4,5,4,4,4 3.87 ms; 1,1,2,2,4,4,4,4,4,4,2 3.77-3.79;
    // 1,1,2,3,4,4,4,4,4,3,2 3.77; 1,2,5,6,6,6,6 3.91; 1,1,2,2,3 x 8,1,1 3.86.
    auto *d_rays = static_cast<dr_ray *>(s->d_stage_rays);
    auto *d_hits = static_cast<dr_hit *>(s->d_stage_hits);
    // chunk boundaries, in 32nds of the rays: short first chunks so the
    // traversal starts sooner, a short last one so less of it waits for the
    // final copy-out (chunks under 2^18 rays join the next)
    std::vector<uint64_t> bounds{0};
    {
        static const int parts[] = {DR_HOST_CHUNKS, 0};
        int total = 0;
        for (int i = 0; parts[i]; ++i) total += parts[i];
        uint64_t acc = 0;
        for (int i = 0; parts[i]; ++i) {
            acc += (uint64_t)parts[i];
            uint64_t e = n * acc / (uint64_t)total;
            if (e - bounds.back() < (1u << 18) && parts[i + 1]) continue;  // too small: merge into the next
            bounds.push_back(e);
        }
        if (bounds.back() != n) bounds.push_back(n);
    }
    for (cudaStream_t &h : s->stage_streams)
        if (!h) DR_CUDA(cudaStreamCreateWithFlags(&h, cudaStreamNonBlocking));
    cudaStream_t copy_in = s->stage_streams[0], copy_out = s->stage_streams[1];
    constexpr int kCompute = DR_HOST_COMPUTE_STREAMS;
    static_assert(kCompute >= 2 && kCompute <= 3, "2 or 3 compute streams");
    const cudaStream_t compute[3] = {st, s->stage_streams[2], s->stage_streams[3]};
    std::vector<cudaEvent_t> ev;
    auto new_event = [&]() {
        cudaEvent_t e;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        ev.push_back(e);
        return e;
    };
    cudaError_t err = cudaSuccess;
    cudaEvent_t start = new_event();
    err = cudaEventRecord(start, st);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(copy_in, start, 0);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(copy_out, start, 0);
    for (int c = 1; c < kCompute && err == cudaSuccess; ++c) err = cudaStreamWaitEvent(compute[c], start, 0);
    for (size_t k = 0; k + 1 < bounds.size() && err == cudaSuccess; ++k) {
        const uint64_t b = bounds[k], m = bounds[k + 1] - bounds[k];
        if (m == 0) continue;
        const cudaStream_t cs = compute[k % kCompute];
        err = cudaMemcpyAsync(d_rays + b, rays_host + b, m * sizeof(dr_ray), cudaMemcpyHostToDevice, copy_in);
        cudaEvent_t in_done = new_event();
        if (err == cudaSuccess) err = cudaEventRecord(in_done, copy_in);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(cs, in_done, 0);
        TraceArgs a = trace_args(s);
        a.rays = d_rays + b;
        a.hits = d_hits + b;
        a.n = m;
        if (err == cudaSuccess) err = launch_trace_closest(a, tri_mode, false, cs);
        cudaEvent_t tr_done = new_event();
        if (err == cudaSuccess) err = cudaEventRecord(tr_done, cs);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(copy_out, tr_done, 0);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(hits_host + b, d_hits + b, m * sizeof(dr_hit), cudaMemcpyDeviceToHost, copy_out);
    }
    cudaEvent_t out_done = new_event();
    if (err == cudaSuccess) err = cudaEventRecord(out_done, copy_out);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(st, out_done, 0);
    for (int c = 1; c < kCompute && err == cudaSuccess; ++c) {
        cudaEvent_t c_done = new_event();
        err = cudaEventRecord(c_done, compute[c]);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(st, c_done, 0);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    for (auto e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return cuda_fail(err, "dr_trace_closest_host");
    return DR_OK;
}

dr_status dr_alias_build(dr_context *ctx, const float *w, uint32_t n, dr_alias_entry *table, int32_t mode,
                         void *stream)
{
    DR_CHECK_ARG(ctx != nullptr, "dr_alias_build: ctx is NULL");
    DR_CHECK_ARG(n == 0 || (w && table), "dr_alias_build: NULL buffer");
    DR_CHECK_ARG(mode == DR_ALIAS_REFERENCE || mode == DR_ALIAS_SWEEP, "dr_alias_build: bad mode");
    DR_CHECK_ARG(n < (1u << 30), "dr_alias_build: n too large");
    if (n == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    const size_t need = alias_scratch_bytes(n, mode);
    if (ctx->scratch_bytes < need) {
        // the scratch may be in use by earlier work on any stream
        DR_CUDA(cudaDeviceSynchronize());
        const dr_status s = ensure_scratch(ctx, need);
        if (s != DR_OK) return s;
    }
    DR_CUDA(launch_alias_build(w, n, table, mode, ctx->scratch, ctx->scratch_bytes, ctx->num_sms, st));
    return DR_OK;
}

dr_status dr_alias_sample(const dr_alias_entry *table, uint32_t n, const float *u, uint64_t ndraws, int32_t *index,
                          float *pdf, void *stream)
{
    DR_CHECK_ARG(ndraws == 0 || (table && u && index && pdf && n > 0), "dr_alias_sample: bad argument");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(u) & 7) == 0, "dr_alias_sample: uniforms must be 8-byte aligned");
    DR_CUDA(launch_alias_sample(table, n, u, ndraws, index, pdf, static_cast<cudaStream_t>(stream)));
    return DR_OK;
}

}  // extern "C"
