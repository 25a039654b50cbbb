/*
 * devilray_gb300.h -- C ABI of the GB300 path-tracing core.
 *
 * The drop-in boundary for DevilRay's hot path. DevilRay itself has no FFI: its
 * plugin surface is the C++ classes Renderer / Scene / GpuTris and the
 * DistributionSamplers functions. Each entry point below names the reference
 * interface it replaces (file:line in the DevilRay tree). The C++ classes of
 * include/devilray/ rebuild that class surface on top of these functions.
 *
 * Conventions
 *   - Every call returns a dr_status; nothing throws across the ABI and nothing
 *     calls exit() (DevilRay's CUDA_ERROR_CHECK exits: src/device/DevUtils.cu:12-22).
 *     dr_last_error_string() describes the last failure of the calling thread.
 *   - Pointers named *_dev are device pointers; *_host are host pointers.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     Calls that take a stream are asynchronous unless stated otherwise.
 *   - No CPU fallback: without a usable GPU, calls fail with DR_ERR_NO_DEVICE.
 */
#ifndef DEVILRAY_GB300_H
#define DEVILRAY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DR_ABI_VERSION 6

typedef enum dr_status {
    DR_OK = 0,
    DR_ERR_INVALID_ARGUMENT = 1,
    DR_ERR_CUDA = 2,
    DR_ERR_OUT_OF_MEMORY = 3,
    DR_ERR_NO_DEVICE = 4,
    DR_ERR_TIMEOUT = 5,        /* a bounded device loop gave up (error word set) */
    DR_ERR_STACK_OVERFLOW = 6, /* a traversal stack would have overflowed */
    DR_ERR_UNSUPPORTED = 7,
    DR_ERR_TOO_LARGE = 8
} dr_status;

/* Triangle test used by traversal. */
typedef enum dr_tri_mode {
    /* FP32 operation sequence of testTriangleIntersection
     * (include/tracing/IntersectionTestsImpl.hpp:253-297): bit-identical t. */
    DR_TRI_REFERENCE = 0,
    /* Watertight test (Woop, Benthin, Wald, JCGT 2013), two-sided. */
    DR_TRI_WATERTIGHT = 1
} dr_tri_mode;

/* Ray record, 32 bytes. A hit counts when its t <= tmax (use INFINITY for an
 * unbounded ray, which is the reference's only kind: Ray, include/Utils.hpp:191). */
typedef struct dr_ray {
    float ox, oy, oz, tmax;
    float dx, dy, dz, pad;
} dr_ray;

/* Closest-hit record, 8 bytes: prim is the triangle's index in the soup given
 * to dr_scene_create (-1 and t = +INFINITY on a miss). Replaces the optional
 * Intersection of getIntersection/cast (IntersectionTestsImpl.hpp:222-251),
 * which carries no triangle index. Ties in t go to the smaller prim. */
typedef struct dr_hit {
    float t;
    int32_t prim;
} dr_hit;

/* Per-call traversal counters (benchmark::HitTests, include/tracing/Benchmark.hpp:3-14). */
typedef struct dr_trace_counters {
    uint64_t rays;
    uint64_t node_visits;    /* BVH nodes fetched */
    uint64_t box_tests;      /* child boxes tested */
    uint64_t tri_tests;      /* triangle tests */
    uint64_t hits;
} dr_trace_counters;

/* ---- context ----------------------------------------------------------------- */

typedef struct dr_context dr_context;

typedef struct dr_context_config {
    int32_t device;          /* CUDA ordinal */
    uint32_t flags;          /* reserved, 0 */
} dr_context_config;

/* Binds a device and creates the per-context scratch (work counters, error word). */
dr_status dr_context_create(const dr_context_config *cfg, dr_context **out);
dr_status dr_context_destroy(dr_context *ctx);
/* Reads and clears the device error word of the context (see dr_status). */
dr_status dr_context_check(dr_context *ctx);
/* Waits for `stream` (NULL: the whole device), then dr_context_check. */
dr_status dr_synchronize(dr_context *ctx, void *stream);

/* Device buffers for callers without a CUDA runtime of their own: the
 * allocate / free / copyFromHost / copyToHost of DeviceMemoryManager
 * (src/device/DeviceMemory.cu:11-60). Copies are synchronous; dr_device_zero is
 * asynchronous on `stream`. */
dr_status dr_device_allocate(dr_context *ctx, uint64_t bytes, void **dev);
dr_status dr_device_free(dr_context *ctx, void *dev);
dr_status dr_device_copy_from_host(dr_context *ctx, void *dev, const void *host, uint64_t bytes);
dr_status dr_device_copy_to_host(dr_context *ctx, void *host, const void *dev, uint64_t bytes);
dr_status dr_device_zero(dr_context *ctx, void *dev, uint64_t bytes, void *stream);

/* ---- materials and scene --------------------------------------------------------- */

/* AliasEntry of include/tracing/DistributionSamplers.hpp:44-51, 20 bytes. */
typedef struct dr_alias_entry {
    float p_A, pdf_A, pdf_B;
    int32_t A, B;
} dr_alias_entry;


/* Flat POD material, replacing the std::variant<TransparentMaterial, DiffuseMaterial>
 * of include/tracing/Material.hpp:9-32. 64 bytes. */
typedef enum dr_material_kind { DR_MAT_DIFFUSE = 0, DR_MAT_DIELECTRIC = 1 } dr_material_kind;
typedef struct dr_material {
    int32_t kind;            /* dr_material_kind */
    float ior;               /* TransparentMaterial::inside_medium.ior (Medium.hpp:3-10) */
    float pad0, pad1;
    float emission[4];       /* DiffuseMaterial::emission */
    float albedo[4];         /* DiffuseMaterial::diffuse_reflectance */
    float debug_color[4];    /* BaseMaterial::debug_color */
} dr_material;

/* An object: a contiguous triangle range of the soup with one material, the
 * flattened form of one TriangleMesh view (include/tracing/TriangleMesh.hpp:9-27).
 * surface_area is TriangleMesh::surface_area (the light-power weight area). */
typedef struct dr_object {
    uint32_t tri_begin;
    uint32_t tri_count;
    int32_t material;
    float surface_area;
} dr_object;

/* How dr_scene_create builds the scene's light tables (the object table over
 * emitted power and each emitting object's triangle table over area). Both
 * give a table of the same distribution; they differ in slot order. */
typedef enum dr_light_tables {
    /* Parallel sweep build (DR_ALIAS_SWEEP) of every table: the object table in
     * one parallel launch sequence, the triangle tables one device thread per
     * object up to 65,536 triangles and a parallel build above. Default. */
    DR_LIGHT_TABLES_SWEEP = 0,
    /* The pairing of generateAliasTable (DR_ALIAS_REFERENCE), bit-identical to
     * Renderer::calculateLightWeights and convertMeshToTris; each table is
     * built by one device thread, which takes about 2.8 us per object for the
     * object table (183 ms at 66,356 objects). */
    DR_LIGHT_TABLES_REFERENCE = 1
} dr_light_tables;

/* Scene description. positions: 9 floats per triangle (A, B, C) in world space
 * (object transforms already applied). When objects is NULL the whole soup is
 * one object using material 0. tri_material (optional) overrides the object's
 * material per triangle. tri_weight (optional) is the per-triangle weight of
 * the second-level light table (reference: triangle area, src/GpuTris.cpp:7-21).
 * light_tables is a dr_light_tables value (0 = sweep). */
typedef struct dr_scene_desc {
    const float *positions_host;
    uint32_t num_triangles;
    const dr_object *objects_host;
    uint32_t num_objects;
    const dr_material *materials_host;
    uint32_t num_materials;
    const int32_t *tri_material_host;
    const float *tri_weight_host;
    uint32_t light_tables;
} dr_scene_desc;

typedef enum dr_builder {
    DR_BUILD_HOST_SAH = 0,     /* binned SAH on the host (threads), either layout */
    DR_BUILD_DEVICE_LBVH = 1   /* linear BVH on the device (Morton order): the binary layout (one triangle per
                                  leaf; layout 0 or 2) or its collapse into compressed 8-wide nodes (layout 8) */
} dr_builder;

typedef struct dr_build_config {
    uint32_t max_leaf_size;  /* 0 = default (tuned) */
    uint32_t sah_bins;       /* 0 = default */
    uint32_t threads;        /* host build threads, 0 = all cores */
    uint32_t layout;         /* 0 = default, 2 = binary, 8 = compressed 8-wide */
    uint32_t builder;        /* dr_builder */
} dr_build_config;

typedef struct dr_scene dr_scene;

/* Builds the acceleration structure (binned-SAH, conservative boxes) on the
 * host and uploads scene, BVH and light tables to the device. Replaces
 * convertMeshToTris + generateSimpleBBH + viewGpuTris + Renderer::setScene /
 * calculateLightWeights (src/GpuTris.cpp:5-85, src/models/BBH.cpp:101-115,
 * src/Renderer.cpp:113-152). Synchronous. */
dr_status dr_scene_create(dr_context *ctx, const dr_scene_desc *desc,
                          const dr_build_config *cfg, dr_scene **out);
dr_status dr_scene_destroy(dr_scene *scene);

typedef struct dr_scene_info {
    uint32_t num_triangles;
    uint32_t num_nodes;
    uint32_t depth;
    uint32_t layout;
    float slack;             /* world-space box widening used for conservative culling */
    float total_radiant_power; /* ObjectsInfo::total_radiant_power (Scene.hpp:10-13) */
    uint64_t device_bytes;
    double build_seconds;
} dr_scene_info;
dr_status dr_scene_get_info(const dr_scene *scene, dr_scene_info *info);
/* The scene's object light table (Renderer::m_light_sampler, over the weights
 * of Renderer::calculateLightWeights, src/Renderer.cpp:113-152, built as
 * dr_scene_desc.light_tables says): *count =
 * number of objects; the table is copied when table_host is not NULL
 * (capacity >= count). Synchronous. */
dr_status dr_scene_get_light_table(const dr_scene *scene, dr_alias_entry *table_host, uint32_t capacity,
                                   uint32_t *count);

typedef struct dr_render_stats {
    uint64_t path_rays;      /* closest-hit rays of path vertices (the reference's ray_casts) */
    uint64_t shadow_rays;    /* next-event visibility rays */
} dr_render_stats;
/* Ray counts of the scene's last dr_render / dr_render_guided call (zeros
 * before the first): path rays as Renderer::getTotalCasts counts them
 * (include/Renderer.hpp:48-69), plus the shadow rays. Synchronous: waits for
 * the device. */
dr_status dr_scene_get_render_stats(const dr_scene *scene, dr_render_stats *stats);

/* ---- traversal ------------------------------------------------------------------- */

/* Closest hit for n rays (device buffers). Replaces cast / getIntersection
 * (IntersectionTestsImpl.hpp:222-251) and the runRaycasts kernel
 * (benchmark/src/benchmark.cu:16-55). counters_host may be NULL (no counting). */
dr_status dr_trace_closest(dr_scene *scene, const dr_ray *rays_dev, uint64_t n, dr_hit *hits_dev,
                           int32_t tri_mode, dr_trace_counters *counters_host, void *stream);

/* Any hit with t <= tmax: occluded_dev[i] = 1 or 0. Replaces visible()
 * (include/tracing/PathGeneration.hpp:213-224), which runs a full closest hit. */
dr_status dr_trace_any(dr_scene *scene, const dr_ray *rays_dev, uint64_t n, uint8_t *occluded_dev,
                       int32_t tri_mode, void *stream);

/* Same as dr_trace_closest over HOST buffers: copies rays in and hits out through
 * pinned staging on `stream`; returns after the hits are in hits_host. */
dr_status dr_trace_closest_host(dr_scene *scene, const dr_ray *rays_host, uint64_t n, dr_hit *hits_host,
                                int32_t tri_mode, void *stream);

/* ---- rendering ----------------------------------------------------------------------- */

/* Pinhole camera (include/tracing/Camera.hpp:6-19): row-major 4x4
 * camera-to-world transform (Matrix4x4f::values), focal length, principal
 * point and physical pixel size in sensor units, resolution in pixels. */
typedef struct dr_camera {
    float transform[16];
    float focal_length;
    float center[2];
    int32_t width, height;
    float pixel_size[2];
} dr_camera;

typedef enum dr_pixel_sampling { DR_PIXEL_CENTER = 0, DR_PIXEL_UNIFORM_RANDOM = 1 } dr_pixel_sampling;

/* First-hit debug views (DebugOptions, include/DebugOptions.hpp): the camera ray's
 * closest hit coloured by material debug colour x 0.5 (UV checker; only hits add
 * a sample), by its barycentrics, or by its winding order. */
typedef enum dr_debug_view {
    DR_DEBUG_OFF = 0,
    DR_DEBUG_UV_CHECKER = 1,
    DR_DEBUG_BARI_COORDS = 2,
    DR_DEBUG_WINDING_ORDER = 3
} dr_debug_view;

typedef struct dr_render_config {
    uint32_t max_depth;      /* path vertices per sample (reference: 10, PathGeneration.hpp:380) */
    uint32_t spp;            /* samples per pixel added by this call */
    uint32_t sample_offset;  /* index of the first sample (progressive rendering) */
    int32_t pixel_sampling;  /* dr_pixel_sampling */
    uint64_t seed;           /* Philox key */
    int32_t tri_mode;        /* dr_tri_mode */
    uint32_t wave_paths;     /* paths in flight per wave, 0 = automatic (2^22) */
    uint32_t flags;          /* reserved, 0 */
    int32_t debug;           /* dr_debug_view */
    uint32_t streams;        /* concurrent waves, 1..3, 0 = 3 */
    uint32_t chunk;          /* rays per warp fetch of the persistent traversal
                                (32, 64, 96 or 128), 0 = adaptive */
    uint32_t stack;          /* traversal-stack entries per lane kept in shared memory
                                by the 8-wide kernels (4, 8 or 16), 0 = 8 */
} dr_render_config;

/* Adds cfg->spp path samples per pixel to accum_dev (float4 per pixel, row
 * major: rgb sums and the sample count in w, as Buffers::color of
 * include/Buffers.hpp:9-22) and the path-ray casts to casts_dev (uint32 per
 * pixel, may be NULL). Replaces Renderer::render / cuda_render / sampleColor
 * (src/Renderer.cpp:198-233, src/device/RendererImpl.hpp:22-102,
 * include/tracing/PathGeneration.hpp:363-515) with a wavefront of kernels:
 * camera rays, closest hit, shading with next-event estimation and MIS, shadow
 * any hit, accumulation. Uniforms come from Philox4x32-10 indexed by (pixel,
 * sample, dimension); samples are added to a pixel in sample order.
 * Asynchronous on `stream`. */
dr_status dr_render(dr_scene *scene, const dr_camera *camera, const dr_render_config *cfg, float *accum_dev,
                    uint32_t *casts_dev, void *stream);

/* Accumulation buffers of a progressive render (Buffers, include/Buffers.hpp:9-22):
 * float4 colour sums with the sample count in w, and uint32 path-ray casts. */
typedef struct dr_framebuffer dr_framebuffer;

dr_status dr_framebuffer_create(dr_context *ctx, int32_t width, int32_t height, dr_framebuffer **out);
dr_status dr_framebuffer_destroy(dr_framebuffer *fb);
/* Zeroes colour and casts (Buffers::reset, src/Renderer.cpp:17-21). Asynchronous. */
dr_status dr_framebuffer_clear(dr_framebuffer *fb, void *stream);
/* Device pointers to pass to dr_render. */
dr_status dr_framebuffer_device_buffers(dr_framebuffer *fb, float **accum_dev, uint32_t **casts_dev);
/* Copies the buffers to the host (either pointer may be NULL) and the total of
 * the casts (Buffers::totalCasts, src/Renderer.cpp:29-35). Synchronous. */
dr_status dr_framebuffer_read(dr_framebuffer *fb, float *accum_host, uint32_t *casts_host, uint64_t *total_casts);
/* Renderer::createPixels (src/Renderer.cpp:51-90) on the device: average of the
 * samples, optional sRGB encoding, 8-bit RGBA with alpha 255, rows flipped so
 * the first row written is the top of the image. rgba_host: width * height
 * uint32 values. Synchronous. */
dr_status dr_framebuffer_tonemap(dr_framebuffer *fb, int32_t gamma_corrected, uint32_t *rgba_host);
/* The same conversion on any device accumulation buffer (float4 per pixel,
 * 16-byte aligned) into a device RGBA8 buffer. Asynchronous on `stream`.
 * height <= 65535. */
dr_status dr_tonemap(const float *accum_dev, int32_t width, int32_t height, int32_t gamma_corrected,
                     uint32_t *rgba_dev, void *stream);
/* The linear image of an accumulation buffer on the device, for headless
 * output: rgb_dev[3 (x + y width) + c] = accum[c] / accum.w (0 for pixels
 * without samples), rows in the accumulation's order (row 0 at the bottom).
 * Replaces the host averaging of Renderer::createPixels
 * (src/Renderer.cpp:51-90) where no display is attached. Asynchronous on
 * `stream`. */
dr_status dr_resolve(const float *accum_dev, int32_t width, int32_t height, float *rgb_dev, void *stream);
/* Writes the framebuffer's linear image (dr_resolve) as a little-endian PFM
 * file ("PF", rows from the bottom, as the format stores them). Synchronous. */
dr_status dr_framebuffer_write_pfm(dr_framebuffer *fb, const char *path);

/* ---- batched rendering ------------------------------------------------------------ */

/* One image of a batch: a scene, its camera, its render settings (spp,
 * max_depth, pixel_sampling, seed, tri_mode; sample_offset of the first render;
 * debug must be DR_DEBUG_OFF) and its device outputs (as dr_render). */
typedef struct dr_job {
    dr_scene *scene;
    dr_camera camera;
    dr_render_config config;
    float *accum_dev;
    uint32_t *casts_dev;
} dr_job;

typedef struct dr_batch_config {
    uint32_t wave_paths;     /* path slots per wave, 0 = 2^22 (at least one sample of the largest image) */
    uint32_t streams;        /* concurrent waves, 1..3, 0 = 3 */
    uint32_t chunk;          /* persistent traversal fetch (32..128, multiple of 32), 0 = adaptive */
    uint32_t use_graph;      /* 1: capture the schedule into a CUDA graph on the first render */
    uint32_t stack;          /* shared-memory traversal-stack entries per lane (4, 8 or 16), 0 = 8 */
} dr_batch_config;

typedef struct dr_batch dr_batch;

typedef struct dr_batch_info {
    uint32_t num_jobs, num_waves, max_wave_paths, layout;
    uint64_t graph_nodes;       /* nodes of the captured graph, 0 before the first render */
    uint64_t paths_per_render;  /* sum of width * height * spp */
    uint64_t device_bytes;      /* concatenated scene arrays */
    uint32_t streams, chunk;
} dr_batch_info;

/* Many images of many scenes (uneven sizes) traced as one schedule: the scenes
 * are concatenated on the device, each wave of path slots mixes images, and one
 * persistent traversal launch per bounce serves every scene in the wave. Scenes
 * must share a hierarchy layout and outlive nothing: the batch keeps its own
 * copy. Synchronous. */
dr_status dr_batch_create(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_batch_config *cfg,
                          dr_batch **out);
/* Adds every job's spp samples to its image; job j starts at sample_offsets[j]
 * (NULL: its config.sample_offset on the first render, then after the previous
 * render's samples). The first render captures the schedule into a CUDA graph
 * (use_graph), later renders replay it. Asynchronous on `stream`; renders of one
 * batch run one after another. */
dr_status dr_batch_render(dr_batch *batch, const uint32_t *sample_offsets, void *stream);
dr_status dr_batch_get_info(const dr_batch *batch, dr_batch_info *info);
dr_status dr_batch_destroy(dr_batch *batch);
/* dr_batch_create + one dr_batch_render without a graph + dr_batch_destroy. Synchronous. */
dr_status dr_render_batch(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_batch_config *cfg,
                          void *stream);

/* ---- autotuning ------------------------------------------------------------------- */

typedef struct dr_autotune_config {
    uint32_t probe_spp;      /* samples per probe render; 0 = min(spp, 2) (dr_autotune), 1 (batch) */
    uint32_t reps;           /* timed renders per candidate, minimum taken; 0 = 2 */
    uint32_t try_layouts;    /* dr_autotune: 1 = build the scene 8-wide and 2-wide and time both */
    uint32_t max_leaf_size;  /* build setting of the probe scenes, 0 = default */
} dr_autotune_config;

typedef struct dr_autotune_candidate {
    uint32_t layout, wave_paths, streams, chunk, stack;
    float ms;
} dr_autotune_candidate;

typedef struct dr_autotune_result {
    uint32_t layout, wave_paths, streams, chunk, stack;  /* the chosen settings */
    float best_ms;                                 /* probe time of the chosen settings */
    uint32_t num_candidates;
    dr_autotune_candidate candidates[64];          /* every probe, in order */
} dr_autotune_result;

/* Picks the hierarchy width (dr_build_config.layout) and the wave schedule
 * (dr_render_config wave_paths / streams / chunk / stack) for rendering `desc` through
 * `camera` with `cfg`, by coordinate descent over timed probe renders of the
 * same samples (images do not depend on these settings). Synchronous. */
dr_status dr_autotune(dr_context *ctx, const dr_scene_desc *desc, const dr_camera *camera,
                      const dr_render_config *cfg, const dr_autotune_config *tc, dr_autotune_result *out);
/* The same for a batch (dr_batch_config wave_paths / streams / chunk / stack; the layout
 * is the scenes'), probing the batch's images with probe_spp samples each. */
dr_status dr_autotune_batch(dr_context *ctx, const dr_job *jobs, uint32_t njobs, const dr_autotune_config *tc,
                            dr_autotune_result *out);

/* ---- path guiding ------------------------------------------------------------------ */

/* A small network that proposes directions at diffuse vertices: 80 inputs
 * (12-frequency sin/cos encoding of the position normalised by center and
 * half_extent, a unit direction, zero padding), 4 hidden layers of 64 (ReLU),
 * 40 outputs = an 8-lobe von Mises-Fisher mixture (per lobe: logit,
 * log-concentration clamped to [-4, 7], unnormalised mean direction). BF16
 * weights, FP32 accumulation on tensor cores; FP32 master weights trained with
 * Adam on the loss -sum c_i log q(d_i | x_i) / n, c_i = weight_i / mean(weight). */
typedef struct dr_guide dr_guide;

typedef struct dr_guide_config {
    uint64_t seed;            /* weight initialisation (He-uniform; last layer x 0.1) */
    float learning_rate;      /* 0 = 1e-3 */
    float beta1, beta2, epsilon;  /* Adam; 0 = 0.9, 0.999, 1e-8 */
    float center[3];          /* position normalisation */
    float half_extent;        /* 0 = 1 */
    uint32_t infer_kernel;    /* dr_guide_infer_kernel: the tensor-core path of inference and of the
                                 forward/backward pass of training */
    uint32_t warmup_steps;    /* the learning rate rises linearly over the first warmup_steps Adam steps
                                 (step s uses learning_rate x min(1, s / warmup_steps)); 0 = none */
} dr_guide_config;

typedef enum dr_guide_infer_kernel {
    DR_GUIDE_INFER_TCGEN05 = 0,   /* tcgen05.mma, accumulators in tensor memory (default) */
    DR_GUIDE_INFER_MMA_SYNC = 1   /* warp-level mma.sync, accumulators in registers */
} dr_guide_infer_kernel;

uint32_t dr_guide_num_params(void);
dr_status dr_guide_create(dr_context *ctx, const dr_guide_config *cfg, dr_guide **out);
dr_status dr_guide_destroy(dr_guide *guide);
/* FP32 master parameters, per layer W [out][in] then b [out] (layer fan-ins 80,
 * 64, 64, 64, 64; fan-outs 64, 64, 64, 64, 48). Setting resets Adam. Synchronous. */
dr_status dr_guide_set_params(dr_guide *guide, const float *params_host, uint32_t n);
dr_status dr_guide_get_params(dr_guide *guide, float *params_host, uint32_t n);
/* Checkpoint and resume of a network that trains: its whole state (the
 * configuration, the Adam step count, the FP32 parameters and both Adam
 * moments) as one host blob of dr_guide_state_bytes() bytes. dr_guide_set_state
 * restores it into any network of this library (its configuration included),
 * after which training continues as the saved network would have. No
 * counterpart in the reference, which has no guiding network; with the image
 * accumulation (the caller's buffer) and the render's sample offset it
 * resumes a guided render. Synchronous. */
uint64_t dr_guide_state_bytes(void);
dr_status dr_guide_get_state(dr_guide *guide, void *state_host, uint64_t bytes);
dr_status dr_guide_set_state(dr_guide *guide, const void *state_host, uint64_t bytes);
/* Network input of each row (pos, dir: 3 floats per row; out: 80 floats per row). */
dr_status dr_guide_encode(dr_guide *guide, const float *pos_dev, const float *dir_dev, uint32_t n, float *out_dev);
/* Network output y (40 floats per row). Asynchronous on `stream`. */
dr_status dr_guide_infer(dr_guide *guide, const float *pos_dev, const float *dir_dev, uint32_t n, float *y_dev,
                         void *stream);
/* Loss and gradient of every parameter for a batch (sampled directions sdir,
 * 3 floats per row; sample weights); nothing is updated. Synchronous. */
dr_status dr_guide_gradients(dr_guide *guide, const float *pos_dev, const float *dir_dev, const float *sdir_dev,
                             const float *weight_dev, uint32_t n, float *loss_host, float *grad_host);
/* One Adam step on a batch. Asynchronous on `stream`. */
dr_status dr_guide_train_step(dr_guide *guide, const float *pos_dev, const float *dir_dev, const float *sdir_dev,
                              const float *weight_dev, uint32_t n, void *stream);
/* The mixture of network outputs y (40 floats per row): a direction drawn
 * from uniforms u (3 per row: lobe, cosine, azimuth) and its density; or the
 * density of given unit directions (y_per_row = 0: one y for every row). */
dr_status dr_guide_mixture_sample(const float *y_dev, const float *u_dev, uint32_t n, float *dir_dev, float *pdf_dev,
                                  void *stream);
dr_status dr_guide_mixture_pdf(const float *y_dev, uint32_t y_per_row, const float *dir_dev, uint32_t n,
                               float *pdf_dev, void *stream);
/* Loss of the last dr_guide_gradients / dr_guide_train_step batch. Synchronous. */
dr_status dr_guide_last_loss(dr_guide *guide, float *loss_host);

typedef struct dr_guided_config {
    float alpha;              /* probability of drawing a diffuse direction from the network (0 <= alpha < 1) */
    uint32_t train;           /* 1: collect samples and train after every wave */
    uint32_t train_batch;     /* rows per training step, 0 = 16384 */
    uint32_t train_steps;     /* Adam steps after every wave, 0 = 4 */
    uint32_t train_budget;    /* no training once the network has taken this many steps, 0 = no limit */
    uint32_t target;          /* training target density: 0 = L cos (incident radiance L along the
                                 sampled direction), 1 = log(1 + L) cos (less dominated by rare bright paths) */
    uint32_t bounces;         /* guide the vertices of bounces 0 .. bounces-1 only (later ones sample the
                                 cosine lobe, no network evaluation), 0 = all */
    uint32_t alpha_ramp;      /* a wave uses alpha x min(1, s / alpha_ramp), s the Adam steps the network
                                 has taken when the wave is issued: an untrained network proposes
                                 little; 0 = alpha throughout */
} dr_guided_config;

/* dr_render with path guiding: at each diffuse vertex the network's mixture
 * (inputs: hit point, normal facing the incoming ray) proposes the next
 * direction with probability alpha, the cosine lobe otherwise, and the
 * estimator divides by the mixture density alpha q + (1 - alpha) cos / pi
 * (one-sample MIS), which also enters the MIS weights of next-event estimation
 * and of emission hits, so the image stays unbiased for any network. With
 * `train`, every finished wave's diffuse vertices (first 3 of each path) give
 * training samples (incident radiance along the sampled direction) and the
 * network takes train_steps Adam steps (in wave order; waves still overlap on
 * cfg->streams streams, and a wave may read weights that another wave's
 * training is updating: each vertex samples and weighs with the one mixture
 * it computed). Asynchronous on `stream`. */
dr_status dr_render_guided(dr_scene *scene, const dr_camera *camera, const dr_render_config *cfg, dr_guide *guide,
                           const dr_guided_config *gcfg, float *accum_dev, uint32_t *casts_dev, void *stream);

/* ---- alias tables ------------------------------------------------------------------- */

typedef enum dr_alias_mode {
    /* The pairing of generateAliasTable (src/DistributionSamplers.cpp:39-149):
     * bit-identical table, built by one device thread. */
    DR_ALIAS_REFERENCE = 0,
    /* Parallel sweeping construction in exact fixed point; slot i holds item i. */
    DR_ALIAS_SWEEP = 1
} dr_alias_mode;

/* Builds the alias table of n weights on the device (negative / non-finite
 * weights count as 0; a total below 1e-5 gives the uniform table, as the
 * reference). Replaces generateAliasTable. Uses the context's scratch, which
 * grows with cudaMalloc when n needs more. Asynchronous on `stream`. */
dr_status dr_alias_build(dr_context *ctx, const float *weights_dev, uint32_t n, dr_alias_entry *table_dev,
                         int32_t mode, void *stream);

/* ndraws draws of sample() (DistributionSamplers.hpp:64-88) with the two
 * uniforms of draw i at uniforms_dev[2i], uniforms_dev[2i+1]. */
dr_status dr_alias_sample(const dr_alias_entry *table_dev, uint32_t n, const float *uniforms_dev, uint64_t ndraws,
                          int32_t *index_dev, float *pdf_dev, void *stream);

/* dr_alias_build over host buffers (copies in and out). Synchronous. */
dr_status dr_alias_build_host(dr_context *ctx, const float *weights_host, uint32_t n, dr_alias_entry *table_host,
                              int32_t mode);

/* Sweep-mode alias build (same table as dr_alias_build with DR_ALIAS_SWEEP)
 * that allocates no device memory. No counterpart in the reference. For
 * callers that may not call cudaMalloc: a host application that owns every
 * device allocation and passes in only pre-allocated buffers, or a frame loop
 * that must not stall on cudaMalloc's implicit synchronisation. Its scratch is
 * a fixed array inside the library (about 2.6 MB on every GPU that loads it),
 * so n is limited to 65,536 weights (DR_ERR_TOO_LARGE above that). Needs no
 * context: it runs on the current device. The first call on a device sets up
 * the array's device address; make it before any stream capture, and do not
 * reset the device (cudaDeviceReset) after it. All calls share the array:
 * calls whose work overlaps on the GPU race. */
dr_status dr_alias_build_noalloc(const float *weights_dev, uint32_t n, dr_alias_entry *table_dev, void *stream);

/* ---- diagnostics ------------------------------------------------------------------- */

/* Streaming-read bandwidth of a device buffer in GB/s (reads it `reps` times
 * with L2-cached 16-byte loads, CUDA events on `stream`). A buffer that fits
 * in L2 measures L2 read bandwidth, one larger than L2 measures HBM. No
 * counterpart in the reference: it supplies the traversal roofline's
 * denominator. Synchronous. */
dr_status dr_probe_read_bandwidth(dr_context *ctx, const void *buf_dev, uint64_t bytes, uint32_t reps,
                                  double *gbs_out, void *stream);

/* ---- failure-path test hooks -------------------------------------------------------- */
/* No counterpart in the reference, which exits the process on any CUDA error
 * (src/device/DevUtils.cu:12-22). These make the library take the error paths
 * that a real timeout, stack overflow or out-of-memory takes, without faulting,
 * trapping or hanging a GPU, so that tests can check the statuses. */

/* One warp waits, with at most `polls` polls, on an mbarrier phase that
 * nothing completes (no copy or MMA in flight on it), through the same
 * bounded wait as the traversal and guiding kernels; giving up, it sets the
 * context's timeout bit as they do. The next dr_context_check or
 * dr_synchronize returns DR_ERR_TIMEOUT and clears it; the context stays
 * usable. Asynchronous on `stream`. */
dr_status dr_debug_expire_wait(dr_context *ctx, uint32_t polls, void *stream);

/* Caps the stack of the context's 8-wide traversals at `entries` (1..64;
 * 0 restores 64, the size the builders' depth limit never exceeds). A ray
 * that needs more stops and sets the stack-overflow bit (reported as
 * DR_ERR_STACK_OVERFLOW); its hit is not valid. */
dr_status dr_debug_stack_limit(dr_context *ctx, uint32_t entries);

/* Makes the `after`-th next device allocation of the library (after = 1:
 * the next one) fail as cudaMalloc does when the device is out of memory;
 * 0 turns it off. Process-wide. The failing call returns DR_ERR_OUT_OF_MEMORY
 * and frees what it had allocated. */
dr_status dr_debug_fail_allocation(uint32_t after);

/* ---- version ----------------------------------------------------------------------- */

uint32_t dr_abi_version(void);
const char *dr_last_error_string(void);

#ifdef __cplusplus
}
#endif

#endif /* DEVILRAY_GB300_H */
