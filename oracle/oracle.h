/*
 * oracle.h -- CPU restatement of DevilRay's tracing path (TEST INFRASTRUCTURE).
 *
 * This library is the oracle the GB300 kernels are compared against. Only the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it; the
 * product library never links or calls it.
 *
 * Every function restates one reference function (file:line cited beside it,
 * paths relative to the DevilRay source tree) in plain C++ compiled with
 * -ffp-contract=off, so that FP32 results are bit-identical to the reference
 * compiled the same way. The restatement is pinned against the reference
 * itself (oracle/_ref harness, tests/golden fixtures).
 */
#ifndef DEVILRAY_ORACLE_H
#define DEVILRAY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- triangle / box tests ------------------------------------------------ */

/* include/tracing/IntersectionTestsImpl.hpp:253-297 (testTriangleIntersection).
 * ray = {px,py,pz,vx,vy,vz}, tri = {A,B,C}. Returns 1 on hit with
 * out = {t, wA, wB, wC}. */
int or_tri_test_ref(const float ray[6], const float tri[9], float out[4]);

/* Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013), two-sided,
 * FP32 with the FP64 edge-function fallback of the paper. out = {t, wA, wB, wC}. */
int or_tri_test_watertight(const float ray[6], const float tri[9], float out[4]);

/* include/tracing/IntersectionTestsImpl.hpp:91-105 (testBoxIntersection). */
int or_box_test_ref(const float box[6], const float ray[6], float *t_out);

/* ---- median-split BBH (src/models/BBH.cpp:38-115) ------------------------ */

typedef struct or_bbh or_bbh;

/* Builds the reference BBH over a triangle soup (9 floats per triangle, triangle
 * k owning vertices 3k..3k+2). `order` receives, for each sorted position, the
 * original triangle index. */
or_bbh *or_bbh_create(const float *positions, int32_t num_triangles);
void or_bbh_destroy(or_bbh *h);
int32_t or_bbh_num_nodes(const or_bbh *h);
int32_t or_bbh_depth(const or_bbh *h);
/* boxes: 6 floats per node; links: 5 ints per node {left,right,parent,begin,end};
 * order: num_triangles ints. Any pointer may be NULL. */
void or_bbh_export(const or_bbh *h, float *boxes, int32_t *links, int32_t *order);

/* Closest hit, reference-exact: restates getIntersectionImpl
 * (IntersectionTestsImpl.hpp:141-220) including its traversal order, its
 * culling and its first-found tie rule. rays: 6 floats each. Outputs per ray:
 * t (+inf on miss), prim (original triangle index, -1 on miss), optional
 * counters (box tests, triangle tests; benchmark::HitTests, Benchmark.hpp:3-14).
 * tri_mode: 0 = reference triangle test, 1 = watertight. */
void or_bbh_trace_reference(const or_bbh *h, const float *rays, int64_t num_rays,
                            float *t_out, int32_t *prim_out,
                            int64_t *box_tests, int64_t *tri_tests,
                            int32_t tri_mode, int32_t threads);

/* Closest hit, canonical semantics shared with the GPU kernels: the minimum t
 * over all triangles (reference triangle test or watertight test), ties broken
 * by the smaller original triangle index; a hit counts when t <= tmax.
 * Implemented as a conservative traversal of the BBH (boxes widened by
 * `slack` world units) so it equals a brute-force scan. rays: 8 floats each
 * {ox,oy,oz,tmax,dx,dy,dz,pad} (the dr_ray layout). */
void or_bbh_trace_canonical(const or_bbh *h, const float *rays8, int64_t num_rays,
                            float slack, float *t_out, int32_t *prim_out,
                            int32_t tri_mode, int32_t threads);

/* Any hit with t <= tmax (same test semantics): occluded[i] = 1 or 0. */
void or_bbh_trace_any(const or_bbh *h, const float *rays8, int64_t num_rays,
                      float slack, uint8_t *occluded, int32_t tri_mode, int32_t threads);

/* Brute force over a soup, canonical semantics. */
void or_trace_brute(const float *positions, int32_t num_triangles,
                    const float *rays8, int64_t num_rays,
                    float *t_out, int32_t *prim_out, int32_t tri_mode, int32_t threads);

/* ---- alias tables (src/DistributionSamplers.cpp:39-149) ------------------ */

/* AliasEntry layout of include/tracing/DistributionSamplers.hpp:44-51. */
typedef struct or_alias_entry { float p_A, pdf_A, pdf_B; int32_t A, B; } or_alias_entry;

/* generateAliasTable restated with the same std::priority_queue pairing. */
void or_alias_build_ref(const float *weights, int32_t n, or_alias_entry *out);

/* Sweep-pairing build restated on the CPU; the device's parallel build must
 * match it bit for bit (see the product's alias kernels). */
void or_alias_build_sweep(const float *weights, int32_t n, or_alias_entry *out);

/* sample(), DistributionSamplers.hpp:64-88, given the two uniforms. */
void or_alias_sample(const or_alias_entry *table, int32_t n, float u0, float u1,
                     int32_t *index, float *pdf);

/* The StressTest input of test/src/test_alias.cpp:193-229:
 * std::mt19937(seed) + std::lognormal_distribution<float>(0,1). */
void or_lognormal_input(int32_t n, uint32_t seed, float *out);

/* ---- integrator (include/tracing/PathGeneration.hpp:363-515) ------------- */

typedef struct or_object { uint32_t tri_begin, tri_count; int32_t material; float surface_area; } or_object;
typedef struct or_material {
    int32_t kind; float ior; float pad0, pad1;
    float emission[4]; float albedo[4]; float debug_color[4];
} or_material;                                           /* the dr_material layout */
typedef struct or_camera {
    float m[16];                                         /* row-major camera-to-world */
    float focal, cx, cy;
    int32_t width, height;
    float psx, psy;
} or_camera;
typedef struct or_render_cfg {
    int32_t max_depth, spp, sample_offset, pixel_sampling;   /* 0 centre, 1 uniform random */
    uint64_t seed;
    int32_t rng_mode;        /* 0: Philox indexed by (pixel, sample, dim); 1: replayed stream */
    int32_t trig_mode;       /* 0: portable polynomials; 1: std::sin/cos/acos */
    int32_t cast_mode;       /* 0: canonical closest hit; 1: the reference's per-object cast */
    int32_t tri_table_order; /* 0: soup order; 1: per-object BBH-sorted order */
    int32_t threads;
    int32_t replay_stride;   /* uniforms per (pixel, sample) in `replay` */
    const float *replay;     /* [pixel][sample][replay_stride] */
    int32_t debug;           /* 0 off, 1 UV checker, 2 barycentrics, 3 winding order */
    const int64_t *pixels;   /* NULL: every pixel; else render only these pixel indices (y * width + x);
                                outputs keep the full image's indexing */
    int64_t num_pixels;
} or_render_cfg;

typedef struct or_scene or_scene;
/* light_tables: 0 = every light table by or_alias_build_sweep (the GPU's
 * default, DR_LIGHT_TABLES_SWEEP), 1 = by or_alias_build_ref (the reference's
 * generateAliasTable pairing, DR_LIGHT_TABLES_REFERENCE). */
or_scene *or_scene_create(const float *positions, int32_t num_tris, const or_object *objects, int32_t num_objects,
                          const or_material *materials, int32_t num_materials, const int32_t *tri_material,
                          int32_t light_tables);
void or_scene_destroy(or_scene *s);
float or_scene_total_power(const or_scene *s);
void or_scene_light_table(const or_scene *s, or_alias_entry *out);
/* sample_rgb: [spp][height*width][3] per-sample colour, accum: [height*width][4]
 * (sum and sample count as Buffers::color), casts: [height*width] path rays.
 * Any output may be NULL. */
void or_render(const or_scene *s, const or_camera *cam, const or_render_cfg *cfg, float *sample_rgb, float *accum,
               uint32_t *casts);

/* FP64 restatement of the same integrator for converged reference images:
 * adds the sum of cfg->spp sample colours of every rendered pixel to
 * sum_rgb [height*width][3] (double). Uses max_depth, spp, sample_offset,
 * pixel_sampling, seed, threads and pixels of cfg; closest hits over a
 * double-precision BVH, lights drawn from double cumulative sums, std trig
 * functions, Philox uniforms of 53 bits on a stream of their own. */
void or_render_f64(const or_scene *s, const or_camera *cam, const or_render_cfg *cfg, double *sum_rgb);

/* Renderer::createPixels (src/Renderer.cpp:51-90): accum [height*width][4]
 * (colour sums, sample count in w) to RGBA8 rows, first row = top of the image.
 * gamma != 0: OutputLinearity::GammaCorrected (sRGB); 0: Linear. */
void or_create_pixels(const float *accum, int32_t width, int32_t height, int32_t gamma, uint32_t *out);

/* ---- path-guiding network (not part of the reference; restates the product's
 * network in FP64 with BF16-rounded weights and layer inputs) ------------- */
int32_t or_mlp_num_params(void);
/* 12-frequency position encoding of (pos - center) / half, then dir, zero padded to 80. */
void or_guide_encode(const float *pos, const float *dir, const float *center, float half, float *out80);
/* inputs [n][80] -> out [n][48] */
void or_mlp_forward(const float *params, const float *inputs, int32_t n, float *out);
/* log q(w) of the 8-lobe vMF mixture of network output y[40] at unit direction w. */
double or_vmf_mixture_log_pdf(const float *y, const float *w);
/* Batch loss -sum c_i log q(dir_i | input_i) / n, c_i = weight_i / mean(weight),
 * and its gradient for every parameter. */
void or_mlp_loss_grad(const float *params, const float *inputs, const float *dirs, const float *weights, int32_t n,
                      double *loss, double *grad);
void or_adam_step(float *params, float *m, float *v, const float *grad, int32_t n, int32_t t, float lr, float beta1,
                  float beta2, float eps);

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------------------- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif

#endif
