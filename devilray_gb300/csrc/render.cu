// render.cu -- wavefront path tracer on sm_103a.
//
// Replaces cuda_render + sampleColor (DevilRay src/device/RendererImpl.hpp:
// 22-102, include/tracing/PathGeneration.hpp:363-515): one thread per pixel
// that builds a whole path, then shades it, becomes a wave of kernels over a
// batch of path slots:
//   camera -> for each bounce: closest hit -> shade (emission with MIS, a light
//   sample, the BSDF sample; compaction of surviving paths and of shadow rays by
//   warp ballot) -> shadow any hit (+ next-event contribution) -> accumulate.
// The shading restates the reference's arithmetic in a forward order that adds
// the same terms in the same sequence (emission of vertex k, then its light
// sample, then vertex k+1), so each sample's colour is bit-identical to the
// reference evaluated on the same random numbers, with the portable sin/cos/acos
// of ptmath.cuh. Uniforms: Philox4x32-10 with counter (pixel, sample, group,
// tag) and key = seed; camera dims 0,1; bounce b: 4 + 12 b + {0,1 sphere,
// 2 Fresnel, 3..8 light sample}.
//
// The same kernels serve one image (dr_render) and a batch of images of many
// scenes (dr_batch): every slot carries its job (image), pixel and sample, and
// the job names the hierarchy root, light tables and camera it uses.

#include "dr_internal.h"
#include "render_internal.h"
#include "alias_kernels.cuh"
#include "ptmath.cuh"
#include "trace_device.cuh"
#include "persistent.cuh"
#include "guide_math.cuh"
#include "guide_internal.h"

#include <algorithm>

namespace dr {
namespace {

constexpr float kPi = 3.14159274f;
constexpr uint32_t kStreamTag = 0x44526E67u;
constexpr int kRenderBlock = 128;
// Resident blocks per SM the plain shading kernel is compiled for (at most 64
// registers). Measured on the box room, 256x256 x 16 spp: a minimum of 1 block
// (138 registers) 2.99 ms, the compiler's choice without a minimum (80
// registers, 6 blocks) about 2.69 ms, 8 blocks 2.60-2.64 ms; many-light 1080p
// (16 spp): 8 blocks 40.6 ms, 10 blocks (48 registers, spills) 41.0 ms, 12
// blocks 41.3 ms. The guided one has its own bound (DR_GUIDE_SHADE_BLOCKS).
#ifndef DR_SHADE_MIN_BLOCKS
#define DR_SHADE_MIN_BLOCKS 8
#endif
constexpr int kShadeMinBlocks = DR_SHADE_MIN_BLOCKS;

struct RenderParams {
    TraceArgs trace;
    const float4 *shade;
    const dr_object *objects;
    const dr_material *materials;
    const dr_alias_entry *light_table;
    const dr_alias_entry *tri_tables;
    const RenderJob *jobs;
    const WaveSegment *segs;   // this wave's segments
    uint32_t nsegs;
    uint32_t wave;             // slots of this wave
    uint32_t wave_pix;         // accumulation threads of this wave
    uint32_t chunk;            // persistent fetch size, 0 = adaptive
    // per-slot buffers
    float4 *rays;              // dr_ray, 2 x float4
    float2 *hits;
    float4 *thr, *color, *prev_p, *prev_n, *pending, *shadow_rays;
    int4 *stack;
    uint32_t *casts;
    uint32_t *slot_job, *slot_pix, *slot_sample;
    uint32_t *list[2];
    uint32_t *shadow_list;
    uint32_t *counts;          // [0, 64): active paths per bounce, [64, 128): shadow rays per bounce
    unsigned long long *work;  // persistent-kernel counters: [b] closest hit, [64 + b] shadow rays
    unsigned long long *ray_totals;  // rays of the render: [0] path rays, [1] shadow rays
    // path guiding (guided kernels only)
    float *guide_y;            // [slot][40] network output at the slot's current vertex
    float *guide_pos, *guide_nrm;  // [slot][3] network inputs
    uint32_t *guide_list;      // slots with a diffuse vertex this bounce
    uint32_t *guide_counts;    // [b] length of guide_list
    float *prev_pdf;           // [slot] solid-angle density of the last sampled diffuse direction
    float *rec;                // [slot][kGuideRecords][kRecFloats] training records
    uint32_t *rec_n;           // [slot] records; bit 31: the last one waits for its radiance
    float guide_alpha;         // probability of sampling the network's mixture
    int guide_bounces;         // bounces b < guide_bounces are guided, later ones sample the cosine lobe
    int guide_target;          // training target: 0 radiance, 1 log(1 + radiance)
    float *train_pos, *train_nrm, *train_dir, *train_w;  // training ring
    uint32_t *train_head;      // [0] rows written so far (ring position), [1] rows this wave took
    uint32_t train_cap;
};

// A training record of a diffuse vertex: position, normal, sampled
// direction, its density, luminance of the throughput after the vertex, and
// luminance of the path's colour when the next vertex is reached.
constexpr int kGuideRecords = 3;
constexpr int kRecFloats = 12;
constexpr uint32_t kRecOpen = 0x80000000u;

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 mul(F3 a, float f) { return f3(a.x * f, a.y * f, a.z * f); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 v)
{
    return f3(a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x);
}
__device__ __forceinline__ float length(F3 a) { return __fsqrt_rn(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ F3 normalized(F3 a)
{
    const float l = length(a);
    return f3(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ F3 divs(F3 a, float f) { return mul(a, 1.0f / f); }  // Vec3::operator/ multiplies by 1/f
__device__ __forceinline__ float4 mul4(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 mul4s(float4 a, float f) { return make_float4(a.x * f, a.y * f, a.z * f, a.w * f); }
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float luminance(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ float power_heuristic(float a, float b) { return a * a / (a * a + b * b); }

// areaToSolidAngle (include/Utils.hpp:236-247)
__device__ __forceinline__ float area_to_solid_angle(F3 from, F3 to, F3 to_n)
{
    const F3 diff = sub(to, from);
    const float d2 = dot(diff, diff);
    const F3 dir = normalized(diff);
    const float c = fabsf(dot(dir, to_n));
    if (c < 1e-6f) return 0.0f;
    return d2 / c;
}

// cosineWeightedHemispherePdf (include/Utils.hpp:249-254)
__device__ __forceinline__ float cosine_pdf(F3 cur, F3 next, F3 n)
{
    const F3 dir = normalized(sub(next, cur));
    const float c = dot(dir, n);
    return c > 0 ? c / kPi : 0.0f;
}

__device__ __forceinline__ void uniforms4(const RenderJob &J, uint32_t pixel, uint32_t sample, uint32_t group,
                                          float u[4])
{
    uint32_t o[4];
    pt::philox4x32_10(pixel, sample, group, kStreamTag, J.seed_lo, J.seed_hi, o);
    u[0] = pt::u01(o[0]);
    u[1] = pt::u01(o[1]);
    u[2] = pt::u01(o[2]);
    u[3] = pt::u01(o[3]);
}

// Appends `slot` to a list with one atomic per warp. Every lane of the warp
// must call it (with keep = false where it has nothing to add).
__device__ __forceinline__ void warp_append(bool keep, uint32_t slot, uint32_t *list, uint32_t *count)
{
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (mask == 0) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (keep) list[base + __popc(mask & ((1u << lane) - 1u))] = slot;
}

// cameraRay (include/tracing/CameraRay.hpp:6-34) for sample `sample` of `pixel`.
__device__ __forceinline__ void camera_ray(const RenderJob &J, uint32_t pixel, uint32_t sample, float3 &o, float3 &d)
{
    const int px = (int)(pixel % (uint32_t)J.width), py = (int)(pixel / (uint32_t)J.width);
    float subx = 0.5f, suby = 0.5f;
    if (J.pixel_sampling == DR_PIXEL_UNIFORM_RANDOM) {
        float u[4];
        uniforms4(J, pixel, sample, 0, u);
        subx = u[0];
        suby = u[1];
    }
    const float pcx = (float)px + subx, pcy = (float)py + suby;
    const float physx = pcx * J.psx - J.cx, physy = pcy * J.psy - J.cy;
    const float dx = physx / J.focal, dy = physy / J.focal;
    const F3 v = normalized(f3(dx, dy, 1.0f));
    o = make_float3(J.m[3], J.m[7], J.m[11]);
    d = make_float3(J.m[0] * v.x + J.m[1] * v.y + J.m[2] * v.z, J.m[4] * v.x + J.m[5] * v.y + J.m[6] * v.z,
                    J.m[8] * v.x + J.m[9] * v.y + J.m[10] * v.z);
}

// Segment of the wave holding `key` in the field selected by FIELD (0: slots,
// 1: accumulation threads); segments are in increasing order of both.
template <int FIELD>
__device__ __forceinline__ uint32_t find_segment(const WaveSegment *segs, uint32_t nsegs, uint32_t key)
{
    uint32_t lo = 0, hi = nsegs;  // first segment with begin > key, minus one
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t begin = FIELD == 0 ? segs[mid].slot_begin : segs[mid].pix_begin;
        if (begin <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Guided directions drawn below the surface are mirrored into the upper
// hemisphere (w - 2 (w.n) n) instead of ending the path. With it the density
// of the guided part at an upper-hemisphere direction w is q(w) + q(R w), R
// the mirror; below the surface it is 0. Every use of the guided density (the
// sampled bounce, the next-event MIS weight, the emission MIS weight through
// prev_pdf) takes this one, so the estimator stays unbiased for any network.
// Measured on the occluded-light scene (480x270, 1024 spp, 3 seeds): equal-spp
// RMSE ratio against the plain tracer 1.32 without the mirror, 1.40 with it.
#ifndef DR_GUIDE_REFLECT
#define DR_GUIDE_REFLECT 1
#endif
// Training target of a guided vertex: the radiance that arrives along its
// sampled direction, with an emitter hit there counted in full (1), or with
// its MIS weight against next-event estimation, as the image counts it (0).
#ifndef DR_GUIDE_FULL_EMISSION
#define DR_GUIDE_FULL_EMISSION 1
#endif

// Decoded mixture in the wave buffer (DR_GUIDE_DECODED): the inference
// kernel writes each guided vertex's mixture already decoded, as five arrays
// of 8 (guide_store_decoded), and the shading kernel reads them from memory at
// each use, lobe by lobe, instead of holding the mixture in registers across
// next-event estimation, so it runs with more warps per SM. Measured on the
// occluded-light scene (480x270, 64 spp, frozen network): guided shading
// 7.1 -> 5.4 ms over its 16 launches.
#ifndef DR_GUIDE_DECODED
#define DR_GUIDE_DECODED 1
#endif
#ifndef DR_GUIDE_SHADE_BLOCKS
#define DR_GUIDE_SHADE_BLOCKS (DR_GUIDE_DECODED ? 6 : 4)
#endif

#if !DR_GUIDE_DECODED
// The mixture held in registers (GuideMix), decoded by the shading kernel.
__device__ __forceinline__ float guide_mix_pdf(const GuideMix &M, F3 w)
{
    float p = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        const float c = M.mx[j] * w.x + M.my[j] * w.y + M.mz[j] * w.z;
        p += M.c[j] * __expf(M.kappa[j] * (c - 1.0f));
    }
    return p;
}

// Lobe by u0 (cumulative weights, as guide_sample), then its vMF by (u1, u2).
__device__ __forceinline__ F3 guide_mix_sample(const GuideMix &M, float u0, float u1, float u2)
{
    float k = M.kappa[0], ax = M.mx[0], ay = M.my[0], az = M.mz[0];
    float acc = M.pi[0];
#pragma unroll
    for (int j = 1; j < kGuideLobes; ++j) {
        if (u0 >= acc) k = M.kappa[j], ax = M.mx[j], ay = M.my[j], az = M.mz[j];
        acc += M.pi[j];
    }
    float wx, wy, wz;
    vmf_sample(k, ax, ay, az, u1, u2, wx, wy, wz);
    return f3(wx, wy, wz);
}

// Density of the guided part at w, for a surface of normal n.
__device__ __forceinline__ float guide_pdf_above(const GuideMix &M, F3 w, F3 n)
{
#if DR_GUIDE_REFLECT
    const float c = dot(w, n);
    if (!(c > 0.0f)) return 0.0f;
    const F3 r = sub(w, mul(n, 2.0f * c));
    return guide_mix_pdf(M, w) + guide_mix_pdf(M, r);
#else
    return guide_mix_pdf(M, w);
#endif
}
#endif

#if DR_GUIDE_DECODED
// Density of the guided part at w above a surface of normal n, from the
// decoded mixture (the mirrored direction in the same pass over the lobes).
__device__ __forceinline__ float guide_dec_pdf_above(const float *y, F3 w, F3 n)
{
    const float cn = dot(w, n);
#if DR_GUIDE_REFLECT
    if (!(cn > 0.0f)) return 0.0f;
#endif
    const F3 r = sub(w, mul(n, 2.0f * cn));
    float p = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; ++j) {
        const float c = y[j], k = y[8 + j], mx = y[16 + j], my = y[24 + j], mz = y[32 + j];
        p += c * __expf(k * (mx * w.x + my * w.y + mz * w.z - 1.0f));
#if DR_GUIDE_REFLECT
        p += c * __expf(k * (mx * r.x + my * r.y + mz * r.z - 1.0f));
#endif
    }
    return p;
}

// Lobe by u0 over the weights pi_j = c_j 2 pi (1 - e^{-2 kappa_j}) / kappa_j,
// then its vMF by (u1, u2). The weights recovered here (fast exponential and
// division) differ from those folded into c_j by about 1e-6 relative, which
// is the mismatch between the sampled and the evaluated density.
__device__ __forceinline__ F3 guide_dec_sample(const float *y, float u0, float u1, float u2)
{
    int sel = 0;
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes - 1; ++j) {
        const float k = y[8 + j];
        acc += __fdividef(y[j] * 6.28318530718f * (1.0f - __expf(-2.0f * k)), k);
        if (u0 >= acc) sel = j + 1;
    }
    float wx, wy, wz;
    vmf_sample(y[8 + sel], y[16 + sel], y[24 + sel], y[32 + sel], u1, u2, wx, wy, wz);
    return f3(wx, wy, wz);
}
#endif

// The guided density and sampler the shading kernel uses.
#if DR_GUIDE_DECODED
__device__ __forceinline__ float guide_density(const float *y, F3 w, F3 n) { return guide_dec_pdf_above(y, w, n); }
__device__ __forceinline__ F3 guide_draw(const float *y, float u0, float u1, float u2)
{
    return guide_dec_sample(y, u0, u1, u2);
}
#else
__device__ __forceinline__ float guide_density(const GuideMix &M, F3 w, F3 n) { return guide_pdf_above(M, w, n); }
__device__ __forceinline__ F3 guide_draw(const GuideMix &M, float u0, float u1, float u2)
{
    return guide_mix_sample(M, u0, u1, u2);
}
#endif

__global__ void __launch_bounds__(kRenderBlock) k_camera(RenderParams p)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) p.counts[0] = p.wave;
    if (i >= p.wave) return;
    const WaveSegment sg = p.segs[find_segment<0>(p.segs, p.nsegs, i)];
    const RenderJob &J = p.jobs[sg.job];
    const uint32_t local = i - sg.slot_begin;
    const uint32_t pixel = local % sg.npix;
    const uint32_t sample = J.sample_offset + sg.sample_rel + local / sg.npix;
    float3 o, d;
    camera_ray(J, pixel, sample, o, d);
    p.rays[2 * i] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
    p.rays[2 * i + 1] = make_float4(d.x, d.y, d.z, 0.0f);
    p.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    p.color[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    p.prev_p[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // w = 0: no diffuse vertex before
    p.stack[i] = make_int4(0, 0, 0, 0);                 // w = size
    p.casts[i] = 0;
    p.slot_job[i] = sg.job;
    p.slot_pix[i] = pixel;
    p.slot_sample[i] = sample;
    if (p.rec_n) p.rec_n[i] = 0;
    p.list[0][i] = i;
}

// First-hit debug views: sampleColorDebug (UV checker) and the debug branch of
// sampleColor (barycentrics, winding order), include/tracing/PathGeneration.hpp:
// 274-299, 393-429. One thread per pixel adds its samples in order. The
// reference's hit uv is always (0, 0) (IntersectionTestsImpl.hpp:58), so the
// checker pattern is its dark colour 0.5 everywhere; the UV view adds a sample
// (w + 1) only where the camera ray hits.
template <int MODE, int LAYOUT>
__global__ void __launch_bounds__(kRenderBlock) k_debug(SceneArrays p, RenderJob J, int view)
{
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= J.npix) return;
    float4 acc = J.accum[pixel];
    uint32_t casts = 0;
    for (uint32_t k = 0; k < J.spp; ++k) {
        float3 o, d;
        camera_ray(J, pixel, J.sample_offset + k, o, d);
        DevRay r;
        const bool valid = make_dev_ray(o, d, __int_as_float(0x7f800000), r);
        float t = r.tmax;
        int32_t prim = INT_MAX;
        TraceStats st;
        if (valid) scene_closest<MODE, false, LAYOUT>(p.trace, r, J.root, t, prim, st);
        ++casts;
        float4 color = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bool counted = true;
        if (prim != INT_MAX) {
            const float4 s0 = p.shade[3 * prim], s1 = p.shade[3 * prim + 1], s2 = p.shade[3 * prim + 2];
            const dr_material &m = p.materials[__float_as_int(s2.z)];
            if (view == DR_DEBUG_UV_CHECKER) {
                color = mul4(make_float4(0.5f, 0.5f, 0.5f, 0.0f),
                             make_float4(m.debug_color[0], m.debug_color[1], m.debug_color[2], m.debug_color[3]));
            } else {
                // testTriangleIntersection's barycentrics and the ccw flag of
                // getIntersectionTris, in the reference's expression order
                const F3 A = f3(s0.x, s0.y, s0.z), B = f3(s0.w, s1.x, s1.y), C = f3(s1.z, s1.w, s2.x);
                const F3 v = f3(d.x, d.y, d.z);
                const F3 nf = cross(sub(A, B), sub(A, C));
                if (view == DR_DEBUG_BARI_COORDS) {
                    const float s2a = dot(nf, nf);
                    const F3 hp = add(f3(o.x, o.y, o.z), mul(v, t));
                    const F3 n1 = cross(sub(hp, A), sub(C, A));
                    const F3 n2 = cross(sub(B, A), sub(hp, A));
                    const float wB = dot(nf, n1) / s2a, wC = dot(nf, n2) / s2a;
                    const float wA = 1 - wB - wC;
                    color = make_float4(wA, wB, wC, 0.0f);
                } else {
                    color = dot(nf, v) > 0 ? make_float4(1.0f, 0.73f, 0.47f, 0.0f) : make_float4(0.53f, 0.82f, 1.0f, 0.0f);
                }
            }
        } else if (view == DR_DEBUG_UV_CHECKER) {
            counted = false;
        }
        if (counted) {
            acc.w = acc.w + 1.0f;
            acc = add4(acc, color);
        }
    }
    J.accum[pixel] = acc;
    if (J.pix_casts) J.pix_casts[pixel] += casts;
}

// Ray sources of the persistent wide kernels: list entry i names a path slot,
// whose job names the hierarchy root.
struct PathSource {
    const uint32_t *list;
    const float4 *rays;
    float2 *hits;
    const uint32_t *slot_job;
    const RenderJob *jobs;
    __device__ __forceinline__ bool load(uint64_t i, DevRay &r, uint32_t &root) const
    {
        const uint32_t slot = list[i];
        root = jobs[slot_job[slot]].root;
        return load_ray(reinterpret_cast<const dr_ray *>(rays), slot, r);
    }
    __device__ __forceinline__ void closest(uint64_t i, float t, int32_t prim) const
    {
        hits[list[i]] = prim != INT_MAX ? make_float2(t, __int_as_float(prim))
                                        : make_float2(__int_as_float(0x7f800000), __int_as_float(-1));
    }
    __device__ __forceinline__ void any(uint64_t, bool) const {}
};

struct ShadowSource {
    const uint32_t *list;
    const float4 *rays;
    float4 *color;
    const float4 *pending;
    const uint32_t *slot_job;
    const RenderJob *jobs;
    __device__ __forceinline__ bool load(uint64_t i, DevRay &r, uint32_t &root) const
    {
        const uint32_t slot = list[i];
        root = jobs[slot_job[slot]].root;
        return load_ray(reinterpret_cast<const dr_ray *>(rays), slot, r);
    }
    __device__ __forceinline__ void closest(uint64_t, float, int32_t) const {}
    __device__ __forceinline__ void any(uint64_t i, bool occluded) const
    {
        if (!occluded) {
            const uint32_t slot = list[i];
            const float4 c = color[slot], q = pending[slot];
            color[slot] = make_float4(c.x + q.x, c.y + q.y, c.z + q.z, c.w + q.w);
        }
    }
};

// STACK: shared-memory entries of each lane's traversal stack (kStackDepths).
template <int MODE, int STACK>
__global__ void __launch_bounds__(kTraceBlock, kP8MinBlocks) k_wave_closest_p8(RenderParams p, int b)
{
    const Wide8Args w{p.trace.nodes8, p.trace.tri_ref, p.trace.tri_wt, p.trace.prim, p.trace.num_nodes, p.trace.error,
                      p.trace.stack_limit};
    const PathSource src{p.list[b & 1], p.rays, p.hits, p.slot_job, p.jobs};
    unsigned long long nn = 0, nb = 0, nt = 0, nh = 0;
    persistent_wide<MODE, false, false, DR_TRI_BATCH_PATHS != 0, STACK>(w, src, p.counts[b], p.work + b, nn, nb, nt,
                                                                         nh, p.chunk);
}

template <int MODE, int STACK>
__global__ void __launch_bounds__(kTraceBlock, kP8MinBlocks) k_wave_shadow_p8(RenderParams p, int b)
{
    const Wide8Args w{p.trace.nodes8, p.trace.tri_ref, p.trace.tri_wt, p.trace.prim, p.trace.num_nodes, p.trace.error,
                      p.trace.stack_limit};
    const ShadowSource src{p.shadow_list, p.shadow_rays, p.color, p.pending, p.slot_job, p.jobs};
    unsigned long long nn = 0, nb = 0, nt = 0, nh = 0;
    persistent_wide<MODE, true, false, DR_TRI_BATCH_SHADOW != 0, STACK>(w, src, p.counts[64 + b], p.work + 64 + b, nn,
                                                                      nb, nt, nh, p.chunk);
}

// The persistent traversal kernels of one (triangle test, stack depth).
struct P8Kernels {
    void (*closest)(RenderParams, int);
    void (*shadow)(RenderParams, int);
};

template <int MODE, int STACK>
constexpr P8Kernels p8_kernels()
{
    return P8Kernels{k_wave_closest_p8<MODE, STACK>, k_wave_shadow_p8<MODE, STACK>};
}

P8Kernels select_p8(int tri_mode, uint32_t stack)
{
    const bool wt = tri_mode == DR_TRI_WATERTIGHT;
    switch (stack) {
    case 4: return wt ? p8_kernels<1, 4>() : p8_kernels<0, 4>();
    case 16: return wt ? p8_kernels<1, 16>() : p8_kernels<0, 16>();
    default: return wt ? p8_kernels<1, 8>() : p8_kernels<0, 8>();
    }
}

// Closest hit of the surviving paths of bounce b (binary hierarchy).
template <int MODE, int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock) k_wave_closest(RenderParams p, int b)
{
    const uint32_t count = p.counts[b];
    const uint32_t *list = p.list[b & 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = list[i];
        DevRay r;
        const bool valid = load_ray(reinterpret_cast<const dr_ray *>(p.rays), slot, r);
        float t = r.tmax;
        int32_t prim = INT_MAX;
        TraceStats st;
        if (valid) scene_closest<MODE, false, LAYOUT>(p.trace, r, p.jobs[p.slot_job[slot]].root, t, prim, st);
        p.hits[slot] = prim != INT_MAX ? make_float2(t, __int_as_float(prim))
                                       : make_float2(__int_as_float(0x7f800000), __int_as_float(-1));
    }
}

__device__ __forceinline__ float object_ior(const RenderParams &p, int obj)
{
    const dr_material &m = p.materials[p.objects[obj].material];
    return m.kind == DR_MAT_DIELECTRIC ? m.ior : 1.0f;
}

template <bool GUIDED>
__global__ void __launch_bounds__(kRenderBlock, GUIDED ? DR_GUIDE_SHADE_BLOCKS : kShadeMinBlocks) k_shade(RenderParams p, int b)
{
    const uint32_t count = p.counts[b];
    const uint32_t *list = p.list[b & 1];
    uint32_t *next_list = p.list[(b + 1) & 1];
    // warp-uniform loop so that every lane reaches the ballots
    const uint32_t warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp_first; base < count; base += stride) {
        const uint32_t i = base + (threadIdx.x & 31);
        bool keep = false, shadow = false, dead = false;
        uint32_t slot = 0;
        if (i < count) {
            slot = list[i];
            p.casts[slot] += 1;
            const RenderJob &J = p.jobs[p.slot_job[slot]];
            float *closed = nullptr;  // guided: the record this vertex closes
            if (GUIDED && p.rec_n) {
                // the radiance gathered before this vertex closes the last record
                const uint32_t rn = p.rec_n[slot];
                if (rn & kRecOpen) {
                    const uint32_t r = (rn & ~kRecOpen) - 1;
                    closed = p.rec + ((size_t)slot * kGuideRecords + r) * kRecFloats;
                    closed[11] = luminance(p.color[slot]);
                    p.rec_n[slot] = rn & ~kRecOpen;
                }
            }
            const float2 h = p.hits[slot];
            const int prim = __float_as_int(h.y);
            if (prim >= 0) {
                const float t = h.x;
                const float4 r0 = p.rays[2 * slot], r1 = p.rays[2 * slot + 1];
                const F3 ro = f3(r0.x, r0.y, r0.z), rv = f3(r1.x, r1.y, r1.z);
                const float4 s0 = __ldg(p.shade + 3 * prim), s1 = __ldg(p.shade + 3 * prim + 1),
                             s2 = __ldg(p.shade + 3 * prim + 2);
                const F3 A = f3(s0.x, s0.y, s0.z), B = f3(s0.w, s1.x, s1.y), C = f3(s1.z, s1.w, s2.x);
                const int obj = __float_as_int(s2.y), mat_id = __float_as_int(s2.z);
                // getIntersectionTris (IntersectionTestsImpl.hpp:36-67), identity transform
                F3 n = normalized(cross(sub(A, B), sub(A, C)));
                if (dot(n, rv) > 0) n = mul(n, -1.0f);
                n = normalized(f3(n.x * 1.0f, n.y * 1.0f, n.z * 1.0f));
                F3 hp = add(ro, mul(rv, t));
                hp = f3(hp.x * 1.0f + 0.0f, hp.y * 1.0f + 0.0f, hp.z * 1.0f + 0.0f);
                const dr_material &M = p.materials[mat_id];
                float4 thr = p.thr[slot];
                float4 col = p.color[slot];
                const float4 pp4 = p.prev_p[slot];
                const uint32_t pixel = p.slot_pix[slot], sample = p.slot_sample[slot];
                float u[12];
                const uint32_t g = 1u + 3u * (uint32_t)b;
                uniforms4(J, pixel, sample, g, u);
                F3 normal = n;
                F3 new_o, new_v;
                if (M.kind == DR_MAT_DIFFUSE) {
                    const float4 E = make_float4(M.emission[0], M.emission[1], M.emission[2], M.emission[3]);
                    const float4 alb = make_float4(M.albedo[0], M.albedo[1], M.albedo[2], M.albedo[3]);
                    // misWeightedEmission (PathGeneration.hpp:306-318) with the
                    // pdfs of computeNextBounceMisPdfs (:320-334) for (prev, this)
                    if (pp4.w == 0.0f) {
                        col = add4(col, mul4(E, thr));
                    } else {
                        const float4 pn4 = p.prev_n[slot];
                        const F3 pp = f3(pp4.x, pp4.y, pp4.z), pn = f3(pn4.x, pn4.y, pn4.z);
                        // guided: the density of the direction actually sampled there
                        const float pdf_bsdf = GUIDED ? p.prev_pdf[slot] : cosine_pdf(pp, hp, pn);
                        const float L = luminance(mul4s(E, kPi));
                        const float pdf_area = L / J.total_power;
                        const float pdf_nee = pdf_area * area_to_solid_angle(pp, hp, n);
                        if (pdf_bsdf + pdf_nee > 0) {
                            const float wm = power_heuristic(pdf_bsdf, pdf_nee);
                            col = add4(col, mul4s(mul4(E, thr), wm));
#if DR_GUIDE_FULL_EMISSION
                            // training only: the emission's share left to next-event
                            // estimation (1 - wm) counts in the closed record's target
                            if (GUIDED && closed) closed[11] -= luminance(mul4(E, thr)) * (1.0f - wm);
#endif
                        }
                    }
                    const float alpha = GUIDED && b < p.guide_bounces ? p.guide_alpha : 0.0f;
#if DR_GUIDE_DECODED
                    const float *lobes = GUIDED ? p.guide_y + (size_t)slot * kGuideOut : nullptr;
#else
                    GuideMix lobes;
                    if (GUIDED && alpha > 0.0f) lobes = guide_mix(p.guide_y + (size_t)slot * kGuideOut);
#endif
                    // next-event estimation: samplePointOnLights (:234-272) and
                    // evaluateDirectLighting (:336-361); visibility is the shadow ray
                    if (J.lights) {
                        uniforms4(J, pixel, sample, g + 1, u + 4);
                        uniforms4(J, pixel, sample, g + 2, u + 8);
                        int32_t oi, ti;
                        float opdf, tpdf;
                        alias_sample(p.light_table + J.obj_base, J.num_objects, u[3], u[4], oi, opdf);
                        const dr_object ob = p.objects[J.obj_base + oi];
                        alias_sample(p.tri_tables + ob.tri_begin, ob.tri_count, u[5], u[6], ti, tpdf);
                        const int lt = (int)ob.tri_begin + ti;
                        const float4 l0 = __ldg(p.shade + 3 * lt), l1 = __ldg(p.shade + 3 * lt + 1),
                                     l2 = __ldg(p.shade + 3 * lt + 2);
                        const F3 LA = f3(l0.x, l0.y, l0.z), LB = f3(l0.w, l1.x, l1.y), LC = f3(l1.z, l1.w, l2.x);
                        float uu = u[7], vv = u[8];
                        if (uu + vv > 1) {
                            uu = 1 - uu;
                            vv = 1 - vv;
                        }
                        F3 lp = add(add(LA, mul(sub(LB, LA), uu)), mul(sub(LC, LA), vv));
                        const F3 Aw = f3(LA.x * 1.0f, LA.y * 1.0f, LA.z * 1.0f);
                        const F3 Bw = f3(LB.x * 1.0f, LB.y * 1.0f, LB.z * 1.0f);
                        const F3 Cw = f3(LC.x * 1.0f, LC.y * 1.0f, LC.z * 1.0f);
                        const F3 perp = cross(sub(Aw, Bw), sub(Aw, Cw));
                        const float plen = length(perp);
                        const F3 ln = divs(perp, plen);
                        const float area = plen / 2.0f;
                        const float lpdf = opdf * tpdf / area;
                        lp = f3(lp.x * 1.0f + 0.0f, lp.y * 1.0f + 0.0f, lp.z * 1.0f + 0.0f);
                        const dr_material &LM = p.materials[ob.material];
                        float nee_pdf_bsdf = cosine_pdf(hp, lp, n);
                        if (GUIDED && alpha > 0.0f) {
                            const F3 wl0 = normalized(sub(lp, hp));
                            nee_pdf_bsdf = alpha * guide_density(lobes, wl0, n) + (1.0f - alpha) * nee_pdf_bsdf;
                        }
                        const float nee_pdf_nee = lpdf * area_to_solid_angle(hp, lp, ln);
                        const float dist = length(sub(lp, hp));
                        const F3 wl = divs(sub(lp, hp), dist);
                        const float cos_s = dot(wl, n);
                        const float cos_l = dot(wl, ln);
                        if (cos_s > 0 && nee_pdf_nee + nee_pdf_bsdf > 0) {
                            const float4 brdf = mul4s(alb, 1.0f / kPi);
                            const float G = cos_s * fabsf(cos_l) / (dist * dist);
                            const float4 LE = make_float4(LM.emission[0], LM.emission[1], LM.emission[2],
                                                          LM.emission[3]);
                            const float4 Ld = mul4s(mul4s(mul4(LE, brdf), G), 1.0f / lpdf);
                            p.pending[slot] = mul4s(mul4(Ld, thr), power_heuristic(nee_pdf_nee, nee_pdf_bsdf));
                            // visible(): ray from p0 + v 1e-5, occluded when a hit has
                            // t <= distance - 2e-5 (evaluated in double)
                            const F3 so = add(hp, mul(wl, 1e-5f));
                            const float tmax = __double2float_rd((double)dist - 1e-5 * 2);
                            p.shadow_rays[2 * slot] = make_float4(so.x, so.y, so.z, tmax);
                            p.shadow_rays[2 * slot + 1] = make_float4(wl.x, wl.y, wl.z, 0.0f);
                            shadow = true;
                        }
                    }
                    if (GUIDED && !J.lights) uniforms4(J, pixel, sample, g + 2, u + 8);
                    bool cosine = true;
                    if (GUIDED && u[9] < alpha) {
                        cosine = false;
                        new_v = guide_draw(lobes, u[10], u[0], u[1]);
#if DR_GUIDE_REFLECT
                        // a direction below the surface is mirrored into the upper
                        // hemisphere (guide_pdf_above is the density of the result)
                        const float cb = dot(new_v, n);
                        if (cb < 0.0f) new_v = sub(new_v, mul(n, 2.0f * cb));
#endif
                    }
                    if (cosine) {
                        // cosineWeightedHemisphereSample (DistributionSamplers.hpp:33-42)
                        const float theta0 = 2 * kPi * u[0];
                        const float theta1 = pt::acos(1 - 2 * u[1]);
                        float sn0, cs0, sn1, cs1;
                        pt::sincos(theta0, sn0, cs0);
                        pt::sincos(theta1, sn1, cs1);
                        const F3 sph = f3(sn1 * sn0, sn1 * cs0, cs1);
                        new_v = normalized(add(sph, normal));
                    }
                    if (GUIDED) {
                        // one-sample MIS over the mixture and the cosine lobe: f cos / pdf_mix
                        const float c = dot(new_v, n);
                        const float pdf_mix = (alpha > 0.0f ? alpha * guide_density(lobes, new_v, n) : 0.0f) +
                                              (1.0f - alpha) * fmaxf(c, 0.0f) / kPi;
                        const float f = c > 0.0f && pdf_mix > 0.0f ? c / (kPi * pdf_mix) : 0.0f;
                        thr = mul4s(mul4(thr, alb), f);
                        p.prev_pdf[slot] = pdf_mix;
                        if (f == 0.0f) dead = true;
                        const uint32_t rn = p.rec_n ? p.rec_n[slot] : (uint32_t)kGuideRecords;
                        if (!dead && alpha > 0.0f && rn < (uint32_t)kGuideRecords && b + 1 < (int)J.max_depth) {
                            // 48-byte record as three 16-byte stores: hit point, normal,
                            // direction, density, throughput (word 11, the radiance at
                            // the next vertex, is written when that vertex closes it)
                            float4 *rc = reinterpret_cast<float4 *>(p.rec + ((size_t)slot * kGuideRecords + rn) * kRecFloats);
                            rc[0] = make_float4(hp.x, hp.y, hp.z, n.x);
                            rc[1] = make_float4(n.y, n.z, new_v.x, new_v.y);
                            rc[2] = make_float4(new_v.z, pdf_mix, luminance(thr), 0.0f);
                            p.rec_n[slot] = (rn + 1) | kRecOpen;
                        }
                    } else {
                        thr = mul4(thr, alb);
                    }
                    new_o = hp;
                    p.prev_p[slot] = make_float4(hp.x, hp.y, hp.z, 1.0f);
                    p.prev_n[slot] = make_float4(n.x, n.y, n.z, 0.0f);
                } else {
                    // transparent branch of generateNewRay (PathGeneration.hpp:138-208),
                    // including Stack::top() popping (:64-67); capacity 3
                    int4 st = p.stack[slot];
                    int stk[3] = {st.x, st.y, st.z};
                    int ss = st.w;
                    float n1, n2;
                    if (ss > 0 && stk[ss - 1] == obj) {
                        n1 = M.ior;
                        --ss;
                        if (ss == 0) n2 = 1;
                        else n2 = object_ior(p, stk[--ss]);
                        if (ss < 3) stk[ss++] = obj;
                    } else {
                        n2 = M.ior;
                        if (ss == 0) n1 = 1;
                        else n1 = object_ior(p, stk[--ss]);
                    }
                    const float eta = n1 / n2;
                    const float d = dot(rv, normal);
                    const float k = 1 - eta * eta * (1 - d * d);
                    if (n1 > n2 && k < 0) {
                        new_v = sub(rv, mul(mul(normal, 2.0f), d));
                    } else {
                        const float rr = (n1 - n2) / (n1 + n2);
                        const float R0 = rr * rr;
                        const float cosT1 = 1 - (-d);
                        const float c2 = cosT1 * cosT1;
                        const float c4 = c2 * c2;
                        const float c5 = c4 * cosT1;
                        const float F = (float)((double)R0 + (1.0 - (double)R0) * (double)c5);
                        if (u[2] < F) {
                            new_v = sub(rv, mul(mul(normal, 2.0f), d));
                        } else {
                            if (ss > 0 && stk[ss - 1] == obj) --ss;
                            else if (ss < 3) stk[ss++] = obj;
                            normal = mul(normal, -1.0f);
                            const float dotp = -d;
                            new_v = add(mul(normal, __fsqrt_rn(k) - dotp * eta), mul(rv, eta));
                        }
                    }
                    new_o = hp;
                    p.stack[slot] = make_int4(stk[0], stk[1], stk[2], ss);
                    p.prev_p[slot] = make_float4(hp.x, hp.y, hp.z, 0.0f);
                }
                new_o = add(new_o, mul(normal, 1e-5f));
                p.rays[2 * slot] = make_float4(new_o.x, new_o.y, new_o.z, __int_as_float(0x7f800000));
                p.rays[2 * slot + 1] = make_float4(new_v.x, new_v.y, new_v.z, 0.0f);
                p.thr[slot] = thr;
                p.color[slot] = col;
                keep = b + 1 < (int)J.max_depth && !dead;
            }
        }
        warp_append(keep, slot, next_list, p.counts + b + 1);
        warp_append(shadow, slot, p.shadow_list, p.counts + 64 + b);
    }
}

// Network inputs of the bounce's diffuse vertices (hit point, normal facing
// the incoming ray, as the shading computes them) and their slot list.
__global__ void __launch_bounds__(kRenderBlock) k_guide_prepare(RenderParams p, int b)
{
    const uint32_t count = p.counts[b];
    const uint32_t *list = p.list[b & 1];
    const uint32_t warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u));
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp_first; base < count; base += stride) {
        const uint32_t i = base + (threadIdx.x & 31);
        bool diffuse = false;
        uint32_t slot = 0;
        if (i < count) {
            slot = list[i];
            const float2 h = p.hits[slot];
            const int prim = __float_as_int(h.y);
            if (prim >= 0) {
                const float4 s0 = __ldg(p.shade + 3 * prim), s1 = __ldg(p.shade + 3 * prim + 1),
                             s2 = __ldg(p.shade + 3 * prim + 2);
                const dr_material &M = p.materials[__float_as_int(s2.z)];
                if (M.kind == DR_MAT_DIFFUSE) {
                    diffuse = true;
                    const float4 r0 = p.rays[2 * slot], r1 = p.rays[2 * slot + 1];
                    const F3 ro = f3(r0.x, r0.y, r0.z), rv = f3(r1.x, r1.y, r1.z);
                    const F3 A = f3(s0.x, s0.y, s0.z), B = f3(s0.w, s1.x, s1.y), C = f3(s1.z, s1.w, s2.x);
                    F3 n = normalized(cross(sub(A, B), sub(A, C)));
                    if (dot(n, rv) > 0) n = mul(n, -1.0f);
                    const F3 hp = add(ro, mul(rv, h.x));
                    float *gp = p.guide_pos + 3 * (size_t)slot, *gn = p.guide_nrm + 3 * (size_t)slot;
                    gp[0] = hp.x, gp[1] = hp.y, gp[2] = hp.z;
                    gn[0] = n.x, gn[1] = n.y, gn[2] = n.z;
                }
            }
        }
        warp_append(diffuse, slot, p.guide_list, p.guide_counts + b);
    }
}

// Training samples of the finished wave: for each closed record, the
// radiance that arrived along the sampled direction, L = (colour at the end -
// colour when the next vertex was reached) / throughput after the vertex, and
// the weight L cos / pdf of that direction (target density L cos). The
// samples go to the training ring (train_cap rows, written round robin, so
// rows a small wave does not reach keep the previous waves' samples). A wave
// writes at most train_cap samples: each warp counts its samples against the
// wave's quota with one atomic (counter [1], reset before this kernel) and
// takes its ring rows with a second one, and warps that find the quota spent
// stop. A large wave (1080p: 33 M paths, about 80 M samples) so costs
// O(train_cap) writes and one atomic per warp, not one per sample. The
// samples kept are then the first ones of the wave (its first samples of
// every pixel); keeping the last ones instead (the ring written by every
// sample) or a scrambled subset trained no better (480x270, 1024 spp, 6
// seeds: equal-spp RMSE ratios 1.35, 1.34, 1.30).
__global__ void __launch_bounds__(256) k_guide_collect(RenderParams p)
{
    constexpr unsigned FULL = 0xffffffffu;
    if (*reinterpret_cast<volatile uint32_t *>(p.train_head + 1) >= p.train_cap) return;  // quota spent
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t n = 0;
    float cf = 0.0f;
    if (slot < p.wave) {
        const uint32_t rn = p.rec_n[slot];
        n = (rn & ~kRecOpen) - ((rn & kRecOpen) ? 1u : 0u);
        if (n) cf = luminance(p.color[slot]);
    }
    float w[kGuideRecords];
    uint32_t take = 0;  // bit r: record r is a sample
#pragma unroll
    for (int r = 0; r < kGuideRecords; ++r) {
        w[r] = 0.0f;
        if ((uint32_t)r >= n) continue;
        const float4 *rq = reinterpret_cast<const float4 *>(p.rec + ((size_t)slot * kGuideRecords + r) * kRecFloats);
        const float4 q0 = rq[0], q1 = rq[1], q2 = rq[2];
        const float T = q2.z, cn = q2.w;
        float L = (cf - cn) / T;
        if (p.guide_target == 1) L = log1pf(fmaxf(L, 0.0f));
        const float c = q0.w * q1.z + q1.x * q1.w + q1.y * q2.x;  // normal . direction
        w[r] = L * fmaxf(c, 0.0f) / q2.y;
        if ((T > 0.0f) && (w[r] > 0.0f) && isfinite(w[r])) take |= 1u << r;
    }
    const uint32_t cnt = (uint32_t)__popc(take);
    uint32_t incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    if (total == 0) return;  // warp-uniform
    uint32_t base = 0, allowed = 0;
    if (lane == 31) {
        const uint32_t used = atomicAdd(p.train_head + 1, total);
        allowed = used >= p.train_cap ? 0u : min(total, p.train_cap - used);
        if (allowed) base = atomicAdd(p.train_head, allowed);
    }
    allowed = __shfl_sync(FULL, allowed, 31);
    if (allowed == 0) return;  // warp-uniform: the wave's quota is spent
    base = __shfl_sync(FULL, base, 31);
    // this lane's samples are the warp's samples [incl - cnt, incl); those at
    // or beyond `allowed` are dropped
    uint32_t k = incl - cnt;
    for (uint32_t m = take; m != 0 && k < allowed; m &= m - 1u, ++k) {
        const int r = __ffs(m) - 1;
        const uint32_t at = (base + k) % p.train_cap;
        const float *rc = p.rec + ((size_t)slot * kGuideRecords + r) * kRecFloats;
        for (int a = 0; a < 3; ++a) {
            p.train_pos[3 * (size_t)at + a] = rc[a];
            p.train_nrm[3 * (size_t)at + a] = rc[3 + a];
            p.train_dir[3 * (size_t)at + a] = rc[6 + a];
        }
        p.train_w[at] = w[r];
    }
}

// Shadow rays of bounce b: the next-event contribution counts when unoccluded.
template <int MODE, int LAYOUT>
__global__ void __launch_bounds__(kTraceBlock) k_wave_shadow(RenderParams p, int b)
{
    const uint32_t count = p.counts[64 + b];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = p.shadow_list[i];
        DevRay r;
        const bool valid = load_ray(reinterpret_cast<const dr_ray *>(p.shadow_rays), slot, r);
        const bool occluded = valid && scene_any<MODE, LAYOUT>(p.trace, r, p.jobs[p.slot_job[slot]].root);
        if (!occluded) p.color[slot] = add4(p.color[slot], p.pending[slot]);
    }
}

// Buffers::color update of the reference (pixel.w++; pixel = pixel + color) for
// the wave's samples: one thread per (segment, pixel) adds the segment's samples
// in sample order. Waves run this pass one after another.
__global__ void __launch_bounds__(256) k_accumulate_wave(RenderParams p)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.wave_pix) return;
    const WaveSegment sg = p.segs[find_segment<1>(p.segs, p.nsegs, t)];
    const RenderJob &J = p.jobs[sg.job];
    const uint32_t pix = t - sg.pix_begin;
    float4 acc = J.accum[pix];
    uint32_t casts = 0;
    for (uint32_t s = 0; s < sg.nsamples; ++s) {
        const uint32_t slot = sg.slot_begin + s * sg.npix + pix;
        acc.w = acc.w + 1.0f;
        acc = add4(acc, p.color[slot]);
        casts += p.casts[slot];
    }
    J.accum[pix] = acc;
    if (J.pix_casts) J.pix_casts[pix] += casts;
    if (t == 0) {
        // the wave's traced rays: paths per bounce and shadow rays per bounce
        unsigned long long np = 0, ns = 0;
        for (int b = 0; b < 64; ++b) {
            np += p.counts[b];
            ns += p.counts[64 + b];
        }
        atomicAdd(p.ray_totals, np);
        atomicAdd(p.ray_totals + 1, ns);
    }
}

template <typename T>
T *carve(char *&ptr, size_t count)
{
    T *out = reinterpret_cast<T *>(ptr);
    ptr += (count * sizeof(T) + 255) & ~size_t(255);
    return out;
}

constexpr size_t kSlotBytes = 2 * 16 + 8 + 16 * 5 + 2 * 16 + 16 + 4 * 7;

constexpr size_t kGuideSlotBytes = kGuideOut * 4 + 3 * 4 + 3 * 4 + 4 + 4 + kGuideRecords * kRecFloats * 4 + 4;

size_t wave_buffer_bytes(uint32_t W, bool guided)
{
    return (size_t)W * (kSlotBytes + (guided ? kGuideSlotBytes : 0)) + 192 * sizeof(uint32_t) +
           128 * sizeof(unsigned long long) + 28 * 256;
}

RenderParams wave_params(const SceneArrays &sc, const RenderJob *d_jobs, void *buffer, uint32_t W, uint32_t chunk,
                         bool guided)
{
    RenderParams p{};
    p.trace = sc.trace;
    p.shade = sc.shade;
    p.objects = sc.objects;
    p.materials = sc.materials;
    p.light_table = sc.light_table;
    p.tri_tables = sc.tri_tables;
    p.jobs = d_jobs;
    p.chunk = chunk;
    char *ptr = static_cast<char *>(buffer);
    p.rays = carve<float4>(ptr, (size_t)W * 2);
    p.hits = carve<float2>(ptr, W);
    p.thr = carve<float4>(ptr, W);
    p.color = carve<float4>(ptr, W);
    p.prev_p = carve<float4>(ptr, W);
    p.prev_n = carve<float4>(ptr, W);
    p.pending = carve<float4>(ptr, W);
    p.shadow_rays = carve<float4>(ptr, (size_t)W * 2);
    p.stack = carve<int4>(ptr, W);
    p.casts = carve<uint32_t>(ptr, W);
    p.slot_job = carve<uint32_t>(ptr, W);
    p.slot_pix = carve<uint32_t>(ptr, W);
    p.slot_sample = carve<uint32_t>(ptr, W);
    p.list[0] = carve<uint32_t>(ptr, W);
    p.list[1] = carve<uint32_t>(ptr, W);
    p.shadow_list = carve<uint32_t>(ptr, W);
    p.counts = carve<uint32_t>(ptr, 128);
    p.work = carve<unsigned long long>(ptr, 128);
    if (guided) {
        p.guide_y = carve<float>(ptr, (size_t)W * kGuideOut);
        p.guide_pos = carve<float>(ptr, (size_t)W * 3);
        p.guide_nrm = carve<float>(ptr, (size_t)W * 3);
        p.guide_list = carve<uint32_t>(ptr, W);
        p.prev_pdf = carve<float>(ptr, W);
        p.rec = carve<float>(ptr, (size_t)W * kGuideRecords * kRecFloats);
        p.rec_n = carve<uint32_t>(ptr, W);
        p.guide_counts = carve<uint32_t>(ptr, 64);
    }
    return p;
}

}  // namespace

WavePlan plan_waves(const std::vector<RenderJob> &jobs, uint32_t wave_paths)
{
    WavePlan plan;
    uint32_t W = std::max<uint32_t>(wave_paths, 1);
    for (const RenderJob &j : jobs) {
        if (j.spp) W = std::max(W, j.npix);
        plan.max_depth = std::max(plan.max_depth, j.spp ? j.max_depth : 0u);
    }
    uint32_t used = 0, pix = 0;
    plan.wave_first.push_back(0);
    auto close_wave = [&] {
        if (used == 0) return;
        plan.wave_first.push_back((uint32_t)plan.segs.size());
        plan.wave_slots.push_back(used);
        plan.wave_pix.push_back(pix);
        plan.max_slots = std::max(plan.max_slots, used);
        used = 0;
        pix = 0;
    };
    for (uint32_t j = 0; j < jobs.size(); ++j) {
        const RenderJob &J = jobs[j];
        uint32_t s = 0;
        while (s < J.spp) {
            uint32_t fit = (W - used) / J.npix;
            if (fit == 0) {
                close_wave();
                fit = W / J.npix;
            }
            const uint32_t k = std::min(fit, J.spp - s);
            plan.segs.push_back(WaveSegment{j, used, pix, J.npix, s, k});
            used += k * J.npix;
            pix += J.npix;
            s += k;
        }
    }
    close_wave();
    return plan;
}

WaveRunner::~WaveRunner()
{
    for (int k = 0; k < kMaxWaveStreams; ++k) {
        cudaFree(d_wave[k]);
        if (stream[k]) cudaStreamDestroy(stream[k]);
        if (acc_done[k]) cudaEventDestroy(acc_done[k]);
    }
    if (fork) cudaEventDestroy(fork);
    cudaFree(d_jobs);
    cudaFree(d_segs);
    cudaFree(d_train);
    cudaFree(d_totals);
}

dr_status WaveRunner::prepare(const std::vector<RenderJob> &jobs, const WavePlan &plan, const WaveConfig &cfg,
                              cudaStream_t st, const GuideRun *gr)
{
    const uint32_t nwaves = (uint32_t)plan.wave_slots.size();
    const int K = (int)std::max<uint32_t>(1, std::min<uint32_t>({cfg.streams, (uint32_t)kMaxWaveStreams, nwaves}));
    const size_t need = wave_buffer_bytes(plan.max_slots, gr != nullptr);
    // occupancy of the persistent kernels, queried here so enqueue (which may
    // be under stream capture) only reads the cache
    for (int mode = 0; mode < 2; ++mode) {
        const P8Kernels k = select_p8(mode, cfg.stack);
        resident_blocks((const void *)k.closest, kTraceBlock);
        resident_blocks((const void *)k.shadow, kTraceBlock);
    }
    const uint32_t train_need = gr ? std::max<uint32_t>(1, gr->batch) * std::max<uint32_t>(1, gr->steps) : 0;
    bool grow = jobs.size() > jobs_capacity || plan.segs.size() > segs_capacity || train_need > train_cap;
    for (int k = 0; k < K; ++k) grow = grow || wave_bytes[k] < need;
    if (grow) {
        // buffers may still be in use by earlier work on any stream
        DR_CUDA(cudaDeviceSynchronize());
        for (int k = 0; k < K; ++k)
            if (wave_bytes[k] < need) {
                cudaFree(d_wave[k]);
                d_wave[k] = nullptr;
                wave_bytes[k] = 0;
                DR_CUDA(dev_malloc(&d_wave[k], need));
                wave_bytes[k] = need;
            }
        if (jobs.size() > jobs_capacity) {
            cudaFree(d_jobs);
            d_jobs = nullptr;
            jobs_capacity = 0;
            DR_CUDA(dev_malloc(&d_jobs, jobs.size() * sizeof(RenderJob)));
            jobs_capacity = jobs.size();
        }
        if (plan.segs.size() > segs_capacity) {
            cudaFree(d_segs);
            d_segs = nullptr;
            segs_capacity = 0;
            DR_CUDA(dev_malloc(&d_segs, plan.segs.size() * sizeof(WaveSegment)));
            segs_capacity = plan.segs.size();
        }
        if (train_need > train_cap) {
            cudaFree(d_train);
            d_train = nullptr;
            train_cap = 0;
            const size_t bytes = (size_t)train_need * 10 * sizeof(float) + 4 * 256;
            DR_CUDA(dev_malloc(&d_train, bytes));
            DR_CUDA(cudaMemset(d_train, 0, bytes));
            train_cap = train_need;
        }
    }
    for (int k = 0; k < K; ++k) {
        if (!stream[k]) DR_CUDA(cudaStreamCreateWithFlags(&stream[k], cudaStreamNonBlocking));
        if (!acc_done[k]) DR_CUDA(cudaEventCreateWithFlags(&acc_done[k], cudaEventDisableTiming));
    }
    if (!fork) DR_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (!d_totals) DR_CUDA(dev_malloc(&d_totals, 2 * sizeof(unsigned long long)));
    // the tables may still be read by the waves of an earlier call
    for (int k = 0; k < kMaxWaveStreams; ++k)
        if (acc_done[k]) DR_CUDA(cudaStreamWaitEvent(st, acc_done[k], 0));
    // pageable copies are staged before the call returns
    DR_CUDA(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(RenderJob), cudaMemcpyHostToDevice, st));
    DR_CUDA(cudaMemcpyAsync(d_segs, plan.segs.data(), plan.segs.size() * sizeof(WaveSegment), cudaMemcpyHostToDevice,
                            st));
    return DR_OK;
}

dr_status WaveRunner::enqueue(const SceneArrays &sc, const WavePlan &plan, const WaveConfig &cfg, int tri_mode,
                              cudaStream_t st, const GuideRun *gr)
{
    const uint32_t nwaves = (uint32_t)plan.wave_slots.size();
    if (nwaves == 0) return DR_OK;
    // the waves' training steps run in wave order: they follow the ordered
    // accumulation pass, which waits for the previous wave's
    const int K = (int)std::max<uint32_t>(1, std::min<uint32_t>({cfg.streams, (uint32_t)kMaxWaveStreams, nwaves}));
    // training ring (SoA): positions, normals, directions, weights, head counter
    float *t_pos = nullptr, *t_nrm = nullptr, *t_dir = nullptr, *t_w = nullptr;
    uint32_t *t_head = nullptr;
    if (gr) {
        char *ptr = static_cast<char *>(d_train);
        t_pos = carve<float>(ptr, (size_t)train_cap * 3);
        t_nrm = carve<float>(ptr, (size_t)train_cap * 3);
        t_dir = carve<float>(ptr, (size_t)train_cap * 3);
        t_w = carve<float>(ptr, train_cap);
        t_head = carve<uint32_t>(ptr, 2);
    }
    const int sms = ctx->num_sms;
    const bool wt = tri_mode == DR_TRI_WATERTIGHT, wide = sc.trace.layout == 8;
    const P8Kernels p8 = select_p8(tri_mode, cfg.stack);
    const int closest_per_sm = resident_blocks((const void *)p8.closest, kTraceBlock);
    const int shadow_per_sm = resident_blocks((const void *)p8.shadow, kTraceBlock);
    DR_CUDA(cudaMemsetAsync(d_totals, 0, 2 * sizeof(unsigned long long), st));
    DR_CUDA(cudaEventRecord(fork, st));
    for (int k = 0; k < K; ++k) DR_CUDA(cudaStreamWaitEvent(stream[k], fork, 0));
    for (uint32_t w = 0; w < nwaves; ++w) {
        const int k = (int)(w % (uint32_t)K);
        cudaStream_t ws = stream[k];
        RenderParams q = wave_params(sc, d_jobs, d_wave[k], plan.max_slots, cfg.chunk, gr != nullptr);
        if (gr) {
            q.guide_alpha = gr->alpha;
            q.guide_target = (int)gr->target;
            q.guide_bounces = (int)gr->bounces;
            q.train_pos = t_pos, q.train_nrm = t_nrm, q.train_dir = t_dir, q.train_w = t_w;
            q.train_head = t_head;
            q.train_cap = train_cap;
        }
        // training records only while the network still trains (a wave
        // enqueued after the step budget is spent writes none)
        const bool learn = gr && gr->train && (gr->budget == 0 || guide_steps(gr->guide) < gr->budget);
        if (gr && !learn) q.rec = nullptr, q.rec_n = nullptr;
        if (gr && gr->alpha_ramp > 0) {
            // the mixture's share rises with the steps the network has taken
            const float f = std::min(1.0f, (float)guide_steps(gr->guide) / (float)gr->alpha_ramp);
            q.guide_alpha = gr->alpha * f;
        }
        q.ray_totals = d_totals;
        q.segs = d_segs + plan.wave_first[w];
        q.nsegs = plan.wave_first[w + 1] - plan.wave_first[w];
        q.wave = plan.wave_slots[w];
        q.wave_pix = plan.wave_pix[w];
        const uint32_t W = q.wave;
        const unsigned trace_grid = (unsigned)std::min<uint64_t>((W + kTraceBlock - 1) / kTraceBlock, (uint64_t)sms * 16);
        const unsigned shade_grid = (unsigned)std::min<uint64_t>((W + kRenderBlock - 1) / kRenderBlock, (uint64_t)sms * 16);
        const uint64_t trace_blocks = (W + kTraceBlock - 1) / kTraceBlock;
        const unsigned pgrid = (unsigned)std::min<uint64_t>(trace_blocks, (uint64_t)sms * closest_per_sm);
        const unsigned sgrid = (unsigned)std::min<uint64_t>(trace_blocks, (uint64_t)sms * shadow_per_sm);
        DR_CUDA(cudaMemsetAsync(q.counts, 0, 128 * sizeof(uint32_t), ws));
        DR_CUDA(cudaMemsetAsync(q.work, 0, 128 * sizeof(unsigned long long), ws));
        if (gr) DR_CUDA(cudaMemsetAsync(q.guide_counts, 0, 64 * sizeof(uint32_t), ws));
        k_camera<<<(W + kRenderBlock - 1) / kRenderBlock, kRenderBlock, 0, ws>>>(q);
        for (int b = 0; b < (int)plan.max_depth; ++b) {
            if (wide) {
                p8.closest<<<pgrid, kTraceBlock, 0, ws>>>(q, b);
            } else {
                if (wt) k_wave_closest<1, 2><<<trace_grid, kTraceBlock, 0, ws>>>(q, b);
                else k_wave_closest<0, 2><<<trace_grid, kTraceBlock, 0, ws>>>(q, b);
            }
            // the guided shading kernel serves the guided bounces and the one
            // after them (its emission weights use the mixture density of the
            // last guided direction, and it closes that vertex's training
            // record); later bounces sample the cosine lobe only, as the plain
            // kernel does
            if (gr && b <= (int)gr->bounces) {
                if (b < (int)gr->bounces) {
                    k_guide_prepare<<<shade_grid, kRenderBlock, 0, ws>>>(q, b);
                    DR_CUDA(launch_guide_infer(gr->guide, q.guide_pos, q.guide_nrm, q.guide_list, q.guide_counts + b,
                                               W, q.guide_y, ws, DR_GUIDE_DECODED != 0));
                }
                k_shade<true><<<shade_grid, kRenderBlock, 0, ws>>>(q, b);
            } else {
                k_shade<false><<<shade_grid, kRenderBlock, 0, ws>>>(q, b);
            }
            if (wide) {
                p8.shadow<<<sgrid, kTraceBlock, 0, ws>>>(q, b);
            } else {
                if (wt) k_wave_shadow<1, 2><<<trace_grid, kTraceBlock, 0, ws>>>(q, b);
                else k_wave_shadow<0, 2><<<trace_grid, kTraceBlock, 0, ws>>>(q, b);
            }
        }
        // images receive the waves in order
        if (w > 0) DR_CUDA(cudaStreamWaitEvent(ws, acc_done[(w - 1) % (uint32_t)K], 0));
        if (learn) {
            DR_CUDA(cudaMemsetAsync(q.train_head + 1, 0, sizeof(uint32_t), ws));
            k_guide_collect<<<(W + 255) / 256, 256, 0, ws>>>(q);
        }
        k_accumulate_wave<<<(q.wave_pix + 255) / 256, 256, 0, ws>>>(q);
        DR_CUDA(cudaGetLastError());
        if (learn)
            for (uint32_t t = 0; t < gr->steps && (gr->budget == 0 || guide_steps(gr->guide) < gr->budget); ++t) {
                const size_t o = (size_t)t * gr->batch;
                const dr_status ts = guide_train_step(gr->guide, t_pos + 3 * o, t_nrm + 3 * o, t_dir + 3 * o, t_w + o,
                                                      gr->batch, ws);
                if (ts != DR_OK) return ts;
            }
        DR_CUDA(cudaEventRecord(acc_done[k], ws));
    }
    for (int k = 0; k < K; ++k) DR_CUDA(cudaStreamWaitEvent(st, acc_done[k], 0));
    return DR_OK;
}

SceneArrays scene_arrays(const dr_scene *s)
{
    SceneArrays a{};
    a.trace.nodes = s->d_nodes;
    a.trace.nodes8 = s->d_nodes8;
    a.trace.layout = (int)s->layout;
    a.trace.tri_ref = s->d_tri_ref;
    a.trace.tri_wt = s->d_tri_wt;
    a.trace.prim = s->d_prim;
    a.trace.num_nodes = s->num_nodes;
    a.trace.error = s->ctx->d_error;
    a.trace.stack_limit = s->ctx->stack_limit;
    a.shade = s->d_shade;
    a.objects = s->d_objects;
    a.materials = s->d_materials;
    a.light_table = s->d_light_table;
    a.tri_tables = s->d_tri_tables;
    return a;
}

RenderJob make_job(const dr_scene *s, const dr_camera *cam, const dr_render_config *cfg, float *accum,
                   uint32_t *casts)
{
    RenderJob J{};
    J.accum = reinterpret_cast<float4 *>(accum);
    J.pix_casts = casts;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) J.m[r * 4 + c] = cam->transform[r * 4 + c];
    J.focal = cam->focal_length;
    J.cx = cam->center[0];
    J.cy = cam->center[1];
    J.psx = cam->pixel_size[0];
    J.psy = cam->pixel_size[1];
    J.width = cam->width;
    J.height = cam->height;
    J.pixel_sampling = cfg->pixel_sampling;
    J.npix = (uint32_t)((uint64_t)cam->width * (uint64_t)cam->height);
    J.root = scene_root(s->num_nodes);
    J.obj_base = 0;
    J.num_objects = s->num_objects;
    J.total_power = s->total_radiant_power;
    J.lights = s->lights ? 1 : 0;
    J.seed_lo = (uint32_t)cfg->seed;
    J.seed_hi = (uint32_t)(cfg->seed >> 32);
    J.sample_offset = cfg->sample_offset;
    J.max_depth = cfg->max_depth;
    J.spp = cfg->spp;
    return J;
}

}  // namespace dr

using namespace dr;

extern "C" dr_status dr_render(dr_scene *s, const dr_camera *cam, const dr_render_config *cfg, float *accum_dev,
                               uint32_t *casts_dev, void *stream)
{
    DR_CHECK_ARG(s && cam && cfg && accum_dev, "dr_render: NULL argument");
    DR_CHECK_ARG(cam->width > 0 && cam->height > 0, "dr_render: empty image");
    DR_CHECK_ARG(cfg->max_depth >= 1 && cfg->max_depth <= (uint32_t)kMaxRenderDepth,
                 "dr_render: max_depth must be in [1, 63]");
    DR_CHECK_ARG(cfg->tri_mode == DR_TRI_REFERENCE || cfg->tri_mode == DR_TRI_WATERTIGHT, "dr_render: bad tri_mode");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(accum_dev) & 15) == 0, "dr_render: accum must be 16-byte aligned");
    DR_CHECK_ARG(cfg->debug >= DR_DEBUG_OFF && cfg->debug <= DR_DEBUG_WINDING_ORDER, "dr_render: bad debug view");
    if (cfg->spp == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(s->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    const uint64_t npix64 = (uint64_t)cam->width * (uint64_t)cam->height;
    DR_CHECK_ARG(npix64 < (1ull << 31) / 16, "dr_render: image too large");
    const RenderJob job = make_job(s, cam, cfg, accum_dev, casts_dev);
    const SceneArrays sc = scene_arrays(s);
    if (cfg->debug != DR_DEBUG_OFF) {
        const unsigned grid = (job.npix + kRenderBlock - 1) / kRenderBlock;
        const bool wt = cfg->tri_mode == DR_TRI_WATERTIGHT;
        if (s->layout == 8) {
            if (wt) k_debug<1, 8><<<grid, kRenderBlock, 0, st>>>(sc, job, cfg->debug);
            else k_debug<0, 8><<<grid, kRenderBlock, 0, st>>>(sc, job, cfg->debug);
        } else {
            if (wt) k_debug<1, 2><<<grid, kRenderBlock, 0, st>>>(sc, job, cfg->debug);
            else k_debug<0, 2><<<grid, kRenderBlock, 0, st>>>(sc, job, cfg->debug);
        }
        DR_CUDA(cudaGetLastError());
        return DR_OK;
    }
    WaveConfig wc;
    if (cfg->wave_paths) wc.wave_paths = cfg->wave_paths;
    if (cfg->streams) wc.streams = cfg->streams;
    wc.chunk = cfg->chunk;
    DR_CHECK_ARGF(cfg->stack == 0 || cfg->stack == 4 || cfg->stack == 8 || cfg->stack == 16,
                  "render: stack must be 0, 4, 8 or 16 (got %u)", cfg->stack);
    if (cfg->stack) wc.stack = cfg->stack;
    const std::vector<RenderJob> jobs{job};
    const WavePlan plan = plan_waves(jobs, wc.wave_paths);
    if (!s->runner) {
        s->runner = new (std::nothrow) WaveRunner;
        if (!s->runner) return fail(DR_ERR_OUT_OF_MEMORY, "dr_render: host allocation failed");
        s->runner->ctx = s->ctx;
    }
    dr_status r = s->runner->prepare(jobs, plan, wc, st);
    if (r != DR_OK) return r;
    return s->runner->enqueue(sc, plan, wc, cfg->tri_mode, st);
}

extern "C" dr_status dr_render_guided(dr_scene *s, const dr_camera *cam, const dr_render_config *cfg, dr_guide *guide,
                                      const dr_guided_config *gcfg, float *accum_dev, uint32_t *casts_dev, void *stream)
{
    DR_CHECK_ARG(s && cam && cfg && guide && accum_dev, "dr_render_guided: NULL argument");
    DR_CHECK_ARG(cam->width > 0 && cam->height > 0, "dr_render_guided: empty image");
    DR_CHECK_ARG(cfg->max_depth >= 1 && cfg->max_depth <= (uint32_t)kMaxRenderDepth,
                 "dr_render_guided: max_depth must be in [1, 63]");
    DR_CHECK_ARG(cfg->tri_mode == DR_TRI_REFERENCE || cfg->tri_mode == DR_TRI_WATERTIGHT, "dr_render_guided: bad tri_mode");
    DR_CHECK_ARG(cfg->debug == DR_DEBUG_OFF, "dr_render_guided: debug views are not guided");
    DR_CHECK_ARG((reinterpret_cast<uintptr_t>(accum_dev) & 15) == 0, "dr_render_guided: accum must be 16-byte aligned");
    GuideRun gr;
    gr.guide = guide;
    if (gcfg) {
        DR_CHECK_ARG(gcfg->alpha >= 0.0f && gcfg->alpha < 1.0f, "dr_render_guided: alpha must be in [0, 1)");
        gr.alpha = gcfg->alpha;
        gr.train = gcfg->train != 0;
        if (gcfg->train_batch) gr.batch = gcfg->train_batch;
        if (gcfg->train_steps) gr.steps = gcfg->train_steps;
        gr.budget = gcfg->train_budget;
        DR_CHECK_ARG(gcfg->target <= 1, "dr_render_guided: target must be 0 or 1");
        gr.target = gcfg->target;
        gr.bounces = gcfg->bounces ? gcfg->bounces : 64;
        gr.alpha_ramp = gcfg->alpha_ramp;
    }
    if (cfg->spp == 0) return DR_OK;
    DR_CUDA(cudaSetDevice(s->ctx->device));
    auto st = static_cast<cudaStream_t>(stream);
    const uint64_t npix64 = (uint64_t)cam->width * (uint64_t)cam->height;
    DR_CHECK_ARG(npix64 < (1ull << 31) / 16, "dr_render_guided: image too large");
    WaveConfig wc;
    if (cfg->wave_paths) wc.wave_paths = cfg->wave_paths;
    if (cfg->streams) wc.streams = cfg->streams;
    wc.chunk = cfg->chunk;
    DR_CHECK_ARGF(cfg->stack == 0 || cfg->stack == 4 || cfg->stack == 8 || cfg->stack == 16,
                  "render: stack must be 0, 4, 8 or 16 (got %u)", cfg->stack);
    if (cfg->stack) wc.stack = cfg->stack;
    const std::vector<RenderJob> jobs{make_job(s, cam, cfg, accum_dev, casts_dev)};
    const WavePlan plan = plan_waves(jobs, wc.wave_paths);
    if (!s->runner) {
        s->runner = new (std::nothrow) WaveRunner;
        if (!s->runner) return fail(DR_ERR_OUT_OF_MEMORY, "dr_render_guided: host allocation failed");
        s->runner->ctx = s->ctx;
    }
    dr_status r = s->runner->prepare(jobs, plan, wc, st, &gr);
    if (r != DR_OK) return r;
    return s->runner->enqueue(scene_arrays(s), plan, wc, cfg->tri_mode, st, &gr);
}
