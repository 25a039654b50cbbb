// dr_internal.h -- internal types of the GB300 path-tracing core.
#pragma once

#include <algorithm>
#include <atomic>

#include "devilray_gb300.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <thread>
#include <vector>

namespace dr {

// ---- errors ------------------------------------------------------------------

void set_error(const char *fmt, ...);
dr_status fail(dr_status code, const char *fmt, ...);
dr_status cuda_fail(cudaError_t e, const char *what);

#define DR_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return ::dr::cuda_fail(e_, #call);            \
    } while (0)

#define DR_CHECK_ARG(cond, msg)                                              \
    do {                                                                     \
        if (!(cond)) return ::dr::fail(DR_ERR_INVALID_ARGUMENT, "%s", msg);   \
    } while (0)

// DR_CHECK_ARG with a printf-style message.
#define DR_CHECK_ARGF(cond, ...)                                             \
    do {                                                                     \
        if (!(cond)) return ::dr::fail(DR_ERR_INVALID_ARGUMENT, __VA_ARGS__); \
    } while (0)

// Device allocations of the library go through dev_malloc: cudaMalloc, except
// that dr_debug_fail_allocation can make the n-th next one fail with
// cudaErrorMemoryAllocation, so that tests reach every allocation's error path
// without exhausting a GPU.
cudaError_t dev_malloc_raw(void **p, size_t bytes);
template <typename T>
inline cudaError_t dev_malloc(T **p, size_t bytes)
{
    return dev_malloc_raw(reinterpret_cast<void **>(p), bytes);
}

// Runs f(begin, end) over [0, n) in contiguous chunks of at least `grain`
// items on up to `max_threads` host threads (0: hardware_concurrency; the
// caller's thread takes the first chunk). Each chunk writes only its own
// outputs, so the result does not depend on the split.
template <typename F>
inline void host_parallel_chunks(size_t n, size_t grain, F &&f, size_t max_threads = 0)
{
    const size_t hw = max_threads ? max_threads : std::max(1u, std::thread::hardware_concurrency());
    const size_t parts = std::max<size_t>(1, std::min(hw, n / std::max<size_t>(1, grain)));
    if (parts == 1) {
        f(size_t(0), n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(parts - 1);
    for (size_t k = 1; k < parts; ++k) pool.emplace_back([&, k] { f(n * k / parts, n * (k + 1) / parts); });
    f(size_t(0), n / parts);
    for (auto &t : pool) t.join();
}

// Device error word bits (dr_context::d_error), set by kernels instead of
// trapping; the host maps them to dr_status.
enum : uint32_t {
    ERR_STACK_OVERFLOW = 1u << 0,
    ERR_TIMEOUT = 1u << 1,
    ERR_BAD_INDEX = 1u << 2,
};

// ---- BVH layouts ----------------------------------------------------------------

// Binary node in the layout of Aila and Laine ("Understanding the Efficiency of
// Ray Traversal on GPUs", HPG 2009): both child boxes in one 64-byte record so
// one node fetch tests two boxes.
//   c0xy = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   c1xy = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   cz   = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   link = (c0, c1, -, -): >= 0 inner node index; < 0 leaf = ~((first << 4) | count)
struct alignas(16) Bvh2Node {
    float4 c0xy, c1xy, cz;
    int4 link;
};
static_assert(sizeof(Bvh2Node) == 64, "Bvh2Node must be 64 bytes");

constexpr int kLeafCountBits = 4;
constexpr uint32_t kMaxLeafSize = (1u << kLeafCountBits) - 1;  // 15
constexpr uint32_t kMaxTriangles = 1u << (31 - kLeafCountBits); // 2^27
constexpr int kStackSize = 64;                                  // traversal stack entries
constexpr uint32_t kNoRoot = 0xffffffffu;                       // root of an empty hierarchy
constexpr int kMaxBuildDepth = 60;                              // < kStackSize

inline int32_t leaf_link(uint32_t first, uint32_t count) { return ~int32_t((first << kLeafCountBits) | count); }

struct Bvh2 {
    std::vector<Bvh2Node> nodes;
    std::vector<uint32_t> order;  // leaf-order position -> original triangle index
    int depth = 0;
    float slack = 0.0f;
};

// Compressed 8-wide node after Ylitie, Karras and Laine ("Efficient Incoherent
// Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017), 80 bytes:
//   w[0] = (p.x, p.y, p.z bits, ex | ey << 8 | ez << 16 | imask << 24)
//          p = quantisation origin, e* = biased FP32 exponents of the per-axis
//          scale 2^e, imask bit s = slot s holds an internal child
//   w[1] = (child_base, tri_base, meta[0..3], meta[4..7])
//          internal children are stored from child_base in slot order, the
//          leaf children's triangles from tri_base; meta[s] of a leaf slot =
//          (unary triangle count << 5) | triangle offset (0..23), 0 = empty
//   w[2] = (qlo.x[0..3], qlo.x[4..7], qhi.x[0..3], qhi.x[4..7]) 8-bit child
//          bounds, rounded outward; w[3], w[4]: y and z
// Child slots are ordered by octant: slot s sits towards the corner
// (s&1 ? +x : -x, s&2 ? +y : -y, s&4 ? +z : -z), so a ray whose direction
// signs are o (bit set = negative) visits slots in the order k ^ o.
struct alignas(16) Bvh8Node {
    uint4 w[5];
};
static_assert(sizeof(Bvh8Node) == 80, "Bvh8Node must be 80 bytes");

struct Bvh8 {
    std::vector<Bvh8Node> nodes;
    std::vector<uint32_t> order;  // wide leaf-order position -> original triangle index
    int depth = 0;
    float slack = 0.0f;
};

struct BuildParams {
    uint32_t max_leaf = 4;
    uint32_t bins = 32;
    uint32_t threads = 0;
};

// Binned-SAH build (Wald, "On fast Construction of SAH-based Bounding Volume
// Hierarchies", RT 2007) over a triangle soup. Child boxes are widened by
// `slack` world units (rounded outward) so box culling is conservative with
// respect to the FP32 triangle tests.
Bvh2 build_bvh2(const float *positions, uint32_t num_tris, const BuildParams &p, float slack);

// Binned-SAH binary tree (leaves of at most 3 triangles) collapsed into
// compressed 8-wide nodes.
Bvh8 build_bvh8(const float *positions, uint32_t num_tris, const BuildParams &p, float slack);

// Device linear-BVH build (lbvh.cu): nodes (binary layout 2, or collapsed
// into 8-wide nodes for layout 8), triangle records and index map of `s` from
// host positions (n >= 1); sets num_nodes and depth.
}  // namespace dr
struct dr_scene;
namespace dr {
dr_status build_lbvh_device(dr_scene *s, const float *positions_host, uint32_t n, float slack, uint32_t layout);

// Conservative world-space widening for a scene whose largest absolute
// coordinate is `mag`.
float scene_slack(float mag);

// Triangle records in leaf order.
//   reference-compat (3 x float4): (A.xyz, n.x) (n.y, n.z, BA.x, BA.y) (BA.z, CA.xyz)
//     n = normalize((A-B) x (A-C)) evaluated like the reference, or 0 when
//     |n_f|^2 < 1e-14 (the reference rejects such triangles).
//   watertight (3 x float4): (A.xyz, B.x) (B.yz, C.xy) (C.z, 0, 0, 0)
void make_tri_records(const float *positions, const std::vector<uint32_t> &order,
                      std::vector<float4> &ref_records, std::vector<float4> &wt_records);

}  // namespace dr

// ---- opaque handles ----------------------------------------------------------------

struct dr_context {
    int device = 0;
    int num_sms = 0;
    uint32_t *d_error = nullptr;                // device error word
    unsigned long long *d_counters = nullptr;   // 8 traversal counters per work counter of the ring
    unsigned long long *d_work = nullptr;       // ring of kWorkCounters persistent-kernel work counters
    std::atomic<uint32_t> work_next{0};         // next counter of the ring
    void *scratch = nullptr;                    // grows on demand (alias builds, staging)
    size_t scratch_bytes = 0;
    uint32_t stack_limit = 64;                  // 8-wide traversal stack entries (dr_debug_stack_limit)
};

// Work counters of the public persistent traversal launches: each launch takes
// the next counter of a ring, so launches on different streams that run at
// the same time count separately (up to this many launches in flight).
constexpr uint32_t kWorkCounters = 64;

namespace dr {
// Ensures ctx->scratch holds at least `bytes` (cudaMalloc when it must grow).
dr_status ensure_scratch(dr_context *ctx, size_t bytes);
}  // namespace dr

struct dr_scene;
namespace dr {
// Uploads the shading records, objects, materials and light tables of a scene
// (part of dr_scene_create).
dr_status build_render_data(dr_scene *s, const dr_scene_desc *d);
}  // namespace dr

namespace dr {
struct WaveRunner;
}

struct dr_scene {
    dr_context *ctx = nullptr;
    uint32_t num_tris = 0;
    uint32_t num_nodes = 0;
    uint32_t depth = 0;
    uint32_t layout = 2;
    float slack = 0.0f;
    double build_seconds = 0.0;
    uint64_t device_bytes = 0;

    dr::Bvh2Node *d_nodes = nullptr;     // layout 2
    dr::Bvh8Node *d_nodes8 = nullptr;    // layout 8
    float4 *d_tri_ref = nullptr;
    float4 *d_tri_wt = nullptr;
    int32_t *d_prim = nullptr;      // leaf-order position -> original triangle index

    // scene data for shading (original triangle order)
    uint32_t num_objects = 0, num_materials = 0;
    dr_material *d_materials = nullptr;
    dr_object *d_objects = nullptr;
    float4 *d_shade = nullptr;            // 3 per triangle: (A, B.x) (B.yz, C.xy) (C.z, object, material, -)
    dr_alias_entry *d_light_table = nullptr;  // over objects, by emitted power
    dr_alias_entry *d_tri_tables = nullptr;   // per object, over its triangles (object-local indices)
    float total_radiant_power = 0.0f;
    bool lights = false;                  // some object emits

    // wavefront state of dr_render, created on first use
    dr::WaveRunner *runner = nullptr;

    // staging for the host-buffer entry points
    void *d_stage_rays = nullptr;
    void *d_stage_hits = nullptr;
    uint64_t stage_capacity = 0;
    cudaStream_t stage_streams[4] = {};  // host-buffer tracing: copy in, copy out, more compute streams
};
