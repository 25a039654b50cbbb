// scene_render.cu -- per-scene data of the renderer: shading records, objects,
// materials and the two-level light tables.
//
// Light selection follows the reference: an object is picked by emitted power
// (Renderer::calculateLightWeights, src/Renderer.cpp:113-152: surface area x
// luminance(pi x emission), normalised by the total), then a triangle of that
// object by area (src/GpuTris.cpp:7-21). Both tables are built on the device:
// by default with the parallel sweep build (the object table of 66,356 objects
// in a few parallel launches), or, with DR_LIGHT_TABLES_REFERENCE, in
// reference mode, so that they equal generateAliasTable's bit for bit.

#include "dr_internal.h"
#include "alias_kernels.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace dr {
namespace {

constexpr float kPi = 3.14159274f;  // std::numbers::pi_v<float>

// triangleArea (include/Utils.hpp:218-224) in FP32.
float triangle_area(const float *q)
{
    const float ux = q[0] - q[3], uy = q[1] - q[4], uz = q[2] - q[5];
    const float vx = q[0] - q[6], vy = q[1] - q[7], vz = q[2] - q[8];
    const float cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    return std::sqrt(cx * cx + cy * cy + cz * cz) / 2;
}

template <typename T>
cudaError_t upload_vec(T **dst, const std::vector<T> &v, uint64_t &bytes)
{
    *dst = nullptr;
    if (v.empty()) return cudaSuccess;
    cudaError_t e = dev_malloc(reinterpret_cast<void **>(dst), sizeof(T) * v.size());
    if (e != cudaSuccess) return e;
    bytes += sizeof(T) * v.size();
    return cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

// A temporary device buffer freed when it leaves scope (also on error returns).
template <typename T>
struct DevTemp {
    T *p = nullptr;
    ~DevTemp() { cudaFree(p); }
};

}  // namespace

dr_status build_render_data(dr_scene *s, const dr_scene_desc *d)
{
    const uint32_t n = d->num_triangles;
    std::vector<dr_object> objects;
    if (d->objects_host && d->num_objects) objects.assign(d->objects_host, d->objects_host + d->num_objects);
    else objects.push_back(dr_object{0, n, 0, 0.0f});
    std::vector<dr_material> materials;
    if (d->materials_host && d->num_materials) materials.assign(d->materials_host, d->materials_host + d->num_materials);
    else {
        dr_material m{};
        m.kind = DR_MAT_DIFFUSE;
        m.ior = 1.0f;
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.5f;
        materials.push_back(m);
    }
    s->num_objects = (uint32_t)objects.size();
    s->num_materials = (uint32_t)materials.size();

    // per-triangle object and material
    std::vector<int32_t> tri_obj(n, 0), tri_mat(n, 0);
    for (uint32_t o = 0; o < objects.size(); ++o)
        for (uint32_t k = 0; k < objects[o].tri_count; ++k) {
            tri_obj[objects[o].tri_begin + k] = (int32_t)o;
            tri_mat[objects[o].tri_begin + k] = objects[o].material;
        }
    if (d->tri_material_host)
        for (uint32_t i = 0; i < n; ++i) {
            const int32_t m = d->tri_material_host[i];
            if (m < 0 || (uint32_t)m >= materials.size())
                return fail(DR_ERR_INVALID_ARGUMENT, "dr_scene_create: triangle %u material out of range", i);
            tri_mat[i] = m;
        }
    std::vector<float4> shade((size_t)n * 3);
    host_parallel_chunks(n, size_t(1) << 16, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            const float *q = d->positions_host + i * 9;
            shade[i * 3 + 0] = make_float4(q[0], q[1], q[2], q[3]);
            shade[i * 3 + 1] = make_float4(q[4], q[5], q[6], q[7]);
            float fo, fm;  // object and material ids travel as int32 bit patterns
            std::memcpy(&fo, &tri_obj[i], 4);
            std::memcpy(&fm, &tri_mat[i], 4);
            shade[i * 3 + 2] = make_float4(q[8], fo, fm, 0.0f);
        }
    });

    // level 1: objects by emitted power
    const size_t N = objects.size();
    std::vector<float> weights(N, 0.0f);
    float total = 0.0f;
    for (size_t i = 0; i < N; ++i) {
        const dr_material &m = materials[objects[i].material];
        float Mx = 0.f, My = 0.f, Mz = 0.f;
        if (m.kind == DR_MAT_DIFFUSE) {
            Mx = m.emission[0] * kPi;
            My = m.emission[1] * kPi;
            Mz = m.emission[2] * kPi;
        }
        const float lum = 0.2126f * Mx + 0.7152f * My + 0.0722f * Mz;
        // an object without triangles cannot be sampled
        weights[i] = objects[i].tri_count ? objects[i].surface_area * lum : 0.0f;
        total += weights[i];
    }
    std::vector<uint8_t> emits(N, 0);
    for (size_t i = 0; i < N; ++i) {
        emits[i] = weights[i] > 0.0f;
        weights[i] /= total;
    }
    s->total_radiant_power = total;
    s->lights = total > 0.0f && std::isfinite(total);

    // level 2: triangles of each emitting object by area (or the caller's weights)
    std::vector<float> tri_w(n, 0.0f);
    std::vector<uint32_t> seg_begin, seg_count;
    for (size_t o = 0; o < N; ++o) {
        if (!emits[o] || objects[o].tri_count == 0) continue;
        for (uint32_t k = 0; k < objects[o].tri_count; ++k) {
            const uint32_t t = objects[o].tri_begin + k;
            tri_w[t] = d->tri_weight_host ? d->tri_weight_host[t] : triangle_area(d->positions_host + (size_t)t * 9);
        }
        seg_begin.push_back(objects[o].tri_begin);
        seg_count.push_back(objects[o].tri_count);
    }

    cudaError_t e;
    if ((e = upload_vec(&s->d_objects, objects, s->device_bytes)) != cudaSuccess ||
        (e = upload_vec(&s->d_shade, shade, s->device_bytes)) != cudaSuccess)
        return cuda_fail(e, "dr_scene_create: upload shading data");
    if (!s->d_materials) {
        if ((e = upload_vec(&s->d_materials, materials, s->device_bytes)) != cudaSuccess)
            return cuda_fail(e, "dr_scene_create: upload materials");
    }
    if (!s->lights) return DR_OK;

    // device builds
    const bool ref_mode = d->light_tables == DR_LIGHT_TABLES_REFERENCE;
    DevTemp<float> d_w, d_tw;
    DevTemp<uint32_t> d_seg;
    DR_CUDA(dev_malloc(&s->d_light_table, N * sizeof(dr_alias_entry)));
    s->device_bytes += N * sizeof(dr_alias_entry);
    DR_CUDA(dev_malloc(&s->d_tri_tables, (size_t)std::max(1u, n) * sizeof(dr_alias_entry)));
    s->device_bytes += (size_t)std::max(1u, n) * sizeof(dr_alias_entry);
    DR_CUDA(cudaMemset(s->d_tri_tables, 0, (size_t)std::max(1u, n) * sizeof(dr_alias_entry)));
    DR_CUDA(dev_malloc(&d_w.p, N * sizeof(float)));
    DR_CUDA(cudaMemcpy(d_w.p, weights.data(), N * sizeof(float), cudaMemcpyHostToDevice));
    // scratch: the object table's build, the reference triangle tables' heaps,
    // and the parallel sweep of the largest triangle table
    size_t need = alias_scratch_bytes((uint32_t)N, ref_mode ? DR_ALIAS_REFERENCE : DR_ALIAS_SWEEP);
    if (ref_mode) need = std::max(need, (size_t)n * (2 * 8 + 4) + 1024);
    std::vector<uint32_t> big;  // sweep mode: segments built by the parallel kernels
    for (size_t k = 0; k < seg_begin.size(); ++k)
        if (!ref_mode && seg_count[k] > kSweepThreadMax) {
            big.push_back((uint32_t)k);
            need = std::max(need, alias_scratch_bytes(seg_count[k], DR_ALIAS_SWEEP));
        }
    const dr_status st = ensure_scratch(s->ctx, need);
    if (st != DR_OK) return st;
    DR_CUDA(launch_alias_build(d_w.p, (uint32_t)N, s->d_light_table, ref_mode ? DR_ALIAS_REFERENCE : DR_ALIAS_SWEEP,
                               s->ctx->scratch, s->ctx->scratch_bytes, s->ctx->num_sms, nullptr));
    DR_CUDA(cudaDeviceSynchronize());
    if (!seg_begin.empty()) {
        DR_CUDA(dev_malloc(&d_tw.p, (size_t)n * sizeof(float)));
        DR_CUDA(cudaMemcpy(d_tw.p, tri_w.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
        // sweep mode: the one-thread kernel skips the large segments (count 0)
        std::vector<uint32_t> small_count = seg_count;
        for (uint32_t k : big) small_count[k] = 0;
        const size_t ns = seg_begin.size();
        DR_CUDA(dev_malloc(&d_seg.p, ns * 2 * sizeof(uint32_t)));
        DR_CUDA(cudaMemcpy(d_seg.p, seg_begin.data(), ns * sizeof(uint32_t), cudaMemcpyHostToDevice));
        DR_CUDA(cudaMemcpy(d_seg.p + ns, small_count.data(), ns * sizeof(uint32_t), cudaMemcpyHostToDevice));
        if (ref_mode)
            DR_CUDA(launch_alias_ref_segments(d_tw.p, n, d_seg.p, d_seg.p + ns, (uint32_t)ns, s->d_tri_tables,
                                              s->ctx->scratch, s->ctx->scratch_bytes, nullptr));
        else
            DR_CUDA(launch_alias_sweep_segments(d_tw.p, d_seg.p, d_seg.p + ns, (uint32_t)ns, s->d_tri_tables, nullptr));
        for (uint32_t k : big)
            DR_CUDA(launch_alias_build(d_tw.p + seg_begin[k], seg_count[k], s->d_tri_tables + seg_begin[k],
                                       DR_ALIAS_SWEEP, s->ctx->scratch, s->ctx->scratch_bytes, s->ctx->num_sms,
                                       nullptr));
        DR_CUDA(cudaDeviceSynchronize());
    }
    return DR_OK;
}

}  // namespace dr
