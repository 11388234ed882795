// cloud_material.cuh — the material plug-ins' SampleSigmaT and CalHeight01
// on the device, shared by the raymarch and the path tracer.
#pragma once

#include "cloud_internal.cuh"

namespace skyr {

// ---------------------------------------------------------------------------
// Device: material SampleSigmaT
// ---------------------------------------------------------------------------
// CalHeight01 (VolumetricCloudCommon.glsl:36-39) with the altitude formed as
// (x^2 + y^2 + z (z + 2R)) / (|p + R z^| + R) (no cancellation).
__device__ __forceinline__ float height01(const CloudConsts& C, float3 p) {
    float rho2 = fmaf(p.x, p.x, fmaf(p.y, p.y, p.z * (p.z + 2.f * C.R)));
    float r = sqrtf(fmaf(C.R, C.R, rho2));
    float alt = __fdividef(rho2, r + C.R);
    return clamp01((alt - C.bottom) * C.inv_layer);
}

// height01 of a point with rho2 = |p + R z^|^2 - R^2 already known
__device__ __forceinline__ float height01_rho2(const CloudConsts& C, float rho2) {
    float r = sqrtf(fmaf(C.R, C.R, rho2));
    float alt = __fdividef(rho2, r + C.R);
    return clamp01(__fsub_rn(alt, C.bottom) * C.inv_layer);
}

// COUNT: instrumented launches count the evaluations that sample the detail
// texture (past Material1's coverage test) in *n_detail.
template <bool COUNT = false>
__device__ __forceinline__ float sample_sigma_t(const MaterialConsts& M, float3 p, float h01, float dist_to_cam,
                                                unsigned* n_detail = nullptr) {
    switch (M.type) {
        case SKYR_MATERIAL_DEFAULT1: {
            // VolumetricCloudDefaultMaterial1.glsl:14-29
            float u = fmaf(p.x, M.cloud_map.frequency, M.cloud_map.bias_x);
            float v = fmaf(p.y, M.cloud_map.frequency, M.cloud_map.bias_y);
            float lg = __log2f(dist_to_cam);
            float cr = dtex_sample(M.cloud_map_tex, 0, u, v, 0.f, __log2f(M.cloud_map.k_lod) + lg + M.lod_bias,
                                   M.min2d);
            float density = clamp01((cr - M.m1_threshold) * M.m1_edge_hardness);
            density *= clamp01((1.f - h01) * M.m1_height_hardness);
            if (density == 0.f) return 0.f;
            if constexpr (COUNT) ++*n_detail;
            float du = fmaf(p.x, M.detail.frequency, M.detail.bias_x);
            float dv = fmaf(p.y, M.detail.frequency, M.detail.bias_y);
            float dw = p.z * M.detail.frequency;
            float dt = dtex_sample(M.detail_tex, 0, du, dv, dw, __log2f(M.detail.k_lod) + lg + M.lod_bias, M.min3d);
            dt = (dt + M.m1_detail_base) * M.m1_detail_scale;
            dt *= fmaxf(clamp01(h01 - M.m1_height_cut), clamp01(M.m1_edge_cut - cr));
            return clamp01(density - dt) * M.density * h01;
        }
        case SKYR_MATERIAL_MINIMAL: return M.density;
        default: return 0.f;
    }
}

// Material0 (VolumetricCloudDefaultMaterial0.glsl:9-32) and Voxel need the
// camera position for the LOD of a displaced / arbitrary point.  Both are kept
// out of line: they hold many texture filters (Material0: eight) that would
// otherwise be inlined at every density call site of the raymarch, whose hot
// loop the usual Material1 / Minimal configurations run.
static __device__ __noinline__ float sigma_t_material0(const CloudConsts& C, const MaterialConsts& M, float3 p,
                                                      float h01, float dist_to_cam) {
    float lg = __log2f(dist_to_cam);
    float u = fmaf(p.x, M.cloud_map.frequency, M.cloud_map.bias_x);
    float v = fmaf(p.y, M.cloud_map.frequency, M.cloud_map.bias_y);
    float lod = __log2f(M.cloud_map.k_lod) + lg + M.lod_bias;
    float cr = dtex_sample(M.cloud_map_tex, 0, u, v, 0.f, lod, M.min2d);
    float cg = dtex_sample(M.cloud_map_tex, 1, u, v, 0.f, lod, M.min2d);
    float xu = fmaf(p.x, M.displacement.frequency, M.displacement.bias_x);
    float xv = fmaf(p.y, M.displacement.frequency, M.displacement.bias_y);
    float xw = p.z * M.displacement.frequency;
    float xl = __log2f(M.displacement.k_lod) + lg + M.lod_bias;
    float3 disp;
    disp.x = dtex_sample(M.displacement_tex, 0, xu, xv, 0.f, xl, M.mindisp) +
             dtex_sample(M.displacement_tex, 2, xu, xw, 0.f, xl, M.mindisp);
    disp.y = dtex_sample(M.displacement_tex, 1, xu, xv, 0.f, xl, M.mindisp);
    disp.z = dtex_sample(M.displacement_tex, 3, xu, xw, 0.f, xl, M.mindisp);
    float3 q = p + disp * M.m0_disp_scale;
    float3 dq = q - C.cam;
    float dl = __log2f(sqrtf(dot3(dq, dq)));
    float du = fmaf(q.x, M.detail.frequency, M.detail.bias_x);
    float dv = fmaf(q.y, M.detail.frequency, M.detail.bias_y);
    float dw = q.z * M.detail.frequency;
    float dt = dtex_sample(M.detail_tex, 0, du, dv, dw, __log2f(M.detail.k_lod) + dl + M.lod_bias, M.min3d);
    dt = fmaf(dt, M.m0_detail_x, M.m0_detail_y);
    // CalHeightMask (VolumetricCloudDefaultMaterial0.glsl:9-12)
    float hit = clamp01(h01 / cg);
    float mask = clamp01(hit * (hit - 1.f) * -4.f);
    return clamp01((cr * mask - dt) / (1.f - dt)) * h01 * M.density;
}

static __device__ __noinline__ float sigma_t_voxel(const MaterialConsts& M, float3 p, float h01, float dist_to_cam) {
    // VolumetricCloudMaterialVoxel.glsl:12-16
    float u = fmaf(p.x, M.vx_freq_x, M.vx_bias_x);
    float v = fmaf(p.y, M.vx_freq_y, M.vx_bias_y);
    float lod = __log2f(M.vx_k_lod * dist_to_cam) + M.lod_bias;
    return dtex_sample(M.voxel_tex, 0, u, v, h01, lod, SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST) * M.density;
}

template <bool COUNT = false>
__device__ __forceinline__ float sigma_t(const CloudConsts& C, const MaterialConsts& M, float3 p, float h01,
                                         float dist_to_cam, unsigned* n_detail = nullptr) {
    if (M.type == SKYR_MATERIAL_DEFAULT1 || M.type == SKYR_MATERIAL_MINIMAL)
        return sample_sigma_t<COUNT>(M, p, h01, dist_to_cam, n_detail);
    if (M.type == SKYR_MATERIAL_DEFAULT0) {
        if constexpr (COUNT) ++*n_detail;  // Material0 samples the detail texture at every evaluation
        return sigma_t_material0(C, M, p, h01, dist_to_cam);
    }
    if (M.type == SKYR_MATERIAL_VOXEL) return sigma_t_voxel(M, p, h01, dist_to_cam);
    return 0.f;
}

}  // namespace skyr
