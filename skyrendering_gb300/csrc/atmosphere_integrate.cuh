// atmosphere_integrate.cuh — the atmosphere integrator shared by the LUT
// passes (atmosphere.cu) and the full-screen composite (composite.cu):
// ComputeScatteredLuminance in cancellation-free FP32 form, the medium, the
// multi-scattering lookup and the space-camera ray start.
#pragma once

#include "atmosphere_kernels.cuh"
#include "lut_access.cuh"

namespace skyr {

struct LutView {
    const float4* t;
    int tw, th;
};

// GetMultiscatteringContribution (Atmosphere.glsl:169-178)
template <class S>
__device__ __forceinline__ float3 ms_contribution(const AtmoConsts& A, const S* ms, int mw, int mh, float h,
                                                  float mu_s) {
    float x_mu_s = mu_s * 0.5f + 0.5f;
    float x_r = h * A.inv_thickness;
    return bilinear_clamp(ms, mw, mh, x_mu_s * (float)(mw - 1), x_r * (float)(mh - 1));
}

// GetExtinction / GetScattering (Atmosphere.glsl:119-132,156-159)
__device__ __forceinline__ void medium(const AtmoConsts& A, float h, float3& ray_s, float3& mie_s, float3& ext) {
    float er = clamp01(__expf(-h * A.inv_rayleigh_h));
    float em = clamp01(__expf(-h * A.inv_mie_h));
    float dz = h - A.ozone_center;
    float oz = fmaxf(0.f, h < A.ozone_center ? 1.f + dz * A.inv_ozone_width : 1.f - dz * A.inv_ozone_width);
    ray_s = A.rayleigh_scattering * er;
    mie_s = A.mie_scattering * em;
    ext = ray_s + A.mie_extinction * em + A.ozone_absorption * oz;
}

// Number of samples of `for (float i = start; i < steps; ++i)`.
__device__ __forceinline__ int sample_count(float start, float steps) {
    float c = ceilf(steps - start);
    return c > 0.f ? (int)c : 0;
}

// State at the start of a ray segment.
struct RayStart {
    float r, h, rho2;  // radius, altitude, r^2 - R^2
    float mu;          // cos(view, up)
    float mu_s;        // cos(sun, up)
    float nu;          // cos(view, sun)
};

// Compose (L, T) pairs of LANES consecutive lanes, earliest chunk first; the
// group leader ends with the whole-ray result.
template <int LANES>
__device__ __forceinline__ void compose_lanes(float3& L, float3& T, float3* Lf) {
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1) {
        float3 Lp, Tp, Fp;
        Lp.x = __shfl_down_sync(0xffffffffu, L.x, o);
        Lp.y = __shfl_down_sync(0xffffffffu, L.y, o);
        Lp.z = __shfl_down_sync(0xffffffffu, L.z, o);
        Tp.x = __shfl_down_sync(0xffffffffu, T.x, o);
        Tp.y = __shfl_down_sync(0xffffffffu, T.y, o);
        Tp.z = __shfl_down_sync(0xffffffffu, T.z, o);
        if (Lf) {
            Fp.x = __shfl_down_sync(0xffffffffu, Lf->x, o);
            Fp.y = __shfl_down_sync(0xffffffffu, Lf->y, o);
            Fp.z = __shfl_down_sync(0xffffffffu, Lf->z, o);
        }
        L = L + T * Lp;
        if (Lf) *Lf = *Lf + T * Fp;
        T = T * Tp;
    }
}

// ComputeScatteredLuminance (Atmosphere.glsl:220-295) over samples
// [k0, k1) of a ray with `n` samples starting at index `start_i`.
// MS = the MULTISCATTERING_COMPUTE_PROGRAM variant.
template <bool MS, class S>
__device__ __forceinline__ void integrate(const AtmoConsts& A, const LutView& L, const S* ms, int mw, int mh,
                                          const RayStart& s0, float dx, float start_i, int k0, int k1, float ph_r,
                                          float ph_m, float3& lum, float3& trans, float3& lf) {
    lum = f3(0.f);
    trans = f3(1.f);
    lf = f3(0.f);
    float b = 2.f * s0.r * s0.mu;
    float rms = s0.r * s0.mu_s;
    for (int k = k0; k < k1; ++k) {
        float d = ((float)k + start_i) * dx;
        float s = fmaf(d, b + d, s0.rho2);  // r_i^2 - R^2
        float r2 = A.R2 + s;
        float inv_r = rsqrtf(r2);
        float r_i = r2 * inv_r;
        float h_i = __fdividef(s, r_i + A.R);
        float mu_s_i = fmaf(d, s0.nu, rms) * inv_r;
        float3 ray_s, mie_s, ext;
        medium(A, h_i, ray_s, mie_s, ext);
        float3 tr_i, phi;
        phi.x = seg_phi(ext.x * dx, tr_i.x);
        phi.y = seg_phi(ext.y * dx, tr_i.y);
        phi.z = seg_phi(ext.z * dx, tr_i.z);
        float3 sv = sun_visibility_lut(A, L.t, L.tw, L.th, r_i, s, h_i, mu_s_i);
        float3 li = (ray_s * ph_r + mie_s * ph_m) * sv;
        float3 sc = ray_s + mie_s;
        if constexpr (!MS) {
            float3 m = ms_contribution(A, ms, mw, mh, h_i, mu_s_i);
            li = (li + m * sc * A.ms_mask) * A.solar_illuminance;
        }
        // (L - L T_i) / ext = L dx phi(ext dx)
        float3 w = trans * phi * dx;
        lum += li * w;
        if constexpr (MS) lf += sc * w;
        trans = trans * tr_i;
    }
}

// ComputeRaymarchingStartPositionAndChangeDistance (AtmosphereRenderer.glsl:56-72)
// + FromSpaceIntersectTopAtmosphereBoundary (AtmosphereInterface.glsl:6-13).
__device__ __forceinline__ RayStart ray_start(const AtmoConsts& A, const ViewConsts& V, float mu, float nu,
                                              float& marching) {
    float mu_s = dot3(V.sun, V.up);
    RayStart s{V.cam_r, V.cam_h, V.cam_rho2, mu, mu_s, nu};
    if (V.in_space != 0.f) {
        float r = V.cam_r, rm = r * mu;
        float c = (V.cam_h - A.thickness) * (r + A.top);  // r^2 - top^2 > 0
        float disc = rm * rm - c;
        if (mu < 0.f && disc >= 0.f) {
            float sq = sqrtf(fmaxf(disc, 0.f));
            float nd = fmaxf(c / (-rm + sq), 0.f);
            marching -= nd;
            // move the start to the top boundary: r = top exactly
            float r_s = A.top;
            s.r = r_s;
            s.h = A.thickness;
            s.rho2 = A.top2_minus_R2;
            s.mu = (rm + nd) / r_s;
            s.mu_s = (r * mu_s + nd * nu) / r_s;
        } else {
            marching = 0.f;
        }
    }
    return s;
}

}  // namespace skyr
