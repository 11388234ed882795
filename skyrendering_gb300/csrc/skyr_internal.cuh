// skyr_internal.cuh — device math shared by the kernels and the host-side
// derivation of kernel constants.  Everything here is FP32 unless marked.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/skyr.h"

#define SKYR_PI 3.14159265358979323846f

// ---------------------------------------------------------------------------
// float3 helpers
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float3 f3(float a) { return make_float3(a, a, a); }
__host__ __device__ __forceinline__ float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__host__ __device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__host__ __device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float3 exp3(float3 a) { return f3(__expf(a.x), __expf(a.y), __expf(a.z)); }

// Optical-depth step x >= 0: returns exp(-x) and phi = (1 - exp(-x)) / x, the
// factor of the analytic segment integral.  Below x = 0.25 both come from the
// Maclaurin series of 1 - e^{-x} = x (1 - x/2! + x^2/3! - ... + x^6/7!)
// (truncation < 1e-9 relative), which avoids the cancellation of 1 - e^{-x}
// and needs no exponential or reciprocal; above it the direct forms are exact
// enough.
__device__ __forceinline__ float seg_phi(float x, float& tr) {
    if (x < 0.25f) {
        float q = fmaf(x, 1.f / 5040.f, -1.f / 720.f);
        q = fmaf(x, q, 1.f / 120.f);
        q = fmaf(x, q, -1.f / 24.f);
        q = fmaf(x, q, 1.f / 6.f);
        q = fmaf(x, q, -0.5f);
        q = fmaf(x, q, 1.f);
        tr = fmaf(-x, q, 1.f);
        return q;
    }
    tr = __expf(-x);
    return __fdividef(1.f - tr, x);
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float t = clamp01((x - e0) / (e1 - e0));
    return t * t * (3.f - 2.f * t);
}

// ---------------------------------------------------------------------------
// Kernel constants of one atmosphere parameter set: AtmosphereBufferData
// (shaders/SkyRendering/Atmosphere.glsl:6-32) plus exactly-derived helpers
// (top^2 - bottom^2 etc.) computed on the host in double.
// ---------------------------------------------------------------------------
struct AtmoConsts {
    float3 solar_illuminance;
    float sun_angular_radius;  // radians
    float3 rayleigh_scattering;
    float inv_rayleigh_h;
    float3 mie_scattering;
    float inv_mie_h;
    float3 mie_extinction;  // scattering + absorption
    float ozone_center;
    float3 ozone_absorption;
    float inv_ozone_width;
    float3 ground_albedo;
    float mie_g;
    float ms_mask;
    float R;          // bottom radius
    float top;        // top radius
    float thickness;  // top - R
    float Hh;         // sqrt(top^2 - R^2): horizon distance at ground
    float R2;         // R^2
    float top2_minus_R2;
    float transmittance_steps;
    float multiscattering_steps;
    float mie_phase_k;  // 3/(8 pi) (1-g^2)/(2+g^2)
    float inv_Hh;        // 1 / Hh
    float inv_thickness;
    float inv_2R_alpha;  // 1 / (2 R sun_angular_radius)
    float pad0;
};

// Kernel constants of one view (AtmosphereRenderBufferData derived by
// AssignBufferData, src/SkyRendering/AtmosphereRenderer.cpp:52-83).
struct ViewConsts {
    float3 sun;    // world sun direction
    float3 up;     // camera up (from Earth centre)
    float3 right;
    float3 front;
    float cam_r;   // |camera - Earth centre|
    float cam_h;   // cam_r - R, from double
    float cam_rho2;  // cam_r^2 - R^2, from double
    float sky_view_steps;
    float ap_steps;
    float ap_max_distance;
    // Aerial-perspective froxel ray: dir(x, y) ~ sign * normalize(a0*x + a1*y + a3)
    // with x, y the NDC of the near-plane point (exact rewrite of
    // normalize(ProjectiveMul(inv_vp, (x, y, 0)) - camera)).
    float3 ap_a0, ap_a1, ap_a3;
    float ap_w0, ap_w1, ap_w3;
    float in_space;  // 1 if cam_r > top
    float pad0;
};

struct LutSetJob {
    AtmoConsts a;
    ViewConsts v;
};

// ---------------------------------------------------------------------------
// Ray / sphere geometry in cancellation-free FP32 form.  All take the point's
// radius r together with rho2 = r^2 - R^2 carried from an exact source, so
// that no r*r - R*R difference is ever formed in FP32.
// ---------------------------------------------------------------------------

// RayIntersectsGround (Atmosphere.glsl:57-59): mu < 0 && r^2 mu^2 >= r^2 - R^2
__device__ __forceinline__ bool ray_hits_ground(float r, float rho2, float mu) {
    float rm = r * mu;
    return mu < 0.f && rm * rm >= rho2;
}

// DistanceToBottomAtmosphereBoundary (Atmosphere.glsl:66-69) for a ray that
// hits the ground: -r mu - sqrt(r^2 mu^2 - rho2) = rho2 / (-r mu + sqrt(.)).
__device__ __forceinline__ float dist_to_bottom(float r, float rho2, float mu) {
    float rm = r * mu;
    float s = sqrtf(fmaxf(rm * rm - rho2, 0.f));
    float den = -rm + s;
    return den > 0.f ? fmaxf(rho2 / den, 0.f) : 0.f;
}

// DistanceToTopAtmosphereBoundary (Atmosphere.glsl:61-64):
// -r mu + sqrt(r^2 mu^2 + (top - r)(top + r)); the mu > 0 branch uses the
// conjugate form.  top_minus_r is passed from an exact source.
__device__ __forceinline__ float dist_to_top(float r, float top_minus_r, float top, float mu) {
    float rm = r * mu;
    float c = top_minus_r * (top + r);
    float s = sqrtf(fmaxf(rm * rm + c, 0.f));
    float d = rm > 0.f ? c / (rm + s) : s - rm;
    return fmaxf(d, 0.f);
}

// Host-side derivation (skyr_api.cu)
namespace skyr {
void derive_atmo_consts(const skyr_atmosphere_parameters& p, AtmoConsts& a);
void derive_view_consts(const skyr_atmosphere_parameters& p, const skyr_atmosphere_render_parameters& r,
                        ViewConsts& v);
}  // namespace skyr
