// lut_access.cuh — reads of the atmosphere LUTs shared by the LUT, cloud and
// path-tracer kernels: texel loads (RGBA32F or RGBA16F), GL LINEAR +
// CLAMP_TO_EDGE filtering and GetSunVisibility.
#pragma once

#include "skyr_internal.cuh"

namespace skyr {

__device__ __forceinline__ float3 load_lut_rgb(const float4* p, int i) {
    float4 v = __ldg(p + i);
    return f3(v.x, v.y, v.z);
}
__device__ __forceinline__ float3 load_lut_rgb(const __half2* p, int i) {  // half4 = 2 x half2
    uint2 raw = __ldg(reinterpret_cast<const uint2*>(p) + i);
    __half2 a = *reinterpret_cast<__half2*>(&raw.x);
    __half2 b = *reinterpret_cast<__half2*>(&raw.y);
    float2 fa = __half22float2(a), fb = __half22float2(b);
    return f3(fa.x, fa.y, fb.x);
}
__device__ __forceinline__ void store_rgba(float4* p, size_t i, float3 v, float a) {
    p[i] = make_float4(v.x, v.y, v.z, a);
}
__device__ __forceinline__ void store_rgba(__half2* p, size_t i, float3 v, float a) {
    __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, a);
    uint2 raw;
    raw.x = *reinterpret_cast<uint32_t*>(&lo);
    raw.y = *reinterpret_cast<uint32_t*>(&hi);
    reinterpret_cast<uint2*>(p)[i] = raw;
}

// GL LINEAR + CLAMP_TO_EDGE fetch at continuous texel coordinate
// (x, y) = (u*W - 0.5, v*H - 0.5).  Clamping the coordinate to [0, W-1] first
// selects the same texels and weights as clamping the two indices.
template <class S>
__device__ __forceinline__ float3 bilinear_clamp(const S* lut, int w, int h, float x, float y) {
    x = fminf(fmaxf(x, 0.f), (float)(w - 1));
    y = fminf(fmaxf(y, 0.f), (float)(h - 1));
    int x0 = min((int)x, w - 2), y0 = min((int)y, h - 2);
    float a = x - (float)x0, b = y - (float)y0;
    int i = y0 * w + x0;
    float3 t00 = load_lut_rgb(lut, i), t10 = load_lut_rgb(lut, i + 1);
    float3 t01 = load_lut_rgb(lut, i + w), t11 = load_lut_rgb(lut, i + w + 1);
    float3 top = t00 + (t10 - t00) * a;
    float3 bot = t01 + (t11 - t01) * a;
    return top + (bot - top) * b;
}

// GetTransmittanceToTopAtmosphereBoundary x horizon smoothstep =
// GetSunVisibility (Atmosphere.glsl:90-117) at a point of radius r with
// rho2 = r^2 - R^2 and altitude h = r - R carried from exact sources.
__device__ __forceinline__ float3 sun_visibility_lut(const AtmoConsts& A, const float4* t, int tw, int th, float r,
                                                     float rho2, float h, float mu_s) {
    float rho = sqrtf(fmaxf(rho2, 0.f));
    float d_min = A.thickness - h;
    float d = dist_to_top(r, d_min, A.top, mu_s);
    float d_max = rho + A.Hh;
    float x_mu = __fdividef(d - d_min, d_max - d_min);
    float x_r = rho * A.inv_Hh;
    float3 tr = bilinear_clamp(t, tw, th, x_mu * (float)(tw - 1), x_r * (float)(th - 1));
    // smoothstep(-e, e, mu_s - cos_h) with e = (R / r) alpha and cos_h = -rho / r:
    // the normalised argument is 1/2 + (mu_s r + rho) / (2 R alpha)
    float u = clamp01(fmaf(fmaf(mu_s, r, rho), A.inv_2R_alpha, 0.5f));
    return tr * (u * u * (3.f - 2.f * u));
}

// GL LINEAR + CLAMP_TO_EDGE fetch of a 3D LUT at continuous texel coordinate
// (x, y, z) = (u*W - 0.5, ...), by the same clamp-first rule.
template <class S>
__device__ __forceinline__ float3 trilinear_clamp(const S* lut, int w, int h, int d, float x, float y, float z) {
    x = fminf(fmaxf(x, 0.f), (float)(w - 1));
    y = fminf(fmaxf(y, 0.f), (float)(h - 1));
    z = fminf(fmaxf(z, 0.f), (float)(d - 1));
    int x0 = min((int)x, w - 2), y0 = min((int)y, h - 2), z0 = min((int)z, d - 2);
    float a = x - (float)x0, b = y - (float)y0, g = z - (float)z0;
    float3 r[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        int base = ((z0 + k) * h + y0) * w + x0;
        float3 t00 = load_lut_rgb(lut, base), t10 = load_lut_rgb(lut, base + 1);
        float3 t01 = load_lut_rgb(lut, base + w), t11 = load_lut_rgb(lut, base + w + 1);
        float3 top = t00 + (t10 - t00) * a, bot = t01 + (t11 - t01) * a;
        r[k] = top + (bot - top) * b;
    }
    return r[0] + (r[1] - r[0]) * g;
}

}  // namespace skyr
