// environment.cuh — the ENVIRONMENT_LUMINANCE program's radiance for a world
// direction (sky-view LUT + ground term), shared by the path tracer (which
// evaluates it per escaping direction) and the environment cube map.
#pragma once

#include "atmosphere_kernels.cuh"
#include "lut_access.cuh"

namespace skyr {

// GetCosLatLonFromViewDirection + GetSkyViewTextureUvFromCosLatLon
// (AtmosphereRenderer.glsl:113-145) and the sky-view LUT reads for world
// direction w seen from the view's camera.
template <class S>
__device__ __forceinline__ void sky_view_lookup(const ViewConsts& E, const S* svl, const S* svt, int sv_w, int sv_h,
                                                float3 w, float3& lum, float3& tr) {
    float cos_lat = dot3(E.up, w);
    float3 lon = w - E.up * cos_lat;
    float l2 = dot3(lon, lon);
    float cos_lon = l2 == 0.f ? 1.f : dot3(lon, E.front) * rsqrtf(l2);
    float r = E.cam_r;
    float hd = acosf(sqrtf(fmaxf(E.cam_rho2, 0.f)) / r);
    float hu = SKYR_PI - hd;
    float lat = acosf(fminf(fmaxf(cos_lat, -1.f), 1.f));
    float xl = lat < hu ? 0.5f - 0.5f * sqrtf(fmaxf(1.f - lat / hu, 0.f)) : sqrtf(fmaxf((lat - hu) / hd, 0.f)) * 0.5f + 0.5f;
    float xo = sqrtf(fmaxf(0.5f - 0.5f * cos_lon, 0.f));
    float x = xo * (float)(sv_w - 1), y = xl * (float)(sv_h - 1);
    lum = bilinear_clamp(svl, sv_w, sv_h, x, y);
    tr = bilinear_clamp(svt, sv_w, sv_h, x, y);
}

// ENVIRONMENT_LUMINANCE (AtmosphereRenderer.glsl:250-273) for world direction w:
// the sky-view luminance, plus the ground term x sky-view transmittance below
// the horizon.
template <class S>
__device__ float3 environment(const AtmoConsts& A, const ViewConsts& E, const float4* tlut, int tw, int th,
                              const S* svl, const S* svt, int sv_w, int sv_h, float3 w) {
    float3 lum, tr;
    sky_view_lookup(E, svl, svt, sv_w, sv_h, w, lum, tr);
    float cos_lat = dot3(E.up, w);
    float r = E.cam_r;
    if (ray_hits_ground(r, E.cam_rho2, cos_lat)) {
        float dist = dist_to_bottom(r, E.cam_rho2, cos_lat);
        float mu_s_g = fmaf(r, dot3(E.sun, E.up), dist * dot3(E.sun, w)) / A.R;
        float3 sv = sun_visibility_lut(A, tlut, tw, th, A.R, 0.f, 0.f, mu_s_g);
        lum += (A.ground_albedo * sv * A.solar_illuminance * (clamp01(mu_s_g) / SKYR_PI)) * tr;
    }
    return lum;
}

}  // namespace skyr
