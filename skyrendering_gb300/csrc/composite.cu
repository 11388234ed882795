// composite.cu — the full-screen atmosphere composite (include/skyr_composite.h):
// the ATMOSPHERE_RENDER fragment shader (AtmosphereRenderer.glsl:345-432) as
// one compute kernel over a viewport.
//
// The reference draws a screen rectangle; its default configuration raymarches
// every pixel (use_sky_view_lut and use_aerial_perspective_lut off,
// AtmosphereRenderer.h:49-51) with raymarching_steps samples and a blue-noise
// start.  Here each thread runs that raymarch with the LUT passes' FP32
// integrator (exact r^2 - R^2 forms, the analytic segment integral), or reads
// the sky-view / aerial-perspective LUTs when they are switched on.
#include <cmath>
#include <cstring>

#include <cuda_fp16.h>

#include "../../include/skyr_composite.h"
#include "atmosphere_integrate.cuh"
#include "cloud_internal.cuh"
#include "environment.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace {

struct CompositeConsts {
    // pixel ray relative to the camera (world space):
    // (frag - cam) = (a0 x + a1 y + a2 e + af) / (w0 x + w1 y + w2 e + wf), NDC x, y, e = z_ndc - 1
    float3 a0, a1, a2, af;
    float w0, w1, w2, wf;
    int width, height;
    float star_scale, steps;
    int use_sv, use_ap, dither;
    float cos_sun_radius, sin_sun_radius, sun_disc;  // sun disc: cos, sin, 1 / (pi r^2)
    const float* depth;
    const float4* object;
    const float* blue_noise;
    const uint8_t* stars;
    int star_w, star_h;
    const uint16_t* froxel;
    int fx_w, fx_h, fx_d;
    float inv_froxel_max;
    int sv_w, sv_h, ap_w, ap_h, ap_d;
};

// the sRGB EOTF of an 8-bit channel (GL decodes sRGB texels before filtering)
__device__ __forceinline__ float srgb_to_linear(uint8_t b) {
    float c = (float)b * (1.f / 255.f);
    return c <= 0.04045f ? c * (1.f / 12.92f) : powf((c + 0.055f) * (1.f / 1.055f), 2.4f);
}

__device__ __forceinline__ float3 star_texel(const CompositeConsts& K, int i, int j) {
    const uint8_t* p = K.stars + ((size_t)j * K.star_w + i) * 3;
    return f3(srgb_to_linear(__ldg(p)), srgb_to_linear(__ldg(p + 1)), srgb_to_linear(__ldg(p + 2)));
}

// GetStarLuminance (AtmosphereRenderer.glsl:325-330): LINEAR + CLAMP_TO_EDGE on the star map
__device__ __forceinline__ float3 star_luminance(const CompositeConsts& K, float3 view) {
    float theta = acosf(fminf(fmaxf(view.y, -1.f), 1.f));
    float phi = atan2f(view.x, view.z);
    float u = (0.5f / SKYR_PI) * phi + 0.5f, v = 1.f - theta * (1.f / SKYR_PI);
    float x = fminf(fmaxf(u * (float)K.star_w - 0.5f, 0.f), (float)(K.star_w - 1));
    float y = fminf(fmaxf(v * (float)K.star_h - 0.5f, 0.f), (float)(K.star_h - 1));
    int x0 = (int)x, y0 = (int)y, x1 = min(x0 + 1, K.star_w - 1), y1 = min(y0 + 1, K.star_h - 1);
    float a = x - (float)x0, b = y - (float)y0;
    float3 t00 = star_texel(K, x0, y0), t10 = star_texel(K, x1, y0);
    float3 t01 = star_texel(K, x0, y1), t11 = star_texel(K, x1, y1);
    float3 top = t00 + (t10 - t00) * a, bot = t01 + (t11 - t01) * a;
    return (top + (bot - top) * b) * K.star_scale;
}

// Registers are cut for 7 resident blocks per SM (72 registers, 32 B spilled,
// from 78): the kernel is issue-bound, and the extra warps fill issue slots
// (0.716 -> 0.671 ms per 1080p frame on a GB300; 8 blocks: 0.688 ms).
template <class S>
__global__ void __launch_bounds__(128, 7) composite_kernel(AtmoConsts A, ViewConsts V, CompositeConsts K,
                                                        LutView T, const S* __restrict__ ms, int mw, int mh,
                                                        const S* __restrict__ svl, const S* __restrict__ svt,
                                                        const S* __restrict__ apl, const S* __restrict__ apt,
                                                        uint2* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= K.width || py >= K.height) return;
    const size_t pix = (size_t)py * K.width + px;
    const float u = ((float)px + 0.5f) / (float)K.width, v = ((float)py + 0.5f) / (float)K.height;
    const float depth = K.depth ? __ldg(K.depth + pix) : 1.f;
    // fragment_position and view_direction (AtmosphereRenderer.glsl:346-348)
    const float x = 2.f * u - 1.f, y = 2.f * v - 1.f, e = 2.f * (depth - 1.f);
    float3 num = K.a0 * x + K.a1 * y + K.a2 * e + K.af;
    float wv = fmaf(K.w0, x, fmaf(K.w1, y, fmaf(K.w2, e, K.wf)));
    float len = sqrtf(dot3(num, num));
    float3 view = num * (copysignf(1.f, wv) / len);
    const float mu = dot3(view, V.up), nu = dot3(view, V.sun);
    // marching distance to the ground, the atmosphere's top or the object (:350-361)
    float marching = ray_hits_ground(V.cam_r, V.cam_rho2, mu) ? dist_to_bottom(V.cam_r, V.cam_rho2, mu)
                                                              : dist_to_top(V.cam_r, A.thickness - V.cam_h, A.top, mu);
    const bool object = depth != 1.f;
    if (object) marching = fminf(marching, len / fabsf(wv));
    RayStart s0 = ray_start(A, V, mu, nu, marching);
    float3 lum = f3(0.f), tr = f3(1.f);
    if (marching > 0.f) {
        if (!object && K.use_sv) {
            sky_view_lookup(V, svl, svt, K.sv_w, K.sv_h, view, lum, tr);
        } else if (object && K.use_ap) {
            // GetAerialPerspectiveTextureUvwFromTexCoordDistance (AtmosphereInterface.glsl:19-23)
            float wz = sqrtf(marching / V.ap_max_distance);
            float ax = u * (float)(K.ap_w - 1), ay = v * (float)(K.ap_h - 1), az = wz * (float)(K.ap_d - 1);
            lum = trilinear_clamp(apl, K.ap_w, K.ap_h, K.ap_d, ax, ay, az);
            tr = trilinear_clamp(apt, K.ap_w, K.ap_h, K.ap_d, ax, ay, az);
        } else {
            float start_i = K.dither ? __ldg(K.blue_noise + (py & 63) * 64 + (px & 63)) : 0.5f;
            float ph_r = 3.f / (16.f * SKYR_PI) * (1.f + nu * nu);
            float g = A.mie_g;
            float den = 1.f + g * g - 2.f * g * nu;
            float ph_m = A.mie_phase_k * (1.f + nu * nu) / (den * sqrtf(den));
            float3 lf;
            integrate<false, S>(A, T, ms, mw, mh, s0, marching / K.steps, start_i, 0, sample_count(start_i, K.steps),
                                ph_r, ph_m, lum, tr, lf);
        }
    }
    // SampleRayScatterVisibility (:399)
    lum = lum * froxel_visibility_at(K.froxel, K.fx_w, K.fx_h, K.fx_d, K.inv_froxel_max, u, v, marching);
    if (object) {
        if (K.object) {
            float4 o = __ldg(K.object + pix);
            lum += tr * f3(o.x, o.y, o.z);
        }
    } else if (nu >= K.cos_sun_radius) {
        // sun limb darkening (:407-423): u = 1, a = (0.397, 0.503, 0.652).  The
        // sine of the view-sun angle is |view x sun|: sqrt(1 - cos^2) cancels
        // in FP32 at the disc's 1/4 degree, where the limb factor's slope is infinite
        float3 cx = f3(view.y * V.sun.z - view.z * V.sun.y, view.z * V.sun.x - view.x * V.sun.z,
                       view.x * V.sun.y - view.y * V.sun.x);
        float sin_vs = sqrtf(dot3(cx, cx));
        float c2e = clamp01(sin_vs / K.sin_sun_radius);
        float m = sqrtf(1.f - c2e * c2e);
        float3 factor = f3(1.f - (1.f - powf(m, 0.397f)), 1.f - (1.f - powf(m, 0.503f)), 1.f - (1.f - powf(m, 0.652f)));
        lum += A.solar_illuminance * tr * factor * K.sun_disc;
    } else if (K.stars) {
        lum += tr * star_luminance(K, view);
    }
    __half2 lo = __floats2half2_rn(lum.x, lum.y), hi = __floats2half2_rn(lum.z, 1.f);
    uint2 raw;
    raw.x = *reinterpret_cast<uint32_t*>(&lo);
    raw.y = *reinterpret_cast<uint32_t*>(&hi);
    out[pix] = raw;
}

}  // namespace
}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_composite_parameters_default(skyr_composite_parameters* out) {
    if (!out) return set_error(SKYR_EINVAL, "null parameters");
    // AtmosphereRenderParameters / AtmosphereRenderInitParameters defaults (AtmosphereRenderer.h:14-52)
    out->star_luminance_scale = 0.005f;
    out->raymarching_steps = 40.f;
    out->use_sky_view_lut = 0;
    out->use_aerial_perspective_lut = 0;
    out->dither_sample_point = 1;
    return SKYR_OK;
}

int skyr_atmosphere_composite(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_atmosphere_render_parameters* render,
                              const skyr_composite_parameters* parameters, const skyr_lut_sizes* sizes,
                              const void* transmittance, const void* multiscattering,
                              const void* sky_view_luminance, const void* sky_view_transmittance,
                              const void* aerial_perspective_luminance,
                              const void* aerial_perspective_transmittance, const skyr_composite_inputs* in,
                              void* out_hdr) {
    if (!ctx || !atmosphere || !render || !parameters || !sizes || !in || !out_hdr)
        return set_error(SKYR_EINVAL, "null argument");
    if (!transmittance || !multiscattering) return set_error(SKYR_EINVAL, "null transmittance or MS LUT");
    if (parameters->use_sky_view_lut && (!sky_view_luminance || !sky_view_transmittance))
        return set_error(SKYR_EINVAL, "use_sky_view_lut needs the sky-view LUTs");
    if (parameters->use_aerial_perspective_lut && (!aerial_perspective_luminance || !aerial_perspective_transmittance))
        return set_error(SKYR_EINVAL, "use_aerial_perspective_lut needs the aerial-perspective LUTs");
    if (!(parameters->raymarching_steps >= 1.f) || parameters->raymarching_steps > 4096.f)
        return set_error(SKYR_EINVAL, "raymarching_steps must be in [1, 4096]");
    if (parameters->dither_sample_point && !in->blue_noise) return set_error(SKYR_EINVAL, "dither needs blue noise");
    if (in->width < 1 || in->height < 1 || in->width > 16384 || in->height > 16384)
        return set_error(SKYR_EINVAL, "viewport must be in [1, 16384]");
    if (in->star_map && (in->star_width < 1 || in->star_height < 1))
        return set_error(SKYR_EINVAL, "bad star map size");
    if (in->shadow_froxel && (in->froxel_width < 1 || in->froxel_height < 1 || in->froxel_depth < 1 ||
                              !(in->shadow_froxel_max_distance > 0.f)))
        return set_error(SKYR_EINVAL, "bad shadow froxel size or distance");
    if (int st = validate_atmosphere(atmosphere, 0)) return st;
    if (int st = validate_render(render, atmosphere, 0)) return st;
    if (int st = validate_sizes(sizes, true)) return st;
    AtmoConsts A;
    derive_atmo_consts(*atmosphere, A);
    ViewConsts V;
    derive_view_consts(*atmosphere, *render, V);
    CompositeConsts K;
    std::memset(&K, 0, sizeof(K));
    {
        // the inverse view-projection's columns relative to the camera, in double
        double vp[16], ivp[16];
        for (int i = 0; i < 16; ++i) vp[i] = render->view_projection[i];
        if (!invert4d(vp, ivp)) return set_error(SKYR_EINVAL, "view_projection is singular");
        const double cam[3] = {render->camera_position[0], render->camera_position[1], render->camera_position[2]};
        auto col = [&](int k, int r) { return ivp[k * 4 + r] - cam[r] * ivp[k * 4 + 3]; };
        K.a0 = make_float3((float)col(0, 0), (float)col(0, 1), (float)col(0, 2));
        K.a1 = make_float3((float)col(1, 0), (float)col(1, 1), (float)col(1, 2));
        K.a2 = make_float3((float)col(2, 0), (float)col(2, 1), (float)col(2, 2));
        K.af = make_float3((float)(col(2, 0) + col(3, 0)), (float)(col(2, 1) + col(3, 1)), (float)(col(2, 2) + col(3, 2)));
        K.w0 = (float)ivp[3];
        K.w1 = (float)ivp[7];
        K.w2 = (float)ivp[11];
        K.wf = (float)(ivp[11] + ivp[15]);
    }
    K.width = in->width;
    K.height = in->height;
    K.star_scale = parameters->star_luminance_scale;
    K.steps = parameters->raymarching_steps;
    K.use_sv = parameters->use_sky_view_lut ? 1 : 0;
    K.use_ap = parameters->use_aerial_perspective_lut ? 1 : 0;
    K.dither = parameters->dither_sample_point ? 1 : 0;
    const double sar = (double)A.sun_angular_radius;
    K.cos_sun_radius = (float)std::cos(sar);
    K.sin_sun_radius = (float)std::sin(sar);
    K.sun_disc = (float)(1.0 / (M_PI * sar * sar));
    K.depth = in->depth;
    K.object = reinterpret_cast<const float4*>(in->object_luminance);
    K.blue_noise = in->blue_noise;
    K.stars = in->star_map;
    K.star_w = in->star_width;
    K.star_h = in->star_height;
    K.froxel = in->shadow_froxel;
    K.fx_w = in->froxel_width;
    K.fx_h = in->froxel_height;
    K.fx_d = in->froxel_depth;
    K.inv_froxel_max = in->shadow_froxel ? (float)(1.0 / in->shadow_froxel_max_distance) : 0.f;
    K.sv_w = sizes->sky_view_width;
    K.sv_h = sizes->sky_view_height;
    K.ap_w = sizes->aerial_perspective_width;
    K.ap_h = sizes->aerial_perspective_height;
    K.ap_d = sizes->aerial_perspective_depth;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    LutView T{reinterpret_cast<const float4*>(transmittance), sizes->transmittance_width, sizes->transmittance_height};
    dim3 block(16, 8), grid((in->width + 15) / 16, (in->height + 7) / 8);
    uint2* o = reinterpret_cast<uint2*>(out_hdr);
    const int mw = sizes->multiscattering_width, mh = sizes->multiscattering_height;
    if (sizes->format == SKYR_FORMAT_RGBA16F) {
        using S = __half2;
        composite_kernel<S><<<grid, block, 0, ctx->stream>>>(
            A, V, K, T, reinterpret_cast<const S*>(multiscattering), mw, mh,
            reinterpret_cast<const S*>(sky_view_luminance), reinterpret_cast<const S*>(sky_view_transmittance),
            reinterpret_cast<const S*>(aerial_perspective_luminance),
            reinterpret_cast<const S*>(aerial_perspective_transmittance), o);
    } else {
        using S = float4;
        composite_kernel<S><<<grid, block, 0, ctx->stream>>>(
            A, V, K, T, reinterpret_cast<const S*>(multiscattering), mw, mh,
            reinterpret_cast<const S*>(sky_view_luminance), reinterpret_cast<const S*>(sky_view_transmittance),
            reinterpret_cast<const S*>(aerial_perspective_luminance),
            reinterpret_cast<const S*>(aerial_perspective_transmittance), o);
    }
    return check_cuda(cudaGetLastError(), "composite kernel");
}

}  // extern "C"
