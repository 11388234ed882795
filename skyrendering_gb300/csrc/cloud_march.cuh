// cloud_march.cuh — the device side of the volumetric-cloud raymarch
// (VolumetricCloudRender.comp): light march, shell segments, shell
// intersections and the raymarch kernel template.  Included by the
// translation units that instantiate the kernel for each launch shape.
#pragma once

#include <type_traits>

#include "atmosphere_kernels.cuh"
#include "cloud_fast.cuh"
#include "cloud_internal.cuh"
#include "cloud_material.cuh"
#include "lut_access.cuh"

namespace skyr {
// ---------------------------------------------------------------------------
// Device: the raymarch
// ---------------------------------------------------------------------------
__device__ __forceinline__ float hg(float c, float g) {  // VolumetricCloudCommon.glsl:58-63
    float a = 1.f - g * g;
    float b = fmaf(-2.f * g, c, 1.f + g * g);
    return (0.25f / SKYR_PI) * __fdividef(a, b * sqrtf(b));
}

// 1 - exp(-x) without cancellation (x >= 0); also returns exp(-x)
__device__ __forceinline__ float one_minus_exp(float x, float& e) {
    float phi = seg_phi(x, e);
    return x * phi;
}

// SampleShadow (VolumetricCloudRender.comp:98-114).  The loop variable
// accumulates in FP32 exactly as the reference's `t += inv_shadow_steps`.
// Sample heights come from rho2(d) = rho2_p + d (2 q + d) with
// q = sun . (p + R z^), exact relative to the primary sample.  FAST: the
// density of cloud_fast.cuh (MaterialConsts::fast_ok).
template <bool FAST, bool COUNT = false>
__device__ __forceinline__ float sample_shadow(const CloudConsts& C, const MaterialConsts& M, float3 pos,
                                               float rho2_p, unsigned* n_detail = nullptr) {
    // Products whose results have several uses are rounded explicitly (_rn), so
    // that no later pass may fuse them into a neighbouring add: every launch
    // shape (register cut, lanes per ray) then gives the same bits.
    float od = 0.f;
    float inv = 1.f / C.shadow_steps;
    float3 sv = C.sun * C.shadow_distance;
    float q2 = 2.f * fmaf(C.sun.x, pos.x, fmaf(C.sun.y, pos.y, C.sun.z * (pos.z + C.R)));
    float prev = 0.f;
    for (float t = inv; t <= 1.f; t += inv) {
        float cur = __fmul_rn(t, t);
        float dt = __fsub_rn(cur, prev);
        float f = fmaf(0.5f, dt, prev);
        float3 sp = make_float3(fmaf(sv.x, f, pos.x), fmaf(sv.y, f, pos.y), fmaf(sv.z, f, pos.z));
        float d = __fmul_rn(C.shadow_distance, f);
        float rho2 = fmaf(d, __fadd_rn(q2, d), rho2_p);
        float h = FAST ? fast_height01(M.fast, rho2) : height01_rho2(C, rho2);
        float3 dc = sp - C.cam;
        float sigma;
        if constexpr (FAST) sigma = fast_sigma_m1<COUNT>(M, sp, h, dot3(dc, dc), n_detail);
        else sigma = sigma_t<COUNT>(C, M, sp, h, sqrtf(dot3(dc, dc)), n_detail);
        od = fmaf(__fmul_rn(sigma, C.shadow_distance), dt, od);
        prev = cur;
    }
    return __expf(-od);
}

// number of light-march samples of `for (float t = inv; t <= 1; t += inv)`
__device__ __forceinline__ unsigned shadow_sample_count(float steps) {
    unsigned n = 0;
    float inv = 1.f / steps;
    for (float t = inv; t <= 1.f; t += inv) ++n;
    return n;
}

struct March {
    float trans, trans_sum, wsum, sun, env;
    // work counters of instrumented launches (COUNT): raymarch samples, density
    // evaluations, evaluations that sampled the detail texture
    unsigned samples, evals, detail;
};

// One shell segment [t0, t1] of the raymarch loop (VolumetricCloudRender.comp:160-187).
// Sample heights are taken relative to the segment entry, whose
// rho2_e = R_e^2 - R^2 is exact: rho2(t0 + e) = rho2_e + e (k_e + e) with
// k_e = 2 (r mu + t0) = 2 R_e mu_e.  COUNT: fill S's work counters; FAST: the
// density of cloud_fast.cuh.
template <bool FAST, bool COUNT>
__device__ __forceinline__ void march_segment(const CloudConsts& C, const MaterialConsts& M, float3 view,
                                              float t0, float t1, float rho2_e, float k_e, float jitter,
                                              float ph_back, float ph_fwd, March& S) {
    float dist = fminf(t1 - t0, C.max_raymarch_distance);
    unsigned n = (unsigned)fmaxf(C.max_raymarch_steps * (dist / C.max_raymarch_distance), 1.f);
    float step = dist / (float)n;
    float e = __fmul_rn(step, jitter);
    float t = __fadd_rn(t0, e);
    unsigned light_samples = 0;
    if constexpr (COUNT) light_samples = shadow_sample_count(C.shadow_steps);
    for (unsigned k = n; k != 0; --k, t += step, e += step) {
        float3 pos = make_float3(fmaf(view.x, t, C.cam.x), fmaf(view.y, t, C.cam.y), fmaf(view.z, t, C.cam.z));
        float rho2 = fmaf(e, k_e + e, rho2_e);
        float h = FAST ? fast_height01(M.fast, rho2) : height01_rho2(C, rho2);
        // RayMarchStep (VolumetricCloudRender.comp:116-137)
        float sigma;
        if constexpr (FAST) sigma = fast_sigma_m1<COUNT>(M, pos, h, t * t, &S.detail);
        else sigma = sigma_t<COUNT>(C, M, pos, h, t, &S.detail);
        if constexpr (COUNT) {
            S.samples++;
            S.evals++;
        }
        if (sigma >= 1e-5f) {
            if constexpr (COUNT) S.evals += light_samples;
            float tr;
            float one_m_tr = one_minus_exp(step * sigma, tr);
            float tsun = sample_shadow<FAST, COUNT>(C, M, pos, rho2, &S.detail);
            float w = __expf(-C.sun_ms_sigma_scale * sigma);
            float phase = ph_back * (1.f - w) + ph_fwd * w;
            float e_dummy;
            float env = fmaf(h, 1.f - C.env_bottom_visibility, C.env_bottom_visibility) *
                        one_minus_exp(C.env_ms_sigma_scale * sigma, e_dummy);
            S.sun += S.trans * (tsun * phase) * one_m_tr;
            S.env += S.trans * env * one_m_tr;
            S.trans_sum += S.trans;
            S.wsum += t * S.trans;
            S.trans *= tr;
        }
        if (S.trans < 0.01f) break;
    }
}

// march_segment with the steps of one ray spread over a group of G lanes
// (G = 2, 4, 8): in each round lane `sub` evaluates step k0 + sub (density, light
// march, phase and extinction terms, which do not depend on the running
// state), then every lane of the group folds the round's G steps into the
// running state in step order with the same FP32 operations as march_segment,
// stopping where it stops (T < 0.01).  It keeps no work counters: instrumented
// launches use one lane per ray.  The step positions are the same
// repeated FP32 sums `t += step`, so the result equals march_segment's; the
// group only shortens the chain of dependent texture reads per ray, which
// bounds launches with few rays per SM (the quarter-resolution pass).
template <int G, bool FAST>
__device__ __forceinline__ void march_segment_lanes(const CloudConsts& C, const MaterialConsts& M, float3 view,
                                                    float t0, float t1, float rho2_e, float k_e, float jitter,
                                                    float ph_back, float ph_fwd, March& S, int sub,
                                                    unsigned gmask) {
    float dist = fminf(t1 - t0, C.max_raymarch_distance);
    unsigned n = (unsigned)fmaxf(C.max_raymarch_steps * (dist / C.max_raymarch_distance), 1.f);
    float step = dist / (float)n;
    float e = __fmul_rn(step, jitter);
    float t = __fadd_rn(t0, e);
    for (unsigned k0 = 0; k0 < n; k0 += G) {
        float tk = t, ek = e;
#pragma unroll
        for (int i = 1; i < G; ++i) {
            if (i <= sub) {
                tk += step;
                ek += step;
            }
        }
        float sigma = 0.f, tp = 0.f, omt = 0.f, env = 0.f, tr = 1.f;
        if (k0 + (unsigned)sub < n) {
            float3 pos = make_float3(fmaf(view.x, tk, C.cam.x), fmaf(view.y, tk, C.cam.y), fmaf(view.z, tk, C.cam.z));
            float rho2 = fmaf(ek, k_e + ek, rho2_e);
            float h = FAST ? fast_height01(M.fast, rho2) : height01_rho2(C, rho2);
            if constexpr (FAST) sigma = fast_sigma_m1(M, pos, h, tk * tk);
            else sigma = sigma_t(C, M, pos, h, tk);
            if (sigma >= 1e-5f) {
                omt = one_minus_exp(step * sigma, tr);
                float tsun = sample_shadow<FAST>(C, M, pos, rho2);
                float w = __expf(-C.sun_ms_sigma_scale * sigma);
                float phase = ph_back * (1.f - w) + ph_fwd * w;
                float e_dummy;
                env = fmaf(h, 1.f - C.env_bottom_visibility, C.env_bottom_visibility) *
                      one_minus_exp(C.env_ms_sigma_scale * sigma, e_dummy);
                tp = tsun * phase;
            }
        }
        bool stop = false;
#pragma unroll
        for (int j = 0; j < G; ++j) {
            float sj = __shfl_sync(gmask, sigma, j, G), tpj = __shfl_sync(gmask, tp, j, G);
            float omtj = __shfl_sync(gmask, omt, j, G), envj = __shfl_sync(gmask, env, j, G);
            float trj = __shfl_sync(gmask, tr, j, G), tj = __shfl_sync(gmask, tk, j, G);
            if (!stop && k0 + (unsigned)j < n) {
                if (sj >= 1e-5f) {
                    S.sun += S.trans * tpj * omtj;
                    S.env += S.trans * envj * omtj;
                    S.trans_sum += S.trans;
                    S.wsum += tj * S.trans;
                    S.trans *= trj;
                }
                if (S.trans < 0.01f) stop = true;
            }
        }
        if (stop) break;
#pragma unroll
        for (int i = 0; i < G; ++i) {
            t += step;
            e += step;
        }
    }
}

// Shell intersections (RayShellIntersect, VolumetricCloudRender.comp:39-71) in
// cancellation-free form: with c = (R_x - r)(R_x + r), -r mu + sqrt(d) equals
// c / (r mu + sqrt(d)) for mu > 0, and -r mu - sqrt(d) equals
// -c / (-r mu + sqrt(d)) for mu < 0.
__device__ __forceinline__ void shell_intersect(const CloudConsts& C, float mu, float t[4], float e[2]) {
    float r = C.R + C.cam.z;
    float rm = r * mu;
    float cb = (C.bottom - C.cam.z) * (C.rb + r);
    float ct = (C.top - C.cam.z) * (C.rt + r);
    float db = fmaf(rm, rm, cb), dt = fmaf(rm, rm, ct);
    float sb = sqrtf(fmaxf(db, 0.f)), st = sqrtf(fmaxf(dt, 0.f));
    auto plus = [&](float c, float s) { return rm > 0.f ? c / (rm + s) : s - rm; };
    auto minus = [&](float c, float s) { return -c / (s - rm); };
    t[0] = t[1] = t[2] = t[3] = 0.f;
    // entry rho2 of each segment: the bottom / top sphere or the camera
    e[0] = C.cam_rho2;
    e[1] = C.rho2_bottom;
    if (C.cam.z < C.bottom) {
        t[0] = plus(cb, sb);
        t[1] = plus(ct, st);
        e[0] = C.rho2_bottom;
    } else if (C.cam.z < C.top) {
        if (db >= 0.f && mu < 0.f) {
            t[1] = minus(cb, sb);
            t[2] = sb - rm;
            t[3] = st - rm;
        } else {
            t[1] = plus(ct, st);
        }
    } else {
        if (db >= 0.f && mu < 0.f) {
            t[0] = minus(ct, st);
            t[1] = minus(cb, sb);
            t[2] = sb - rm;
            t[3] = st - rm;
            e[0] = C.rho2_top;
        } else if (dt >= 0.f && mu < 0.f) {
            t[0] = minus(ct, st);
            t[1] = st - rm;
            e[0] = C.rho2_top;
        }
    }
}

// MINB: resident blocks per SM the register budget is cut for (a tuning
// choice, skyr_tuning::cloud_blocks_per_sm).  G: lanes per ray
// (skyr_tuning::cloud_ray_lanes); a warp then covers 32 / G rays.  COUNT (with
// G = 1): the instrumented launch, which adds the frame's raymarch samples,
// density evaluations and detail-texture evaluations to counters[0..2].
// FAST: the density evaluation of cloud_fast.cuh (only when M.fast_ok).  The
// parameter blocks are __grid_constant__: device code reads them in place
// (a run-time index into them is a constant load, not a local copy).
template <class S, int MINB, int G, bool COUNT, bool FAST>
__global__ void __launch_bounds__(128, MINB) cloud_render_kernel(const __grid_constant__ CloudConsts C,
                                                           const __grid_constant__ MaterialConsts M, AtmoConsts A,
                                                           const float4* __restrict__ tlut, int tw, int th,
                                                           const S* __restrict__ ap_lum,
                                                           const S* __restrict__ ap_trans,
                                                           const float* __restrict__ blue_noise,
                                                           const float* __restrict__ depth,
                                                           __half2* __restrict__ out_rgba,
                                                           float* __restrict__ out_dist,
                                                           unsigned long long* __restrict__ counters,
                                                           int tile_w, int warps_x) {
    // a warp covers rw x (32 / G / rw) pixels, rw = min(tile_w, 32 / G); the
    // block's 4 warps sit warps_x across and 4 / warps_x down (skyr_tuning)
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int ray = lane / G, sub = lane % G;
    int rw = min(tile_w, 32 / G), tile_h = 32 / G / rw, warps_y = 4 / warps_x;
    int px = blockIdx.x * (rw * warps_x) + (warp % warps_x) * rw + (ray % rw);
    int py = march_row((int)blockIdx.y, (int)gridDim.y, C.row_pivot, C.row_dir) * (tile_h * warps_y) +
             (warp / warps_x) * tile_h + (ray / rw);
    if (px >= C.width || py >= C.height) return;  // the whole ray group leaves together
    const unsigned gmask = G == 1 ? 1u << lane : ((1u << G) - 1u) << (lane & ~(G - 1));
    size_t pix = (size_t)py * C.width + px;
    float u, v, e;
    if (C.cb_index) {
        // VolumetricCloudRender.comp:140-146: the checkerboard texel chosen
        // for this frame gives the ray; (px, py) the noise and the output
        unsigned idx = (unsigned)(int)__ldg(&C.cb_index[pix].x) & 3u;
        int cx = 2 * px + (int)(((idx + 1u) >> 1) & 1u), cy = 2 * py + (int)(((idx + 2u) >> 1) & 1u);
        u = ((float)cx + 0.5f) / (float)C.cb_w;
        v = ((float)cy + 0.5f) / (float)C.cb_h;
        e = 2.f * (__ldg(C.cb_depth + (size_t)cy * C.cb_w + cx) - 1.f);
    } else {
        u = ((float)px + 0.5f) / (float)C.width;
        v = ((float)py + 0.5f) / (float)C.height;
        e = depth ? 2.f * (__ldg(depth + pix) - 1.f) : 0.f;
    }
    float x = 2.f * u - 1.f, y = 2.f * v - 1.f;
    float3 dir = C.a0 * x + C.a1 * y + C.a2 * e + C.af;
    float wv = fmaf(C.w0, x, fmaf(C.w1, y, fmaf(C.w2, e, C.wf)));
    float len = sqrtf(dot3(dir, dir));
    float3 view = dir * (copysignf(1.f, wv) / len);
    float frag_dist = len / fabsf(wv);
    float mu = view.z;
    float it[4], ent[2];
    shell_intersect(C, mu, it, ent);
    float vis = fminf(frag_dist, C.max_visible_distance);
    it[1] = fminf(fmaxf(vis, it[0]), it[1]);
    it[3] = fminf(fmaxf(vis, it[2]), it[3]);
    float cos_sv = dot3(C.sun, view);
    float ph_back = hg(cos_sv, C.g_back) * C.back_scale, ph_fwd = hg(cos_sv, C.g_fwd);
    float noise = __ldg(blue_noise + (py & 63) * 64 + (px & 63));
    float j = noise + C.jitter_offset;
    float jitter = j - floorf(j);
    March mk{1.f, 0.f, 0.f, 0.f, 0.f, 0u, 0u, 0u};
    float rmu = (C.R + C.cam.z) * mu;
    // the (up to) two shell segments share one inlined copy of the march
#pragma unroll 1
    for (int sg = 0; sg < 2; ++sg) {
        float t0 = sg ? it[2] : it[0], t1 = sg ? it[3] : it[1];
        if (sg && !(t1 - t0 > 0.f)) break;
        if constexpr (G == 1)
            march_segment<FAST, COUNT>(C, M, view, t0, t1, sg ? ent[1] : ent[0], 2.f * (rmu + t0), jitter, ph_back,
                                       ph_fwd, mk);
        else
            march_segment_lanes<G, FAST>(C, M, view, t0, t1, sg ? ent[1] : ent[0], 2.f * (rmu + t0), jitter,
                                         ph_back, ph_fwd, mk, sub, gmask);
    }

    // The LUTs are first read here.  A raymarch launched as a programmatic
    // dependent of the view-LUT pass (skyr_render_frame) marches while the LUT
    // passes finish and waits here for them to complete; for any other launch
    // this is a no-op.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    float avg_t = mk.wsum == 0.f ? frag_dist : mk.wsum / mk.trans_sum;
    float3 ap = C.cam + view * avg_t;
    // GetSunVisibility(transmittance_texture, pos) at the mean depth
    float rho2 = fmaf(ap.x, ap.x, fmaf(ap.y, ap.y, ap.z * (ap.z + 2.f * C.R)));
    float r2 = fmaf(C.R, C.R, rho2);
    float inv_r = rsqrtf(r2);
    float rr = r2 * inv_r;
    float hh = __fdividef(rho2, rr + C.R);
    float mu_s = fmaf(C.sun.x, ap.x, fmaf(C.sun.y, ap.y, C.sun.z * (ap.z + C.R))) * inv_r;
    float3 sunvis = sun_visibility_lut(A, tlut, tw, th, rr, rho2, hh, mu_s);
    float sun_cos = clamp01(mu_s);
    float3 lum = sunvis * (mk.sun * C.sun_illuminance_scale) * A.solar_illuminance +
                 C.env_color_scale * (mk.env * __powf(sun_cos, C.env_sun_height_curve_exp));
    // GetAerialPerspective (VolumetricCloudCommon.glsl:81-98)
    float ta = avg_t;
    if (C.atmo_in_space != 0.f) {
        float r = C.R + C.cam.z, rm = r * mu;
        float c = (C.cam.z - A.thickness) * (r + A.top);
        float disc = rm * rm - c;
        if (mu < 0.f && disc >= 0.f) ta -= fmaxf(c / (-rm + sqrtf(disc)), 0.f);
        else ta = 0.f;
    }
    float wz = sqrtf(fmaxf(ta, 0.f) * C.inv_ap_max_distance);
    float3 at = trilinear_clamp(ap_trans, C.ap_w, C.ap_h, C.ap_d, u * (float)(C.ap_w - 1), v * (float)(C.ap_h - 1),
                                wz * (float)(C.ap_d - 1));
    float3 al = trilinear_clamp(ap_lum, C.ap_w, C.ap_h, C.ap_d, u * (float)(C.ap_w - 1), v * (float)(C.ap_h - 1),
                                wz * (float)(C.ap_d - 1));
    al = al * froxel_visibility(C, u, v, avg_t);  // VolumetricCloudRender.comp:198
    lum = lum * at + al * (1.f - mk.trans);
    lum = lum * (1.f / fmaxf(1e-5f, 1.f - mk.trans));
    float fade = smoothstepf(C.max_visible_distance * 0.75f, C.max_visible_distance, it[0]);
    float trans = mk.trans + (1.f - mk.trans) * fade;
    lum = lum * (1.f - trans);
    if (out_rgba && sub == 0) {
        __half2 lo = __floats2half2_rn(lum.x, lum.y), hi = __floats2half2_rn(lum.z, trans);
        uint2 raw;
        raw.x = *reinterpret_cast<uint32_t*>(&lo);
        raw.y = *reinterpret_cast<uint32_t*>(&hi);
        reinterpret_cast<uint2*>(out_rgba)[pix] = raw;
    }
    if (out_dist && sub == 0) out_dist[pix] = avg_t;
    if constexpr (COUNT) {
        static_assert(G == 1, "instrumented launches use one lane per ray");
        unsigned long long a = mk.samples, b = mk.evals, c = mk.detail;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(__activemask(), a, o);
            b += __shfl_xor_sync(__activemask(), b, o);
            c += __shfl_xor_sync(__activemask(), c, o);
        }
        if ((threadIdx.x & 31) == __ffs(__activemask()) - 1) {
            atomicAdd(counters, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
        }
    }
}

// Launches the raymarch kernel for G lanes per ray and the register cut MINB
// (resident blocks per SM: 5 to 10) with the LUT storage type (half:
// RGBA16F, else RGBA32F) and the density evaluation M.fast_ok selects.  Every (G, MINB) pair is instantiated in one of the
// cloud_raymarch_l<G>_c<cuts>.cu translation units, two cuts per unit, so the
// kernel variants compile in parallel.
template <int G, int MINB>
void launch_cloud_render_cut(bool half, dim3 grid, cudaStream_t stream, const CloudConsts& C,
                             const MaterialConsts& M, const AtmoConsts& A, const float4* tlut, int tw, int th,
                             const void* ap_lum, const void* ap_trans, const float* blue_noise, const float* depth,
                             __half2* out_rgba, float* out_dist, unsigned long long* counters, int tile_w,
                             int warps_x, bool pdl) {
    // pdl: a programmatic dependent launch (programmatic stream serialisation),
    // whose blocks may start before the previous kernel on the stream ends
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    auto go = [&](auto tag, auto fast) {
        using S = decltype(tag);
        cudaLaunchKernelEx(&cfg, cloud_render_kernel<S, MINB, G, false, decltype(fast)::value>, C, M, A, tlut, tw, th,
                           reinterpret_cast<const S*>(ap_lum), reinterpret_cast<const S*>(ap_trans), blue_noise,
                           depth, out_rgba, out_dist, counters, tile_w, warps_x);
    };
    using Fast = std::true_type;
    using General = std::false_type;
    if (half) {
        if (M.fast_ok) go(__half2{}, Fast{});
        else go(__half2{}, General{});
    } else {
        if (M.fast_ok) go(float4{}, Fast{});
        else go(float4{}, General{});
    }
}

#define SKYR_CLOUD_CUT_SIGNATURE(G, B)                                                                          \
    void launch_cloud_render_cut<G, B>(bool, dim3, cudaStream_t, const CloudConsts&, const MaterialConsts&,    \
                                       const AtmoConsts&, const float4*, int, int, const void*, const void*,   \
                                       const float*, const float*, __half2*, float*, unsigned long long*, int, \
                                       int, bool)
#define SKYR_CLOUD_CUTS(X, G) X(G, 5); X(G, 6); X(G, 7); X(G, 8); X(G, 9); X(G, 10)
#define SKYR_CLOUD_CUT_EXTERN(G, B) extern template SKYR_CLOUD_CUT_SIGNATURE(G, B)
SKYR_CLOUD_CUTS(SKYR_CLOUD_CUT_EXTERN, 1);
SKYR_CLOUD_CUTS(SKYR_CLOUD_CUT_EXTERN, 2);
SKYR_CLOUD_CUTS(SKYR_CLOUD_CUT_EXTERN, 4);
SKYR_CLOUD_CUTS(SKYR_CLOUD_CUT_EXTERN, 8);

// The instrumented raymarch (one lane per ray, counters[0..2]); its own
// translation unit (cloud_raymarch_counted.cu).
void launch_cloud_render_counted(bool half, dim3 grid, cudaStream_t stream, const CloudConsts& C,
                                 const MaterialConsts& M, const AtmoConsts& A, const float4* tlut, int tw, int th,
                                 const void* ap_lum, const void* ap_trans, const float* blue_noise,
                                 const float* depth, __half2* out_rgba, float* out_dist,
                                 unsigned long long* counters, int tile_w, int warps_x);

// The raymarch launch for G lanes per ray at the tuning's register cut.
template <int G>
void launch_cloud_render(bool half, int blocks_per_sm, dim3 grid, cudaStream_t stream, const CloudConsts& C,
                         const MaterialConsts& M, const AtmoConsts& A, const float4* tlut, int tw, int th,
                         const void* ap_lum, const void* ap_trans, const float* blue_noise, const float* depth,
                         __half2* out_rgba, float* out_dist, unsigned long long* counters, int tile_w,
                         int warps_x, bool pdl) {
    auto cut = [&](auto minb) {
        launch_cloud_render_cut<G, decltype(minb)::value>(half, grid, stream, C, M, A, tlut, tw, th, ap_lum,
                                                          ap_trans, blue_noise, depth, out_rgba, out_dist,
                                                          counters, tile_w, warps_x, pdl);
    };
    switch (blocks_per_sm) {
        case 10: cut(std::integral_constant<int, 10>{}); break;
        case 9: cut(std::integral_constant<int, 9>{}); break;
        case 8: cut(std::integral_constant<int, 8>{}); break;
        case 7: cut(std::integral_constant<int, 7>{}); break;
        case 6: cut(std::integral_constant<int, 6>{}); break;
        default: cut(std::integral_constant<int, 5>{}); break;
    }
}

}  // namespace skyr
