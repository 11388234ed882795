// cloud_fast.cuh — the density evaluation of the cloud raymarch specialised for
// the configuration the reference ships in bin/config.json and the frame
// workload uses: Material1 (VolumetricCloudDefaultMaterial1.glsl:14-29) with
// NEAREST_MIPMAP_NEAREST minification on both textures, REPEAT wrapping and the
// expanded level-0 layouts of skyr_noise_expand.  It computes what
// sample_sigma_t computes for that configuration with fewer instructions:
//   * the GL level of detail lambda = log2(k_lod |p - cam|) + lod_bias is
//     needed only to tell magnification (lambda <= 1/2: LINEAR at level 0)
//     from minification, which is |p - cam|^2 <= mag_d2, a constant per
//     texture; the logarithm is taken (of |p - cam|^2) only for minified
//     samples, whose NEAREST_MIPMAP_NEAREST level is ceil(lambda + 1/2) - 1
//     (GL 4.6 section 8.14.3);
//   * filters return the UNORM8 value in 0..255 units and the 1/255 is folded
//     into the material's constants, each clamp01(a x + b) being one fused
//     multiply-add with saturation;
//   * a level's byte offset is one constant load (kernel parameters are
//     __grid_constant__), not a loop over the levels above it;
//   * where the caller gives hardware samplers (skyr_noise_sampler), the
//     magnified LINEAR fetch is one texture instruction -- the texture unit
//     filters UNORM8 texels with 8-bit fixed-point weights, as GL does for the
//     reference's textures, and the filter arithmetic leaves the SM's pipes --
//     and the minified NEAREST fetch is one texture instruction at the level
//     computed here (the texel addressing and the REPEAT wrap leave the SM).
// The host picks this path (MaterialConsts::fast_ok) only when every
// condition holds, square / cubic textures included; anything else runs the
// general sample_sigma_t.
#pragma once

#include "cloud_internal.cuh"

namespace skyr {

__device__ __forceinline__ float sat(float x) { return __saturatef(x); }

// UNORM8 byte k of a packed word in 0..255 (exact): PRMT builds 2^23 + b, one FADD removes 2^23.
__device__ __forceinline__ float byte255(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (unsigned)k)) - 8388608.f;
}

// GL LINEAR at level 0 with REPEAT, from the expanded layout: one 4-byte load.
__device__ __forceinline__ float fast_bilinear(const FastTex& T, float u, float v) {
    float x = fmaf(u, T.fw, -0.5f), y = fmaf(v, T.fh, -0.5f);
    float fx = floorf(x), fy = floorf(y);
    float a = x - fx, b = y - fy;
    unsigned ix = (unsigned)(int)fx & (unsigned)(T.w - 1), iy = (unsigned)(int)fy & (unsigned)(T.h - 1);
    uint32_t q = __ldg(reinterpret_cast<const uint32_t*>(T.ex) + (iy * (unsigned)T.w + ix));
    float t00 = byte255(q, 0), t10 = byte255(q, 1), t01 = byte255(q, 2), t11 = byte255(q, 3);
    float top = fmaf(a, t10 - t00, t00), bot = fmaf(a, t11 - t01, t01);
    return fmaf(b, bot - top, top);
}

// GL LINEAR at level 0 with REPEAT in 3D, from the expanded layout: one 8-byte load.
__device__ __forceinline__ float fast_trilinear(const FastTex& T, float u, float v, float s) {
    float x = fmaf(u, T.fw, -0.5f), y = fmaf(v, T.fh, -0.5f), z = fmaf(s, T.fd, -0.5f);
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float a = x - fx, b = y - fy, g = z - fz;
    unsigned ix = (unsigned)(int)fx & (unsigned)(T.w - 1), iy = (unsigned)(int)fy & (unsigned)(T.h - 1),
             iz = (unsigned)(int)fz & (unsigned)(T.d - 1);
    unsigned long long q = __ldg(reinterpret_cast<const unsigned long long*>(T.ex) +
                                 ((iz * (unsigned)T.h + iy) * (unsigned)T.w + ix));
    uint32_t lo = (uint32_t)q, hi = (uint32_t)(q >> 32);
    float t000 = byte255(lo, 0), t100 = byte255(lo, 1), t010 = byte255(lo, 2), t110 = byte255(lo, 3);
    float t001 = byte255(hi, 0), t101 = byte255(hi, 1), t011 = byte255(hi, 2), t111 = byte255(hi, 3);
    float top0 = fmaf(a, t100 - t000, t000), bot0 = fmaf(a, t110 - t010, t010);
    float top1 = fmaf(a, t101 - t001, t001), bot1 = fmaf(a, t111 - t011, t011);
    float r0 = fmaf(b, bot0 - top0, top0), r1 = fmaf(b, bot1 - top1, top1);
    return fmaf(g, r1 - r0, r0);
}

// NEAREST at the NEAREST_MIPMAP_NEAREST level of a minified sample (lambda > 1/2), REPEAT.
// The texture is square (2D) or cubic (3D), so every dimension of level l is
// size >> l >= 1.
template <bool D3>
__device__ __forceinline__ float fast_nearest(const FastTex& T, float u, float v, float s, float d2) {
    float lambda = fminf(fmaf(0.5f, __log2f(d2), T.lod_k), 1000.f);
    int l = min((int)ceilf(lambda + 0.5f) - 1, T.last);
    if (T.tex_near) {  // the texture unit's NEAREST at level l (REPEAT), the byte itself
        const cudaTextureObject_t o = (cudaTextureObject_t)T.tex_near;
        const unsigned b = D3 ? (unsigned)tex3DLod<unsigned char>(o, u, v, s, (float)l)
                              : (unsigned)tex2DLod<unsigned char>(o, u, v, (float)l);
        return __uint_as_float(0x4B000000u | b) - 8388608.f;
    }
    unsigned wl = (unsigned)T.w >> l, mask = wl - 1;
    float scale = T.fw * __int_as_float((127 - l) << 23);  // (size >> l) as a float: size * 2^-l
    unsigned x = (unsigned)(int)floorf(u * scale) & mask, y = (unsigned)(int)floorf(v * scale) & mask;
    unsigned i = y * wl + x;
    if constexpr (D3) i += ((unsigned)(int)floorf(s * scale) & mask) * (wl * wl);
    return __uint_as_float(0x4B000000u | (unsigned)__ldg(T.base + T.off[l] + i)) - 8388608.f;
}

// CalHeight01 (VolumetricCloudCommon.glsl:36-39) of a point with
// rho2 = |p + R z^|^2 - R^2, by the series of FastConsts (no square root, no
// division).  Products of several uses are rounded explicitly (see
// sample_shadow).
__device__ __forceinline__ float fast_height01(const FastConsts& F, float rho2) {
    float x = __fmul_rn(rho2, F.h_ir2);
    float poly = fmaf(x, fmaf(x, 0.125f, -0.25f), 1.f);
    return sat(fmaf(__fmul_rn(rho2, poly), F.h_k1, F.h_k0));
}

// Material1's SampleSigmaT at p with height fraction h and squared camera
// distance d2 (VolumetricCloudDefaultMaterial1.glsl:14-29).  n_detail
// (COUNT): evaluations past the coverage test.
template <bool COUNT = false>
__device__ __forceinline__ float fast_sigma_m1(const MaterialConsts& M, float3 p, float h, float d2,
                                               unsigned* n_detail = nullptr) {
    const FastConsts& F = M.fast;
    float u = fmaf(p.x, M.cloud_map.frequency, M.cloud_map.bias_x);
    float v = fmaf(p.y, M.cloud_map.frequency, M.cloud_map.bias_y);
    float cr;
    if (d2 <= F.cm.mag_d2)
        cr = F.cm.tex ? 255.f * tex2D<float>((cudaTextureObject_t)F.cm.tex, u, v) : fast_bilinear(F.cm, u, v);
    else
        cr = fast_nearest<false>(F.cm, u, v, 0.f, d2);
    float density = sat(fmaf(cr, F.cov_a, F.cov_b)) * sat(fmaf(h, F.hh_a, F.hh_b));
    if (density == 0.f) return 0.f;
    if constexpr (COUNT) ++*n_detail;
    float du = fmaf(p.x, M.detail.frequency, M.detail.bias_x);
    float dv = fmaf(p.y, M.detail.frequency, M.detail.bias_y);
    float dw = p.z * M.detail.frequency;
    float dt;
    if (d2 <= F.dt.mag_d2)
        dt = F.dt.tex ? 255.f * tex3D<float>((cudaTextureObject_t)F.dt.tex, du, dv, dw)
                      : fast_trilinear(F.dt, du, dv, dw);
    else
        dt = fast_nearest<true>(F.dt, du, dv, dw, d2);
    float erode = fmaxf(sat(h - F.height_cut), sat(fmaf(cr, F.ec_a, F.ec_b)));
    return sat(fmaf(-fmaf(dt, F.det_a, F.det_b), erode, density)) * F.density * h;
}

}  // namespace skyr
