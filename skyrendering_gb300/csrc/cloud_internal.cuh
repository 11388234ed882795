// cloud_internal.cuh — kernel constants and GL-exact texture sampling of the
// cloud raymarch (shared by the cloud and path-tracer kernels).
#pragma once

#include "../../include/skyr_cloud.h"
#include "skyr_internal.cuh"

namespace skyr {

constexpr int kMaxLevels = 16;

// Device view of a UNORM8 texture in the layout of skyr_cloud.h.
struct DTex {
    const uint8_t* base;
    const void* ex;  // expanded level 0 (skyr_noise_expand), or null
    int w, h, d;     // level-0 size (powers of two)
    int levels;
    int border;      // 1: CLAMP_TO_BORDER (0), 0: REPEAT
    int channels;
    int ex_channels;  // channels present in `ex`
};

// UNORM8 byte k of a packed word as an exact float 0..255: PRMT builds
// 0x4B0000bb = 2^23 + b, one FADD removes 2^23.
__device__ __forceinline__ float byte_f(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (unsigned)k)) - 8388608.f;
}

// Byte offset of mip level l (levels are stored consecutively).  A short loop
// instead of a table: a kernel-parameter array indexed at run time would be
// copied to local memory.
__device__ __forceinline__ size_t dtex_level_offset(const DTex& t, int l) {
    size_t off = 0;
#pragma unroll 1
    for (int k = 0; k < l; ++k) off += (size_t)max(t.w >> k, 1) * max(t.h >> k, 1) * max(t.d >> k, 1);
    return off * t.channels;
}

__device__ __forceinline__ float dtex_texel(const DTex& t, int l, int c, int x, int y, int z) {
    int W = max(t.w >> l, 1), H = max(t.h >> l, 1), D = max(t.d >> l, 1);
    if (t.border) {
        if ((unsigned)x >= (unsigned)W || (unsigned)y >= (unsigned)H || (unsigned)z >= (unsigned)D) return 0.f;
    } else {
        x &= W - 1;
        y &= H - 1;
        z &= D - 1;
    }
    // the index within one channel of one level stays below 2^31 (noise texture
    // sizes are capped at 2^31 texels), so only the level and channel offsets need 64 bits
    unsigned i = ((unsigned)z * (unsigned)H + (unsigned)y) * (unsigned)W + (unsigned)x;
    size_t off = (l ? dtex_level_offset(t, l) : 0) + (size_t)c * W * H * D;
    return (float)__ldg(t.base + off + i) * (1.f / 255.f);
}

__device__ __forceinline__ float dtex_nearest(const DTex& t, int l, int c, float u, float v, float s) {
    int W = max(t.w >> l, 1), H = max(t.h >> l, 1), D = max(t.d >> l, 1);
    return dtex_texel(t, l, c, (int)floorf(u * (float)W), (int)floorf(v * (float)H),
                      t.d > 1 ? (int)floorf(s * (float)D) : 0);
}

__device__ __forceinline__ float dtex_linear(const DTex& t, int l, int c, float u, float v, float s) {
    int W = max(t.w >> l, 1), H = max(t.h >> l, 1), D = max(t.d >> l, 1);
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float a = x - fx, b = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    if (l == 0 && t.ex != nullptr && c < t.ex_channels && !t.border) {
        // expanded level 0: one word holds every corner of the footprint
        // indices within one channel stay below 2^31 (see dtex_texel)
        size_t n = (size_t)W * H * D;
        unsigned ix = (unsigned)(x0 & (W - 1)), iy = (unsigned)(y0 & (H - 1));
        if (t.d <= 1) {
            uint32_t q = __ldg(reinterpret_cast<const uint32_t*>(t.ex) + (size_t)c * n + (iy * (unsigned)W + ix));
            float t00 = byte_f(q, 0), t10 = byte_f(q, 1), t01 = byte_f(q, 2), t11 = byte_f(q, 3);
            float top = fmaf(a, t10 - t00, t00), bot = fmaf(a, t11 - t01, t01);
            return fmaf(b, bot - top, top) * (1.f / 255.f);
        }
        float z = s * (float)D - 0.5f;
        float fz = floorf(z);
        float g = z - fz;
        unsigned iz = (unsigned)((int)fz & (D - 1));
        unsigned long long q = __ldg(reinterpret_cast<const unsigned long long*>(t.ex) + (size_t)c * n +
                                     ((iz * (unsigned)H + iy) * (unsigned)W + ix));
        uint32_t lo = (uint32_t)q, hi = (uint32_t)(q >> 32);
        float t000 = byte_f(lo, 0), t100 = byte_f(lo, 1), t010 = byte_f(lo, 2), t110 = byte_f(lo, 3);
        float t001 = byte_f(hi, 0), t101 = byte_f(hi, 1), t011 = byte_f(hi, 2), t111 = byte_f(hi, 3);
        float top0 = fmaf(a, t100 - t000, t000), bot0 = fmaf(a, t110 - t010, t010);
        float top1 = fmaf(a, t101 - t001, t001), bot1 = fmaf(a, t111 - t011, t011);
        float r0 = fmaf(b, bot0 - top0, top0), r1 = fmaf(b, bot1 - top1, top1);
        return fmaf(g, r1 - r0, r0) * (1.f / 255.f);
    }
    if (t.d <= 1) {
        float t00 = dtex_texel(t, l, c, x0, y0, 0), t10 = dtex_texel(t, l, c, x0 + 1, y0, 0);
        float t01 = dtex_texel(t, l, c, x0, y0 + 1, 0), t11 = dtex_texel(t, l, c, x0 + 1, y0 + 1, 0);
        float top = fmaf(a, t10 - t00, t00), bot = fmaf(a, t11 - t01, t01);
        return fmaf(b, bot - top, top);
    }
    float z = s * (float)D - 0.5f;
    float fz = floorf(z);
    float g = z - fz;
    int z0 = (int)fz;
    float r[2];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz) {
        float t00 = dtex_texel(t, l, c, x0, y0, z0 + dz), t10 = dtex_texel(t, l, c, x0 + 1, y0, z0 + dz);
        float t01 = dtex_texel(t, l, c, x0, y0 + 1, z0 + dz), t11 = dtex_texel(t, l, c, x0 + 1, y0 + 1, z0 + dz);
        float top = fmaf(a, t10 - t00, t00), bot = fmaf(a, t11 - t01, t01);
        r[dz] = fmaf(b, bot - top, top);
    }
    return fmaf(g, r[1] - r[0], r[0]);
}

// textureLod with LINEAR magnification and minification `minf` (GL 4.6
// sections 8.14-8.15): magnified when lambda <= c (c = 0.5 for the
// NEAREST_MIPMAP_* filters, else 0).
__device__ __forceinline__ float dtex_sample(const DTex& t, int c, float u, float v, float s, float lod, int minf) {
    float lambda = fminf(fmaxf(lod, -1000.f), 1000.f);
    bool nearest_mip_filter = minf == SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST || minf == SKYR_MIPMAP_NEAREST_MIPMAP_LINEAR;
    float cs = nearest_mip_filter ? 0.5f : 0.f;
    if (!(lambda > cs)) return dtex_linear(t, 0, c, u, v, s);
    int q = t.levels - 1;
    bool lin = minf == SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST || minf == SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR;
    if (minf == SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST || minf == SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST) {
        int dl = lambda <= 0.5f ? 0 : (int)ceilf(lambda + 0.5f) - 1;
        dl = min(dl, q);
        return lin ? dtex_linear(t, dl, c, u, v, s) : dtex_nearest(t, dl, c, u, v, s);
    }
    if (lambda >= (float)q) return lin ? dtex_linear(t, q, c, u, v, s) : dtex_nearest(t, q, c, u, v, s);
    int d1 = (int)floorf(lambda);
    float f = lambda - (float)d1;
    int d2 = min(d1 + 1, q);
    float a = lin ? dtex_linear(t, d1, c, u, v, s) : dtex_nearest(t, d1, c, u, v, s);
    float b = lin ? dtex_linear(t, d2, c, u, v, s) : dtex_nearest(t, d2, c, u, v, s);
    return (1.f - f) * a + f * b;
}

struct SampleInfoD {
    float bias_x, bias_y, frequency, k_lod;
};

// Constants of the specialised density evaluation (cloud_fast.cuh): Material1
// with NEAREST_MIPMAP_NEAREST minification, REPEAT and expanded level 0.
struct FastTex {
    const uint8_t* base;  // channel 0 of level l at base + off[l]
    const void* ex;       // expanded level 0 of channel 0 (uint32 per 2D texel, uint64 per 3D texel)
    unsigned long long tex;       // hardware sampler of level 0, channel 0, LINEAR (cudaTextureObject_t), or 0
    unsigned long long tex_near;  // hardware sampler of every level, channel 0, NEAREST per level, or 0
    int w, h, d;          // level-0 size (powers of two; d = 1 for a 2D texture)
    int last;             // index of the last mip level
    float fw, fh, fd;     // level-0 size as floats
    float mag_d2;         // GL magnifies (lambda <= 1/2) while |p - cam|^2 <= mag_d2
    float lod_k;          // lambda = 0.5 log2 |p - cam|^2 + lod_k  (lod_k = log2 k_lod + lod_bias)
    unsigned off[kMaxLevels];
};

struct FastConsts {
    FastTex cm, dt;          // cloud map (2D, channel R), detail texture (3D, channel R)
    float cov_a, cov_b;      // clamp01((cr - threshold) * edge_hardness) = sat(cr255 cov_a + cov_b)
    float hh_a, hh_b;        // clamp01((1 - h) * height_hardness)         = sat(h hh_a + hh_b)
    float det_a, det_b;      // (detail + detail_base) * detail_scale      = dt255 det_a + det_b
    float height_cut;        // clamp01(h - height_cut)
    float ec_a, ec_b;        // clamp01(edge_cut - cr)                     = sat(cr255 ec_a + ec_b)
    float density;           // uDensity
    // CalHeight01 from rho2 = |p + R z|^2 - R^2 by its series in x = rho2 / R^2:
    // altitude = rho2 / (2R) (1 - x/4 + x^2/8 - 5x^3/64 ...); the host admits the
    // path only while |x| <= 0.02 for every sample (the cubic term < 2e-7)
    float h_ir2;             // 1 / R^2
    float h_k1, h_k0;        // height01 = sat(altitude h_k1 + h_k0): inv_layer, -bottom inv_layer, with 1/(2R)
};

// Material constants (the material's Update + VolumetricCloudDefaultMaterialCommon)
struct MaterialConsts {
    int type;
    int min2d, min3d, mindisp;
    SampleInfoD cloud_map, detail, displacement;
    float lod_bias, density;
    float m1_threshold, m1_height_hardness, m1_edge_hardness, m1_detail_base, m1_detail_scale, m1_height_cut,
        m1_edge_cut;
    float m0_detail_x, m0_detail_y, m0_disp_scale;
    float vx_freq_x, vx_freq_y, vx_bias_x, vx_bias_y, vx_k_lod;
    DTex cloud_map_tex, detail_tex, displacement_tex, voxel_tex;
    int fast_ok;      // the configuration cloud_fast.cuh specialises (set by derive_cloud_consts)
    FastConsts fast;  // its constants, when fast_ok
};

// Frame constants (VolumetricCloud::Update, VolumetricCloud.cpp:168-280)
struct CloudConsts {
    // pixel ray: (frag - cam) = (a0 x + a1 y + a2 e + af) / (w0 x + w1 y + w2 e + wf) with NDC x, y
    // and e = z_ndc - 1 = 2 (depth - 1); af = a2 + a3 and wf = w2 + w3 are summed in double,
    // so that far-plane points (depth near 1) do not cancel in FP32
    float3 a0, a1, a2, af;
    float w0, w1, w2, wf;
    float3 a3;  // NDC z = 0 rays: (frag - cam) = (a0 x + a1 y + a3) / (w0 x + w1 y + w3)
    float w3;
    float3 cam;  // local z-up
    float3 sun;  // local
    float R, bottom, top;       // Earth radius, cloud layer altitudes
    float rb, rt;               // R + bottom, R + top
    float inv_layer;            // 1 / (top - bottom)
    float rho2_bottom, rho2_top, cam_rho2;  // R_x^2 - R^2 of the layer spheres and the camera (exact)
    float jitter_offset;        // frame_id * 0.61803398875
    float sun_illuminance_scale, max_raymarch_distance, max_raymarch_steps, max_visible_distance;
    float3 env_color_scale;
    float shadow_steps;
    float sun_ms_sigma_scale, env_ms_sigma_scale, shadow_distance, env_bottom_visibility, env_sun_height_curve_exp;
    float g_fwd, g_back, back_scale;
    float ap_max_distance, inv_ap_max_distance;
    float atmo_in_space;  // camera beyond the atmosphere top
    int width, height;
    int ap_w, ap_h, ap_d;
    const uint16_t* froxel;  // shadow froxel, or null for a visibility of 1
    int fx_w, fx_h, fx_d;
    float inv_froxel_max_distance;
    // checkerboard mode (the quarter-resolution pass): pixel (x, y) of the
    // width x height raymarch is checkerboard texel 2 (x, y) + IndexToOffset(index)
    // of the cb_w x cb_h checkerboard depth; null: a full-resolution raymarch
    const float2* cb_index;
    const float* cb_depth;
    int cb_w, cb_h;
    // the order in which the raymarch's block rows start (march_row): outward
    // from block row row_pivot, the side of row_dir (+1 or -1) first
    int row_pivot, row_dir;
};

// The block row that the k-th of n block rows marches: p, then alternately
// p + d, p - d, p + 2d, p - 2d, ... while both sides last, then the rest of
// the longer side outward.  A bijection of [0, n) for p in [0, n) and d = +-1.
__device__ __forceinline__ int march_row(int k, int n, int p, int d) {
    p = min(max(p, 0), n - 1);
    d = d < 0 ? -1 : 1;
    const int first = d > 0 ? n - 1 - p : p, second = d > 0 ? p : n - 1 - p, m = min(first, second);
    int off;
    if (k <= 2 * m) off = (k & 1) ? (k + 1) >> 1 : -(k >> 1);
    else off = first > second ? k - m : -(k - m);
    return p + d * off;
}

// The checkerboard input of a quarter-resolution raymarch.
struct CloudCheckerboard {
    const float2* index;  // quarter: (index, linear depth)
    const float* depth;   // half: checkerboard depth
    int half_w, half_h, quarter_w, quarter_h;
};

// SampleRayScatterVisibility (VolumetricCloudShadowInterface.glsl:10-13): the
// unorm16 shadow froxel (w x h x d) read with GL LINEAR + CLAMP_TO_EDGE at
// (u, v, dist / max) and faded to 1 by clamp(1 / w, 0, 1) beyond its last
// slice; 1 without a froxel.
__device__ __forceinline__ float froxel_visibility_at(const uint16_t* froxel, int fw, int fh, int fd,
                                                      float inv_max_distance, float u, float v, float dist) {
    if (!froxel) return 1.f;
    float w = dist * inv_max_distance;
    // clamping the texel coordinate first is CLAMP_TO_EDGE's rule for LINEAR
    float x = fminf(fmaxf(u * (float)fw - 0.5f, 0.f), (float)(fw - 1));
    float y = fminf(fmaxf(v * (float)fh - 0.5f, 0.f), (float)(fh - 1));
    float z = fminf(fmaxf(w * (float)fd - 0.5f, 0.f), (float)(fd - 1));
    int x0 = (int)x, y0 = (int)y, z0 = (int)z;
    int x1 = min(x0 + 1, fw - 1), y1 = min(y0 + 1, fh - 1), z1 = min(z0 + 1, fd - 1);
    float a = x - (float)x0, b = y - (float)y0, g = z - (float)z0;
    const size_t slice = (size_t)fw * fh;
    float r[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint16_t* s = froxel + (size_t)(k ? z1 : z0) * slice;
        float t00 = (float)__ldg(s + (size_t)y0 * fw + x0), t10 = (float)__ldg(s + (size_t)y0 * fw + x1);
        float t01 = (float)__ldg(s + (size_t)y1 * fw + x0), t11 = (float)__ldg(s + (size_t)y1 * fw + x1);
        float top = t00 + (t10 - t00) * a, bot = t01 + (t11 - t01) * a;
        r[k] = top + (bot - top) * b;
    }
    float f = (r[0] + (r[1] - r[0]) * g) * (1.f / 65535.f);
    float k = fminf(fmaxf(__frcp_rn(w), 0.f), 1.f);  // w = 0 gives +inf, clamped to 1
    return 1.f + (f - 1.f) * k;
}

__device__ __forceinline__ float froxel_visibility(const CloudConsts& C, float u, float v, float dist) {
    return froxel_visibility_at(C.froxel, C.fx_w, C.fx_h, C.fx_d, C.inv_froxel_max_distance, u, v, dist);
}

// Column-major 4x4 helpers of the host derivations (double).
bool invert4d(const double* m, double* out);
void matmul4d(const double* a, const double* b, double* c);
// The local z-up cloud frame of a camera (column-major model matrix).
void cloud_local_frame(double R, const float cam_world[3], double model[16]);

int derive_cloud_consts(const skyr_atmosphere_parameters& atmo, const skyr_cloud_parameters& cp,
                        const skyr_cloud_material& m, const skyr_cloud_textures& tex, const skyr_cloud_view& v,
                        const skyr_lut_sizes& sizes, CloudConsts& c, MaterialConsts& mc);

int noise_levels(const skyr_noise_texture_desc* d);
size_t noise_level_offset(const skyr_noise_texture_desc* d, int level);
int validate_noise_desc(const skyr_noise_texture_desc* d, bool generator);

}  // namespace skyr
