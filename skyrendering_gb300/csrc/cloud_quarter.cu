// cloud_quarter.cu — the quarter-resolution cloud pass with temporal
// reconstruction (include/skyr_cloud_quarter.h): checkerboard depth, index,
// the raymarch in checkerboard mode (cloud.cu), reconstruct and upscale.
//
// The reference runs five GL compute programs (VolumetricCloud.cpp:327-423)
// and reads its inputs through textureGather / texelFetch with nearest,
// clamp-to-edge samplers.  Here each gather's footprint is computed in
// integers (a gather at the centre of texel x of an n-texel image reading an
// m-texel texture starts at floor(((2x + 1) m - n) / 2n)), so that the kernels
// and the oracle pick the same texels without texture-coordinate rounding.
// texelFetch outside an image reads 0, as GL's robust access returns.
#include <cmath>
#include <cstring>

#include <cuda_fp16.h>

#include "../../include/skyr_cloud_quarter.h"
#include "cloud_internal.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace {

struct TemporalConsts {
    float ld_n, ld_f;  // 1 / near, 1 / far
    int base;          // uBaseShadingIndex
    int history;       // a previous reconstruction is blended
    int W, H, hw, hh, qw, qh;
    float rp[16];      // uReprojectMat
};

// DepthToLinearDepth (VolumetricCloudCommon.glsl:32-34), 1 / (1/n - (1/n - 1/f) d),
// as 1 / ((1 - d) / n + d / f): the same value without the cancellation of
// the two ~1/n terms at d near 1 (1 - d is exact there)
__device__ __forceinline__ float linear_depth(const TemporalConsts& T, float d) {
    return 1.f / fmaf(T.ld_n, 1.f - d, T.ld_f * d);
}

// IndexToOffset (VolumetricCloudCommon.glsl:41-51): textureGather order
__device__ __forceinline__ int2 index_offset(unsigned i) {
    return make_int2((int)(((i + 1u) >> 1) & 1u), (int)(((i + 2u) >> 1) & 1u));
}

// PosToIndex (VolumetricCloudIndexGen.comp:7-9)
__device__ __forceinline__ unsigned pos_to_index(const TemporalConsts& T, int x, int y) {
    return ((unsigned)T.base + (unsigned)((x + y) & 1)) & 3u;
}

// first texel of a textureGather footprint (x >= 0, m >= n)
__device__ __forceinline__ int gather_base(int x, int n, int m) {
    return (int)(((long long)(2 * x + 1) * m - n) / (2LL * n));
}

__device__ __forceinline__ float4 load_half4(const uint2* p, size_t i) {
    uint2 raw = __ldg(p + i);
    float2 a = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    float2 b = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ void store_half4(uint2* p, size_t i, float4 v) {
    __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, v.w);
    uint2 raw;
    raw.x = *reinterpret_cast<uint32_t*>(&lo);
    raw.y = *reinterpret_cast<uint32_t*>(&hi);
    p[i] = raw;
}

// Reinhard / InverseReinhard on rgb (VolumetricCloudReconstruct.comp:17-26)
__device__ __forceinline__ float4 reinhard(float4 c) {
    return make_float4(c.x / (1.f + c.x), c.y / (1.f + c.y), c.z / (1.f + c.z), c.w);
}
__device__ __forceinline__ float4 inverse_reinhard(float4 c) {
    return make_float4(c.x / (1.f - c.x), c.y / (1.f - c.y), c.z / (1.f - c.z), c.w);
}
__device__ __forceinline__ float4 operator+(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 operator-(float4 a, float4 b) {
    return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 operator*(float4 a, float s) {
    return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}
__device__ __forceinline__ float4 min4(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w));
}
__device__ __forceinline__ float4 max4(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
}

// CheckerboardGen.comp:7-13: the max (x, y of equal parity) or min of the 2x2
// footprint of the window depth; an empty depth buffer is 1.
__global__ void __launch_bounds__(256) checkerboard_kernel(TemporalConsts T, const float* __restrict__ depth,
                                                           float* __restrict__ cb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= T.hw || y >= T.hh) return;
    float d = 1.f;
    if (depth) {
        int x0 = min(gather_base(x, T.hw, T.W), T.W - 1), y0 = min(gather_base(y, T.hh, T.H), T.H - 1);
        int x1 = min(x0 + 1, T.W - 1), y1 = min(y0 + 1, T.H - 1);
        float a = __ldg(depth + (size_t)y1 * T.W + x0), b = __ldg(depth + (size_t)y1 * T.W + x1);
        float c = __ldg(depth + (size_t)y0 * T.W + x1), e = __ldg(depth + (size_t)y0 * T.W + x0);
        d = ((x & 1) == (y & 1)) ? fmaxf(fmaxf(a, b), fmaxf(c, e)) : fminf(fminf(a, b), fminf(c, e));
    }
    cb[(size_t)y * T.hw + x] = d;
}

// VolumetricCloudIndexGen.comp:12-41
__global__ void __launch_bounds__(256) index_kernel(TemporalConsts T, const float* __restrict__ cb,
                                                    float2* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= T.qw || y >= T.qh) return;
    int x0 = min(gather_base(x, T.qw, T.hw), T.hw - 1), y0 = min(gather_base(y, T.qh, T.hh), T.hh - 1);
    int x1 = min(x0 + 1, T.hw - 1), y1 = min(y0 + 1, T.hh - 1);
    float tile[4] = {__ldg(cb + (size_t)y1 * T.hw + x0), __ldg(cb + (size_t)y1 * T.hw + x1),
                     __ldg(cb + (size_t)y0 * T.hw + x1), __ldg(cb + (size_t)y0 * T.hw + x0)};
    unsigned ni = 0, fi = 0;
    float nd = tile[0], fd = tile[0];  // the running nearest / farthest depths (registers, no indexing)
#pragma unroll
    for (unsigned i = 1; i < 4; ++i) {
        if (tile[i] < nd) {
            ni = i;
            nd = tile[i];
        }
        if (tile[i] > fd) {
            fi = i;
            fd = tile[i];
        }
    }
    const float nld = linear_depth(T, nd), fld = linear_depth(T, fd);
    const int ox[8] = {0, 1, 1, 1, 0, -1, -1, -1}, oy[8] = {1, 1, 0, -1, -1, -1, 0, 1};
    unsigned cn = 0, cf = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int tx = x + ox[k], ty = y + oy[k];
        int2 o = index_offset(pos_to_index(T, tx, ty));
        int cx = 2 * tx + o.x, cy = 2 * ty + o.y;
        float d = ((unsigned)cx < (unsigned)T.hw && (unsigned)cy < (unsigned)T.hh)
                      ? __ldg(cb + (size_t)cy * T.hw + cx) : 0.f;
        float ld = linear_depth(T, d);
        float tol = ld * 0.25f;
        cn += fabsf(ld - nld) < tol ? 1u : 0u;
        cf += fabsf(ld - fld) < tol ? 1u : 0u;
    }
    unsigned idx = cn == 0 ? ni : cf == 0 ? fi : pos_to_index(T, x, y);
    float d = idx == 0 ? tile[0] : idx == 1 ? tile[1] : idx == 2 ? tile[2] : tile[3];
    out[(size_t)y * T.qw + x] = make_float2((float)idx, linear_depth(T, d));
}

// VolumetricCloudReconstruct.comp:28-110 (USE_TONEMAPPING 1, USE_VARIANCE 0)
__global__ void __launch_bounds__(256) reconstruct_kernel(CloudConsts C, TemporalConsts T,
                                                          const float* __restrict__ cb,
                                                          const float2* __restrict__ index,
                                                          const uint2* __restrict__ render,
                                                          const float* __restrict__ rdist,
                                                          const uint2* __restrict__ previous, uint2* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= T.hw || y >= T.hh) return;
    const float u = ((float)x + 0.5f) / (float)T.hw, v = ((float)y + 0.5f) / (float)T.hh;
    const float depth = __ldg(cb + (size_t)y * T.hw + x);
    const float ld = linear_depth(T, depth);
    const int qx = x >> 1, qy = y >> 1;
    const int ox[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1}, oy[9] = {0, 1, 1, 0, -1, -1, -1, 0, 1};
    // the 9 rendered linear depths (gathers and texelFetchClamp: clamped)
    float rld[9], dl[9];
    unsigned at[9];
    float mind = 1e10f;
    unsigned nearest = 0;  // the texel index of the depth-nearest neighbour
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        int tx = min(max(qx + ox[i], 0), T.qw - 1), ty = min(max(qy + oy[i], 0), T.qh - 1);
        at[i] = (unsigned)(ty * T.qw + tx);
        rld[i] = __ldg(&index[at[i]].y);
        dl[i] = fabsf(rld[i] - ld);
        if (dl[i] < mind) {
            mind = dl[i];
            nearest = at[i];
        }
    }
    const float4 rn = reinhard(load_half4(render, nearest));
    float4 lo = rn, hi = rn;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        float4 r = reinhard(load_half4(render, at[i]));
        if (dl[i] < rld[i] * 0.3f || fabsf(r.w - rn.w) / fmaxf(1e-6f, 1.f - fmaxf(r.w, rn.w)) < 0.2f) {
            lo = min4(lo, r);
            hi = max4(hi, r);
        }
    }
    // texelFetch at pos >> 1 (unclamped: outside the quarter image it reads 0)
    const bool inside = qx < T.qw && qy < T.qh;
    const size_t q = (size_t)qy * T.qw + qx;
    const float4 rendered = inside ? reinhard(load_half4(render, q)) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rd = inside ? __ldg(rdist + q) : 0.f;
    const unsigned ri = inside ? ((unsigned)(int)__ldg(&index[q].x) & 3u) : 0u;
    // frag_pos = ProjectiveMul(uInvMVP, (uv, depth) * 2 - 1); cloud_pos on the view ray
    const float xn = 2.f * u - 1.f, yn = 2.f * v - 1.f, e = 2.f * (depth - 1.f);
    float3 dir = C.a0 * xn + C.a1 * yn + C.a2 * e + C.af;
    float wv = fmaf(C.w0, xn, fmaf(C.w1, yn, fmaf(C.w2, e, C.wf)));
    float3 view = dir * (copysignf(1.f, wv) * rsqrtf(dot3(dir, dir)));
    float3 cp = C.cam + view * rd;
    const float* m = T.rp;
    float hx = fmaf(m[0], cp.x, fmaf(m[4], cp.y, fmaf(m[8], cp.z, m[12])));
    float hy = fmaf(m[1], cp.x, fmaf(m[5], cp.y, fmaf(m[9], cp.z, m[13])));
    float hw = fmaf(m[3], cp.x, fmaf(m[7], cp.y, fmaf(m[11], cp.z, m[15])));
    float pnx = hx / hw, pny = hy / hw;
    float4 pre = make_float4(0.f, 0.f, 0.f, 0.f);
    if (T.history) {
        // texture(preframe_reconstruct_texture, pre_uv): LINEAR + CLAMP_TO_EDGE (clamp first)
        float px = fminf(fmaxf((pnx * 0.5f + 0.5f) * (float)T.hw - 0.5f, 0.f), (float)(T.hw - 1));
        float py = fminf(fmaxf((pny * 0.5f + 0.5f) * (float)T.hh - 0.5f, 0.f), (float)(T.hh - 1));
        int x0 = (int)px, y0 = (int)py;
        int x1 = min(x0 + 1, T.hw - 1), y1 = min(y0 + 1, T.hh - 1);
        float a = px - (float)x0, b = py - (float)y0;
        float4 t00 = load_half4(previous, (size_t)y0 * T.hw + x0), t10 = load_half4(previous, (size_t)y0 * T.hw + x1);
        float4 t01 = load_half4(previous, (size_t)y1 * T.hw + x0), t11 = load_half4(previous, (size_t)y1 * T.hw + x1);
        float4 top = t00 + (t10 - t00) * a, bot = t01 + (t11 - t01) * a;
        pre = top + (bot - top) * b;
    }
    pre = max4(min4(reinhard(pre), hi), lo);  // clamp(pre, aabb_min, aabb_max)
    const bool out_of_screen = fmaxf(fabsf(pnx), fabsf(pny)) > 1.f;
    const int2 o = index_offset(ri);
    const bool is_rendered = (x & 1) == o.x && (y & 1) == o.y;
    const float w = (!T.history || out_of_screen) ? 1.f : is_rendered ? 0.2f : 0.f;
    const float4 rec = pre * (1.f - w) + rendered * w;  // mix(pre_frame, rendered, weight)
    store_half4(out, (size_t)y * T.hw + x, inverse_reinhard(rec));
}

// VolumetricCloudUpscale.comp:11-55
__global__ void __launch_bounds__(256) upscale_kernel(TemporalConsts T, const float* __restrict__ depth,
                                                      const float* __restrict__ cb, const uint2* __restrict__ rec,
                                                      uint2* __restrict__ hdr) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= T.W || y >= T.H) return;
    const size_t pix = (size_t)y * T.W + x;
    const float ld = linear_depth(T, depth ? __ldg(depth + pix) : 1.f);
    const int ox[4] = {-1, 1, 1, -1}, oy[4] = {1, 1, -1, -1};
    float4 n[4];
    float mind = 1e10f;
    int ni = 0;
    bool edge = false;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int hx = min(max((x + ox[i]) >> 1, 0), T.hw - 1), hy = min(max((y + oy[i]) >> 1, 0), T.hh - 1);
        size_t h = (size_t)hy * T.hw + hx;
        n[i] = load_half4(rec, h);
        float dlt = fabsf(ld - linear_depth(T, __ldg(cb + h)));
        if (dlt < mind) {
            ni = i;
            mind = dlt;
        }
        if (dlt > ld * 0.1f) edge = true;
    }
    float max_a = fmaxf(fmaxf(n[0].w, n[1].w), fmaxf(n[2].w, n[3].w));
    float min_a = fminf(fminf(n[0].w, n[1].w), fminf(n[2].w, n[3].w));
    float4 up;
    if (edge && (max_a - min_a) / fmaxf(1e-6f, 1.f - min_a) > 0.2f) {
        up = ni == 0 ? n[0] : ni == 1 ? n[1] : ni == 2 ? n[2] : n[3];
    } else {
        up = ((n[0] + n[1]) + (n[2] + n[3])) * 0.25f;
    }
    float4 c = load_half4(hdr, pix);
    float t = up.w <= 0.01f ? 0.f : up.w;  // kMinTransmittance
    c.x = c.x * t + up.x;
    c.y = c.y * t + up.y;
    c.z = c.z * t + up.z;
    store_half4(hdr, pix, c);
}

}  // namespace
}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_cloud_temporal_frame_derive(const skyr_atmosphere_parameters* atmosphere, const skyr_cloud_view* view,
                                     const skyr_cloud_view* previous_view, const float* wind_delta, float z_near,
                                     float z_far, int frame_index, skyr_cloud_temporal_frame* out) {
    if (!atmosphere || !view || !out) return set_error(SKYR_EINVAL, "null argument");
    if (!(z_near > 0.f) || !(z_far > z_near) || !std::isfinite(z_far))
        return set_error(SKYR_EINVAL, "camera planes must satisfy 0 < z_near < z_far");
    skyr_cloud_temporal_frame f;
    std::memset(&f, 0, sizeof(f));
    f.z_near = z_near;
    f.z_far = z_far;
    f.base_shading_index = frame_index & 3;
    for (int i = 0; i < 16; ++i) f.reproject[i] = (i % 5) == 0 ? 1.f : 0.f;
    if (previous_view) {
        // uReprojectMat = pre_mvp * delta_mat (VolumetricCloud.cpp:204-234)
        const double R = atmosphere->bottom_radius;
        double model[16], pmodel[16], pvp[16], pmvp[16], ivp[16];
        cloud_local_frame(R, view->camera_position, model);
        cloud_local_frame(R, previous_view->camera_position, pmodel);
        for (int i = 0; i < 16; ++i) pvp[i] = previous_view->view_projection[i];
        if (!invert4d(pvp, ivp)) return set_error(SKYR_EINVAL, "previous view_projection is singular");
        matmul4d(pvp, pmodel, pmvp);
        // delta_local = mat3(inverse(model)) * (camera - previous camera) + wind
        double dw[3], dl[3];
        for (int k = 0; k < 3; ++k) dw[k] = (double)view->camera_position[k] - previous_view->camera_position[k];
        for (int r = 0; r < 3; ++r)  // the model's rotation is orthonormal: its inverse is the transpose
            dl[r] = model[r * 4 + 0] * dw[0] + model[r * 4 + 1] * dw[1] + model[r * 4 + 2] * dw[2];
        if (wind_delta) {
            dl[0] += wind_delta[0];
            dl[1] += wind_delta[1];
        }
        double delta[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, dl[0], dl[1], 0, 1};
        double r[16];
        matmul4d(pmvp, delta, r);
        for (int i = 0; i < 16; ++i) f.reproject[i] = (float)r[i];
        f.has_previous = 1;
    }
    *out = f;
    return SKYR_OK;
}

int skyr_cloud_render_quarter(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                              const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                              const skyr_lut_sizes* sizes, const void* transmittance,
                              const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                              const float* blue_noise, const float* depth, const skyr_cloud_temporal_frame* frame,
                              const skyr_cloud_quarter_buffers* buffers, void* hdr) {
    if (!ctx || !atmosphere || !cloud || !material || !textures || !view || !sizes || !frame || !buffers)
        return set_error(SKYR_EINVAL, "null argument");
    const skyr_cloud_quarter_buffers& B = *buffers;
    if (!B.checkerboard_depth || !B.index_linear_depth || !B.render_rgba || !B.render_distance || !B.reconstruct)
        return set_error(SKYR_EINVAL, "null viewport buffer");
    if (B.previous_reconstruct == B.reconstruct) return set_error(SKYR_EINVAL, "reconstruct buffers must differ");
    if (view->width < 4 || view->height < 4 || view->width > 16384 || view->height > 16384)
        return set_error(SKYR_EINVAL, "viewport must be in [4, 16384]");
    if (!(frame->z_near > 0.f) || !(frame->z_far > frame->z_near))
        return set_error(SKYR_EINVAL, "camera planes must satisfy 0 < z_near < z_far");
    TemporalConsts T;
    std::memset(&T, 0, sizeof(T));
    const double zn = frame->z_near, zf = frame->z_far;
    T.ld_n = (float)(1.0 / zn);
    T.ld_f = (float)(1.0 / zf);
    T.base = frame->base_shading_index & 3;
    T.history = (frame->has_previous && B.previous_reconstruct) ? 1 : 0;
    T.W = view->width;
    T.H = view->height;
    T.hw = T.W / 2;
    T.hh = T.H / 2;
    T.qw = T.hw / 2;
    T.qh = T.hh / 2;
    for (int i = 0; i < 16; ++i) T.rp[i] = frame->reproject[i];
    // the full-resolution constants of the view (unprojection, camera) for the reconstruct pass
    skyr_lut_sizes none;
    std::memset(&none, 0, sizeof(none));
    CloudConsts C;
    MaterialConsts M;
    if (int st = derive_cloud_consts(*atmosphere, *cloud, *material, *textures, *view, none, C, M)) return st;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    cudaStream_t stream = ctx->stream;
    dim3 b2(32, 8);
    auto grid = [&](int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); };
    checkerboard_kernel<<<grid(T.hw, T.hh), b2, 0, stream>>>(T, depth, B.checkerboard_depth);
    if (int e = check_cuda(cudaGetLastError(), "checkerboard kernel")) return e;
    index_kernel<<<grid(T.qw, T.qh), b2, 0, stream>>>(T, B.checkerboard_depth,
                                                      reinterpret_cast<float2*>(B.index_linear_depth));
    if (int e = check_cuda(cudaGetLastError(), "index kernel")) return e;
    CloudCheckerboard cbin{reinterpret_cast<const float2*>(B.index_linear_depth), B.checkerboard_depth, T.hw, T.hh,
                           T.qw, T.qh};
    if (int st = cloud_render_on(ctx, stream, atmosphere, cloud, material, textures, view, sizes, transmittance,
                                 aerial_perspective_luminance, aerial_perspective_transmittance, blue_noise, nullptr,
                                 B.render_rgba, B.render_distance, nullptr, &cbin))
        return st;
    reconstruct_kernel<<<grid(T.hw, T.hh), b2, 0, stream>>>(
        C, T, B.checkerboard_depth, reinterpret_cast<const float2*>(B.index_linear_depth),
        reinterpret_cast<const uint2*>(B.render_rgba), B.render_distance,
        reinterpret_cast<const uint2*>(B.previous_reconstruct), reinterpret_cast<uint2*>(B.reconstruct));
    if (int e = check_cuda(cudaGetLastError(), "reconstruct kernel")) return e;
    if (!hdr) return SKYR_OK;
    upscale_kernel<<<grid(T.W, T.H), b2, 0, stream>>>(T, depth, B.checkerboard_depth,
                                                      reinterpret_cast<const uint2*>(B.reconstruct),
                                                      reinterpret_cast<uint2*>(hdr));
    return check_cuda(cudaGetLastError(), "upscale kernel");
}

}  // extern "C"
