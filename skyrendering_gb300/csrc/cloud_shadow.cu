// cloud_shadow.cu — the volumetric cloud's shadow passes (include/skyr_cloud_shadow.h):
// the light transform of a frame (host), the light-space shadow map, its
// separable blur and the shadow froxel (device).
//
// The reference runs them as three GL compute programs with a texture-fetch
// barrier between each (src/SkyRendering/VolumetricCloud.cpp:282-325):
//   VolumetricCloudShadowMap.comp:37-75    one invocation per texel of a 512^2 RG32F map
//   VolumetricCloudShadowMapBlur.comp:9-42 two dispatches (x, then y) through a temporary
//   VolumetricCloudShadowFroxel.comp:10-27 one invocation per froxel column, 128 slices
// Here the two blur directions are one kernel (a tile and its 4-texel apron
// in shared memory, the x pass kept on chip), and the froxel's running mean
// is split over 16-slice chunks of a column joined by a block-level scan.
#include <cmath>
#include <cstring>

#include "../../include/skyr_cloud_shadow.h"
#include "cloud_internal.cuh"
#include "cloud_material.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace {

// ---------------------------------------------------------------------------
// Host: the light transform (VolumetricCloud::Update, VolumetricCloud.cpp:188-235)
// ---------------------------------------------------------------------------
struct V3d {
    double x, y, z;
};
V3d operator-(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3d operator+(V3d a, V3d b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3d operator*(V3d a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dot(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3d cross(V3d a, V3d b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3d normalized(V3d a) { return a * (1.0 / std::sqrt(dot(a, a))); }

// column-major M * (p, w)
void transform(const double* m, const double p[4], double out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = m[r] * p[0] + m[4 + r] * p[1] + m[8 + r] * p[2] + m[12 + r] * p[3];
}

void identity4(double* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5) == 0 ? 1.0 : 0.0;
}

int validate_shadow_sizes(const skyr_cloud_shadow_sizes* s, bool froxel) {
    if (!s) return set_error(SKYR_EINVAL, "null shadow sizes");
    if (s->map_width < 1 || s->map_height < 1 || s->map_width > 16384 || s->map_height > 16384)
        return set_error(SKYR_EINVAL, "shadow map size must be in [1, 16384]");
    if (froxel && (s->froxel_width < 1 || s->froxel_height < 1 || s->froxel_width > 16384 ||
                   s->froxel_height > 16384 || s->froxel_depth < 1 || s->froxel_depth > 512))
        return set_error(SKYR_EINVAL, "shadow froxel size out of range (depth 1..512)");
    return SKYR_OK;
}

// ---------------------------------------------------------------------------
// Device
// ---------------------------------------------------------------------------
constexpr float kBorderDepth = 1e10f;  // shadow_map_sampler_ border (VolumetricCloud.cpp:111)
constexpr int kBlurTile = 32;          // output texels per blur block side
constexpr int kBlurApron = 4;          // KERNEL_HALF_WIDTH - 1
constexpr int kFroxelChunk = 16;       // slices per thread of the froxel kernel

// Launch constants of the shadow-map pass.
struct ShadowMapConsts {
    // texel origin on the light's z = 0 plane: (o0 x + o1 y + o3) / (q0 x + q1 y + q3), NDC x, y
    float3 o0, o1, o3;
    float q0, q1, q3;
    float3 dir;            // -sun, local
    float rho2_bottom, rho2_top;  // |p|^2 - R^2 of the layer spheres (exact)
    float max_dist;        // (top - bottom) / cos(85 deg)
    float steps;           // mix(12, 6, |dir.z|)
    int width, height;
    int reproject;         // blend with the previous map
    float rp[16];          // uShadowMapReprojectMat, column-major
};

// Launch constants of the froxel pass.
struct FroxelConsts {
    float lvp[16];    // uLightVP
    int width, height, depth;
    int map_w, map_h;
    float step;       // shadow_froxel_max_distance / depth
};

// GL LINEAR fetch of a float2 texture at (u, v) with CLAMP_TO_BORDER border
// (1e10, 1) (the shadow map sampler, VolumetricCloud.cpp:106-112).
__device__ __forceinline__ float2 map_bilinear_border(const float2* map, int w, int h, float u, float v) {
    float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float a = x - fx, b = y - fy;
    int x0 = (int)fmaxf(fminf(fx, 1e8f), -1e8f), y0 = (int)fmaxf(fminf(fy, 1e8f), -1e8f);
    float2 t[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int xi = x0 + (k & 1), yi = y0 + (k >> 1);
        t[k] = ((unsigned)xi < (unsigned)w && (unsigned)yi < (unsigned)h) ? __ldg(map + (size_t)yi * w + xi)
                                                                          : make_float2(kBorderDepth, 1.f);
    }
    float2 r;
    float top = t[0].x + (t[1].x - t[0].x) * a, bot = t[2].x + (t[3].x - t[2].x) * a;
    r.x = top + (bot - top) * b;
    top = t[0].y + (t[1].y - t[0].y) * a;
    bot = t[2].y + (t[3].y - t[2].y) * a;
    r.y = top + (bot - top) * b;
    return r;
}

// The shadow map (VolumetricCloudShadowMap.comp:37-75), one thread per texel.
// LineShellFirstIntersect in the stable form: with p the origin seen from the
// Earth's centre, b = p.dir and c_x = r_x^2 - |p|^2 (= rho2_x - rho2_o, no
// cancellation), the sphere roots are -b -/+ sqrt(b^2 + c_x); the near root is
// -c_x / (sqrt(.) - b) for b < 0 and the far one c_x / (b + sqrt(.)) for b >= 0.
__global__ void __launch_bounds__(128) shadow_map_kernel(CloudConsts C, MaterialConsts M, ShadowMapConsts S,
                                                         const float* __restrict__ blue_noise,
                                                         const float2* __restrict__ previous, float2* raw) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= S.width || py >= S.height) return;
    const float nx = ((float)px + 0.5f) / (float)S.width * 2.f - 1.f;
    const float ny = ((float)py + 0.5f) / (float)S.height * 2.f - 1.f;
    const float inv_q = 1.f / fmaf(S.q0, nx, fmaf(S.q1, ny, S.q3));
    const float3 o = (S.o0 * nx + S.o1 * ny + S.o3) * inv_q;
    const float3 d = S.dir;
    const float b = fmaf(o.x, d.x, fmaf(o.y, d.y, o.z * d.z)) + C.R * d.z;
    const float rho2_o = fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * (o.z + 2.f * C.R)));
    const float ct = S.rho2_top - rho2_o, cb = S.rho2_bottom - rho2_o;
    const float bb = b * b;
    float t1 = 0.f, t2 = 0.f;
    const float disc_t = bb + ct;
    if (disc_t > 0.f) {
        float st = sqrtf(disc_t);
        t1 = b < 0.f ? -ct / (st - b) : -b - st;
        float disc_b = bb + cb;
        if (disc_b >= 0.f) {
            float sb = sqrtf(disc_b);
            t2 = b < 0.f ? -cb / (sb - b) : -b - sb;
        } else {
            t2 = b < 0.f ? st - b : ct / (b + st);
        }
    }
    float dist = fminf(fmaxf(t2 - t1, 0.f), S.max_dist);
    float od = 0.f;
    if (dist > 0.f) {
        const float step = dist / S.steps;
        float j = __ldg(blue_noise + (py & 63) * 64 + (px & 63)) + C.jitter_offset;
        float t = t1 + step * (j - floorf(j));
        const unsigned n = (unsigned)S.steps;  // uint(steps) <= 12
#pragma unroll 1
        for (unsigned k = 0; k < n; ++k, t += step) {
            float3 p = o + d * t;
            float h = height01(C, p);
            float3 dc = p - C.cam;
            od = fmaf(sigma_t(C, M, p, h, sqrtf(dot3(dc, dc))), step, od);
        }
    }
    float2 res = make_float2(0.5f * t1 + 0.5f * t2, expf(-od));
    if (S.reproject) {
        // ProjectiveMul(uShadowMapReprojectMat, (ndc, 0)).xy * 0.5 + 0.5
        const float* m = S.rp;
        float hw = fmaf(m[3], nx, fmaf(m[7], ny, m[15]));
        float pu = fmaf(m[0], nx, fmaf(m[4], ny, m[12])) / hw * 0.5f + 0.5f;
        float pv = fmaf(m[1], nx, fmaf(m[5], ny, m[13])) / hw * 0.5f + 0.5f;
        float lo_u = 0.5f / (float)S.width, hi_u = ((float)S.width - 0.5f) / (float)S.width;
        float lo_v = 0.5f / (float)S.height, hi_v = ((float)S.height - 0.5f) / (float)S.height;
        if (pu >= lo_u && pu <= hi_u && pv >= lo_v && pv <= hi_v) {
            float2 pre = map_bilinear_border(previous, S.width, S.height, pu, pv);
            res.x = pre.x * 0.8f + res.x * 0.2f;  // mix(pre, res, 0.2)
            res.y = pre.y * 0.8f + res.y * 0.2f;
        }
    }
    raw[(size_t)py * S.width + px] = res;
}

// 9-tap Gaussian half-kernel (VolumetricCloudShadowMapBlur.comp:10)
__constant__ float kBlurWeight[5] = {0.227027f, 0.1945946f, 0.1216216f, 0.054054f, 0.016216f};

// Both blur passes (VolumetricCloudShadowMapBlur.comp:14-42) for one 32 x 32
// tile: the raw texels of the tile and its apron (indices clamped to the map,
// as the passes clamp theirs) are staged in shared memory, the x pass is
// computed for every apron row, then the y pass reads it there.  Each output
// is the same sum, in the same order, as the two-dispatch form.
__global__ void __launch_bounds__(256) shadow_blur_kernel(const float2* __restrict__ raw, float2* out, int w, int h) {
    constexpr int kRows = kBlurTile + 2 * kBlurApron;
    __shared__ float2 src[kRows][kBlurTile + 2 * kBlurApron];
    __shared__ float2 hx[kRows][kBlurTile];
    const int x0 = blockIdx.x * kBlurTile, y0 = blockIdx.y * kBlurTile;
    const int tid = threadIdx.x;
    for (int i = tid; i < kRows * kRows; i += blockDim.x) {
        int r = i / kRows, c = i % kRows;
        int gy = min(max(y0 - kBlurApron + r, 0), h - 1), gx = min(max(x0 - kBlurApron + c, 0), w - 1);
        src[r][c] = __ldg(raw + (size_t)gy * w + gx);
    }
    __syncthreads();
    for (int i = tid; i < kRows * kBlurTile; i += blockDim.x) {
        int r = i / kBlurTile, c = i % kBlurTile;
        int gx = x0 + c;
        if (gx >= w) continue;
        float2 v = src[r][c + kBlurApron];
        float2 s = make_float2(v.x * kBlurWeight[0], v.y * kBlurWeight[0]);
#pragma unroll
        for (int k = 1; k < 5; ++k) {
            // indices clamped against the map: max(x - k, 0), min(x + k, w - 1)
            float2 l = src[r][max(gx - k, 0) - x0 + kBlurApron];
            float2 rr = src[r][min(gx + k, w - 1) - x0 + kBlurApron];
            s.x = fmaf(l.x, kBlurWeight[k], s.x);
            s.y = fmaf(l.y, kBlurWeight[k], s.y);
            s.x = fmaf(rr.x, kBlurWeight[k], s.x);
            s.y = fmaf(rr.y, kBlurWeight[k], s.y);
        }
        hx[r][c] = s;
    }
    __syncthreads();
    for (int i = tid; i < kBlurTile * kBlurTile; i += blockDim.x) {
        int r = i / kBlurTile, c = i % kBlurTile;
        int gx = x0 + c, gy = y0 + r;
        if (gx >= w || gy >= h) continue;
        float2 v = hx[r + kBlurApron][c];
        float2 s = make_float2(v.x * kBlurWeight[0], v.y * kBlurWeight[0]);
#pragma unroll
        for (int k = 1; k < 5; ++k) {
            float2 l = hx[max(gy - k, 0) - y0 + kBlurApron][c];
            float2 rr = hx[min(gy + k, h - 1) - y0 + kBlurApron][c];
            s.x = fmaf(l.x, kBlurWeight[k], s.x);
            s.y = fmaf(l.y, kBlurWeight[k], s.y);
            s.x = fmaf(rr.x, kBlurWeight[k], s.x);
            s.y = fmaf(rr.y, kBlurWeight[k], s.y);
        }
        out[(size_t)gy * w + gx] = s;
    }
}

// The shadow froxel (VolumetricCloudShadowFroxel.comp:10-27).  Block = 32
// columns along x by G = ceil(depth / 16) chunk threads; a thread samples its
// 16 slices (SampleCloudShadowTransmittance, VolumetricCloudShadowInterface.glsl:4-8),
// the chunk totals are scanned across the block, and each slice stores
// (sum of the slices up to it) / (z + 1) as unorm16.
__global__ void __launch_bounds__(1024) shadow_froxel_kernel(CloudConsts C, FroxelConsts F,
                                                             const float2* __restrict__ map, uint16_t* froxel) {
    __shared__ float totals[32][33];
    const int lane = threadIdx.x, g = threadIdx.y;
    const int fx = blockIdx.x * 32 + lane, fy = blockIdx.y;
    const bool live = fx < F.width;
    // view ray through the column centre at NDC z = 0
    const float nx = ((float)min(fx, F.width - 1) + 0.5f) / (float)F.width * 2.f - 1.f;
    const float ny = ((float)fy + 0.5f) / (float)F.height * 2.f - 1.f;
    float3 num = C.a0 * nx + C.a1 * ny + C.a3;
    float wv = fmaf(C.w0, nx, fmaf(C.w1, ny, C.w3));
    float3 dir = num * (copysignf(1.f, wv) * rsqrtf(dot3(num, num)));
    // light clip coordinates of cam + t dir: h0 + t h1
    const float* L = F.lvp;
    float4 h0, h1;
    h0.x = fmaf(L[0], C.cam.x, fmaf(L[4], C.cam.y, fmaf(L[8], C.cam.z, L[12])));
    h0.y = fmaf(L[1], C.cam.x, fmaf(L[5], C.cam.y, fmaf(L[9], C.cam.z, L[13])));
    h0.z = fmaf(L[2], C.cam.x, fmaf(L[6], C.cam.y, fmaf(L[10], C.cam.z, L[14])));
    h0.w = fmaf(L[3], C.cam.x, fmaf(L[7], C.cam.y, fmaf(L[11], C.cam.z, L[15])));
    h1.x = fmaf(L[0], dir.x, fmaf(L[4], dir.y, L[8] * dir.z));
    h1.y = fmaf(L[1], dir.x, fmaf(L[5], dir.y, L[9] * dir.z));
    h1.z = fmaf(L[2], dir.x, fmaf(L[6], dir.y, L[10] * dir.z));
    h1.w = fmaf(L[3], dir.x, fmaf(L[7], dir.y, L[11] * dir.z));
    const int z0 = g * kFroxelChunk;
    float vis[kFroxelChunk];
    float run = 0.f;
#pragma unroll
    for (int k = 0; k < kFroxelChunk; ++k) {
        int z = z0 + k;
        float s = 0.f;
        if (z < F.depth) {
            float t = ((float)z + 0.5f) * F.step;
            float iw = 1.f / fmaf(t, h1.w, h0.w);
            float lx = fmaf(t, h1.x, h0.x) * iw, ly = fmaf(t, h1.y, h0.y) * iw, lz = fmaf(t, h1.z, h0.z) * iw;
            float2 dt = map_bilinear_border(map, F.map_w, F.map_h, lx * 0.5f + 0.5f, ly * 0.5f + 0.5f);
            // mix(T, 1, clamp((depth - z) / 0.5, 0, 1))
            float kk = fminf(fmaxf((dt.x - lz) * 2.f, 0.f), 1.f);
            s = dt.y + (1.f - dt.y) * kk;
        }
        run += s;
        vis[k] = run;
    }
    totals[g][lane] = run;
    __syncthreads();
    float base = 0.f;
    for (int k = 0; k < g; ++k) base += totals[k][lane];
    if (!live) return;
    const size_t slice = (size_t)F.width * F.height;
    uint16_t* col = froxel + (size_t)fy * F.width + fx;
#pragma unroll
    for (int k = 0; k < kFroxelChunk; ++k) {
        int z = z0 + k;
        if (z < F.depth) {
            float m = (base + vis[k]) / (float)(z + 1);
            col[(size_t)z * slice] = (uint16_t)__float2uint_rn(fminf(fmaxf(m, 0.f), 1.f) * 65535.f);
        }
    }
}

}  // namespace
}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_cloud_shadow_sizes_default(int viewport_width, int viewport_height, skyr_cloud_shadow_sizes* out) {
    if (!out) return set_error(SKYR_EINVAL, "null shadow sizes");
    if (viewport_width < 12 || viewport_height < 12) return set_error(SKYR_EINVAL, "viewport must be >= 12 x 12");
    out->map_width = out->map_height = 512;
    out->froxel_width = viewport_width / 12;
    out->froxel_height = viewport_height / 12;
    out->froxel_depth = 128;
    return SKYR_OK;
}

int skyr_cloud_light_frame_derive(const skyr_atmosphere_parameters* atmosphere,
                                  const skyr_cloud_parameters* cloud, const skyr_cloud_view* view,
                                  const skyr_cloud_shadow_sizes* sizes, const skyr_cloud_light_frame* previous,
                                  const float* wind_delta, skyr_cloud_light_frame* out) {
    if (!atmosphere || !cloud || !view || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int st = validate_shadow_sizes(sizes, false)) return st;
    const double dmax = cloud->shadow_map_max_distance;
    if (!(dmax > 0.0) || !std::isfinite(dmax)) return set_error(SKYR_EINVAL, "bad shadow_map_max_distance");
    const double deg = M_PI / 180.0;
    const double R = atmosphere->bottom_radius;
    // the local z-up frame (VolumetricCloud.cpp:188-201)
    const V3d center{0.0, -R, 0.0};
    const V3d cam{view->camera_position[0], view->camera_position[1], view->camera_position[2]};
    const V3d up = normalized(cam - center);
    const V3d origin = center + up * R;
    const V3d front = normalized(cross(up, V3d{1.0, 0.0, 0.0}));
    const V3d right = normalized(cross(up, front));
    double model[16] = {front.x, front.y, front.z, 0, right.x, right.y, right.z, 0,
                        up.x,    up.y,    up.z,    0, origin.x, origin.y, origin.z, 1};
    auto to_local = [&](V3d p) {  // inverse(model): the rotation is orthonormal
        V3d q = p - origin;
        return V3d{dot(front, q), dot(right, q), dot(up, q)};
    };
    auto dir_to_local = [&](V3d v) { return V3d{dot(front, v), dot(right, v), dot(up, v)}; };
    const V3d cam_l = to_local(cam);
    const double th = view->sun_direction_theta * deg, ph = view->sun_direction_phi * deg;
    const V3d sun_w{std::cos(ph) * std::sin(th), std::cos(th), std::sin(ph) * std::sin(th)};
    const V3d sun_l0 = dir_to_local(sun_w);
    if (!(dot(sun_l0, sun_l0) > 0.0)) return set_error(SKYR_EINVAL, "zero sun direction");
    const V3d sun_l = normalized(sun_l0);
    // light view: glm::lookAt(cam, cam - sun, up) (VolumetricCloud.cpp:222-223)
    const V3d lup = (sun_l.x == 0.0 && sun_l.y == 0.0) ? V3d{1, 0, 0} : V3d{0, 0, 1};
    const V3d f = normalized(sun_l * -1.0);
    const V3d s = normalized(cross(f, lup));
    const V3d u = cross(s, f);
    double light_view[16] = {s.x, u.x, -f.x, 0, s.y, u.y, -f.y, 0, s.z, u.z, -f.z, 0,
                             -dot(s, cam_l), -dot(u, cam_l), dot(f, cam_l), 1};
    // GetLightProjection (VolumetricCloud.cpp:138-166): the camera and the four
    // corners of the frustum's cross-section at shadow_map_max_distance.  The
    // corners lie on the rays through NDC (+-1, +-1), the section's centre on
    // the ray through NDC (0, 0) (Camera::ViewProjection is a symmetric
    // glm::perspective times a lookAt).
    double vp[16], ivp[16];
    for (int i = 0; i < 16; ++i) vp[i] = view->view_projection[i];
    if (!invert4d(vp, ivp)) return set_error(SKYR_EINVAL, "view_projection is singular");
    auto ray = [&](double x, double y) {
        double p[4] = {x, y, 0.0, 1.0}, q[4];
        transform(ivp, p, q);
        return V3d{q[0] / q[3], q[1] / q[3], q[2] / q[3]} - cam;
    };
    const V3d fr = normalized(ray(0.0, 0.0));
    V3d verts[5];
    verts[0] = cam;
    const double cx[4] = {1, -1, 1, -1}, cy[4] = {1, 1, -1, -1};
    for (int k = 0; k < 4; ++k) {
        V3d dk = ray(cx[k], cy[k]);
        double along = dot(dk, fr);
        if (!(along > 0.0)) return set_error(SKYR_EINVAL, "view_projection has no forward frustum");
        verts[k + 1] = cam + dk * (dmax / along);
    }
    double mn[2] = {1e300, 1e300}, mx[2] = {-1e300, -1e300};
    for (const V3d& vw : verts) {
        V3d vl = to_local(vw);
        double p[4] = {vl.x, vl.y, vl.z, 1.0}, q[4];
        transform(light_view, p, q);
        for (int i = 0; i < 2; ++i) {
            mn[i] = std::fmin(mn[i], q[i]);
            mx[i] = std::fmax(mx[i], q[i]);
        }
    }
    const double res[2] = {(double)sizes->map_width, (double)sizes->map_height};
    for (int i = 0; i < 2; ++i) {
        double pad = 0.5 * (mx[i] - mn[i]) / res[i];
        mn[i] -= pad;
        mx[i] += pad;
        if (!(mx[i] > mn[i])) return set_error(SKYR_EINVAL, "degenerate light projection");
    }
    // glm::ortho(l, r, b, t, -1, 1), OpenGL clip depth
    double proj[16] = {2.0 / (mx[0] - mn[0]), 0, 0, 0, 0, 2.0 / (mx[1] - mn[1]), 0, 0, 0, 0, -1.0, 0,
                       -(mx[0] + mn[0]) / (mx[0] - mn[0]), -(mx[1] + mn[1]) / (mx[1] - mn[1]), 0.0, 1.0};
    double lvp[16], ilvp[16];
    matmul4d(proj, light_view, lvp);
    if (!invert4d(lvp, ilvp)) return set_error(SKYR_EINVAL, "singular light view-projection");
    skyr_cloud_light_frame o;
    std::memset(&o, 0, sizeof(o));
    for (int i = 0; i < 16; ++i) {
        o.light_view_projection[i] = (float)lvp[i];
        o.inverse_light_view_projection[i] = (float)ilvp[i];
        o.model[i] = (float)model[i];
    }
    if (previous) {
        // pre_light_vp * inverse(pre_model) * model * translate(wind) * inv_light_vp (VolumetricCloud.cpp:235)
        double pvp[16], pm[16], ipm[16], wind[16], a[16], b[16], c[16], r[16];
        for (int i = 0; i < 16; ++i) {
            pvp[i] = previous->light_view_projection[i];
            pm[i] = previous->model[i];
        }
        if (!invert4d(pm, ipm)) return set_error(SKYR_EINVAL, "previous model is singular");
        identity4(wind);
        if (wind_delta) {
            wind[12] = wind_delta[0];
            wind[13] = wind_delta[1];
        }
        matmul4d(pvp, ipm, a);
        matmul4d(a, model, b);
        matmul4d(b, wind, c);
        matmul4d(c, ilvp, r);
        for (int i = 0; i < 16; ++i) o.shadow_map_reproject[i] = (float)r[i];
        o.has_previous = 1;
    } else {
        double id[16];
        identity4(id);
        for (int i = 0; i < 16; ++i) o.shadow_map_reproject[i] = (float)id[i];
    }
    *out = o;
    return SKYR_OK;
}

int skyr_cloud_shadow_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                             const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                             const skyr_cloud_textures* textures, const skyr_cloud_view* view,
                             const skyr_cloud_shadow_sizes* sizes, const skyr_cloud_light_frame* frame,
                             const float* blue_noise, const float* previous_raw_map, float* raw_map,
                             float* shadow_map, uint16_t* froxel) {
    if (!ctx || !atmosphere || !cloud || !material || !textures || !view || !frame)
        return set_error(SKYR_EINVAL, "null argument");
    if (!blue_noise || !raw_map) return set_error(SKYR_EINVAL, "null blue noise or raw map");
    if (froxel && !shadow_map) return set_error(SKYR_EINVAL, "the froxel pass needs the blurred shadow map");
    if (int st = validate_shadow_sizes(sizes, froxel != nullptr)) return st;
    if (previous_raw_map == raw_map || shadow_map == raw_map || (shadow_map && shadow_map == previous_raw_map))
        return set_error(SKYR_EINVAL, "shadow map buffers must be distinct");
    if (material->type < SKYR_MATERIAL_DEFAULT0 || material->type > SKYR_MATERIAL_VOXEL)
        return set_error(SKYR_EINVAL, "unknown material type %d", material->type);
    if (!(cloud->thickness > 0.f)) return set_error(SKYR_EINVAL, "cloud thickness must be > 0");
    if (froxel && !(cloud->shadow_froxel_max_distance > 0.f))
        return set_error(SKYR_EINVAL, "bad shadow_froxel_max_distance");
    if (view->viewport_width < 1 || view->viewport_height < 1) return set_error(SKYR_EINVAL, "bad viewport size");
    skyr_lut_sizes none;
    std::memset(&none, 0, sizeof(none));
    CloudConsts C;
    MaterialConsts M;
    if (int st = derive_cloud_consts(*atmosphere, *cloud, *material, *textures, *view, none, C, M)) return st;

    // texel origins: ProjectiveMul(uInvLightVP, (x, y, 0)) as (o0 x + o1 y + o3) / (q0 x + q1 y + q3)
    ShadowMapConsts S;
    std::memset(&S, 0, sizeof(S));
    const float* il = frame->inverse_light_view_projection;
    S.o0 = make_float3(il[0], il[1], il[2]);
    S.o1 = make_float3(il[4], il[5], il[6]);
    S.o3 = make_float3(il[12], il[13], il[14]);
    S.q0 = il[3];
    S.q1 = il[7];
    S.q3 = il[15];
    // dir = -uSunDirection: the local sun of the view, as the raymarch uses it
    S.dir = make_float3(-C.sun.x, -C.sun.y, -C.sun.z);
    S.rho2_bottom = C.rho2_bottom;
    S.rho2_top = C.rho2_top;
    S.max_dist = (float)(1.0 / std::cos(85.0 * M_PI / 180.0) * ((double)C.top - (double)C.bottom));
    S.steps = 12.f + (6.f - 12.f) * fabsf(S.dir.z);  // mix(12, 6, |dir.z|)
    S.width = sizes->map_width;
    S.height = sizes->map_height;
    S.reproject = (previous_raw_map && frame->has_previous) ? 1 : 0;
    for (int i = 0; i < 16; ++i) S.rp[i] = frame->shadow_map_reproject[i];

    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    cudaStream_t stream = ctx->stream;
    dim3 mb(16, 8), mg((S.width + 15) / 16, (S.height + 7) / 8);
    shadow_map_kernel<<<mg, mb, 0, stream>>>(C, M, S, blue_noise, reinterpret_cast<const float2*>(previous_raw_map),
                                             reinterpret_cast<float2*>(raw_map));
    if (int e = check_cuda(cudaGetLastError(), "shadow map kernel")) return e;
    if (!shadow_map) return SKYR_OK;
    dim3 bg((S.width + kBlurTile - 1) / kBlurTile, (S.height + kBlurTile - 1) / kBlurTile);
    shadow_blur_kernel<<<bg, 256, 0, stream>>>(reinterpret_cast<const float2*>(raw_map),
                                               reinterpret_cast<float2*>(shadow_map), S.width, S.height);
    if (int e = check_cuda(cudaGetLastError(), "shadow blur kernel")) return e;
    if (!froxel) return SKYR_OK;
    FroxelConsts F;
    std::memset(&F, 0, sizeof(F));
    for (int i = 0; i < 16; ++i) F.lvp[i] = frame->light_view_projection[i];
    F.width = sizes->froxel_width;
    F.height = sizes->froxel_height;
    F.depth = sizes->froxel_depth;
    F.map_w = S.width;
    F.map_h = S.height;
    F.step = cloud->shadow_froxel_max_distance / (float)F.depth;
    const int chunks = (F.depth + kFroxelChunk - 1) / kFroxelChunk;
    dim3 fb(32, chunks), fg((F.width + 31) / 32, F.height);
    shadow_froxel_kernel<<<fg, fb, 0, stream>>>(C, F, reinterpret_cast<const float2*>(shadow_map), froxel);
    return check_cuda(cudaGetLastError(), "shadow froxel kernel");
}

}  // extern "C"
