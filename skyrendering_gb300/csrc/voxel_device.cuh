// voxel_device.cuh — device helpers shared by the voxel path tracer and the
// surrogate raymarch: launch constants of the dense FP16 grid, the path
// tracer's random numbers, trilinear grid lookup, the cloud region box, the
// sun's illuminance through the atmosphere, HG phase and the camera ray.
#pragma once

#include <cuda_fp16.h>

#include "../../include/skyr_pathtrace.h"
#include "cloud_internal.cuh"
#include "lut_access.cuh"
#include "noise_device.cuh"

namespace skyr {

// The samples of one free-flight / ratio-tracking walk are bounded by
// PtConsts::tracking_steps (skyr_device_limits, default 2^20).  A valid scene
// needs ~sigma_max x chord samples (tens to hundreds); the bound only stops
// pathological inputs, ends the path and raises the status flag.

struct PtConsts {
    float3 box_min, box_max;
    int max_bounces, importance_sampling, prng, env;
    float g_fwd, g_back, ratio, sigma_t_max;
    int use_bricks;
    // dense grid
    const unsigned short* grid;
    int nx, ny, nz;
    float3 origin;
    float inv_voxel, density;
    const float* maj;
    int bx, by, bz;
    float brick_size;
    // local -> world directions (kModelMatrix3 columns)
    float3 m_front, m_right, m_up;
    int sv_w, sv_h;
    int width, height;
    int x0, y0, x1, y1;
    int tiles_x, n_items;  // work items of one frame (8x4 pixel tiles x 32)
    // pixel-list source: n_items pixels (y * width + x), else the region tiles
    const int* pixel_list;
    // point source: paths start at points[i] = (position, direction) as if the
    // direction had just scattered there; their radiance is added to
    // point_out[i] (rgb)
    const float* points;
    float* point_out;
    int* status;         // bit 0: a tracking walk hit tracking_steps
    int tracking_steps;  // bound on the samples of one walk
};

__device__ __forceinline__ void flag_overrun(const PtConsts& P) {
    if (P.status) atomicOr(P.status, 1);
}

__device__ __forceinline__ uint32_t pt_prng(const PtConsts& P, uint32_t s) {
    return P.prng == SKYR_PRNG_WANG_HASH ? wang_hash(s) : pcg_hash(s);
}

// Random01 (PathTracing.comp:44-48): float(seed) / 2^32
__device__ __forceinline__ float rand01(const PtConsts& P, uint32_t& seed) {
    float r = (float)seed * 2.3283064365386963e-10f;
    seed = pt_prng(P, seed);
    return r;
}

// Trilinear between texel centres of an FP16 volume of nx x ny x nz texels
// with a zero border, at continuous texel coordinates (gx, gy, gz) (texel
// centres at integers): a texel outside the volume reads 0.  The eight texels
// are addressed from one base offset, and each axis is tested once per end;
// a texel that fails its test is not loaded.
__device__ __forceinline__ float trilinear_zero_border(const unsigned short* __restrict__ data, int nx, int ny,
                                                       int nz, float gx, float gy, float gz) {
    float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    float a = gx - fx, b = gy - fy, c = gz - fz;
    int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    const bool vx0 = (unsigned)x0 < (unsigned)nx, vx1 = (unsigned)(x0 + 1) < (unsigned)nx;
    const bool vy0 = (unsigned)y0 < (unsigned)ny, vy1 = (unsigned)(y0 + 1) < (unsigned)ny;
    const long long sy = nx, sz = (long long)nx * ny;
    const long long base = (long long)z0 * sz + (long long)y0 * sy + x0;
    auto texel = [&](long long i, bool v) -> float {
        return v ? __half2float(__ushort_as_half(__ldg(data + i))) : 0.f;
    };
    float r[2];
#pragma unroll
    for (int dz = 0; dz < 2; ++dz) {
        const bool vz = (unsigned)(z0 + dz) < (unsigned)nz;
        const long long i = base + dz * sz;
        float t00 = texel(i, vz && vy0 && vx0), t10 = texel(i + 1, vz && vy0 && vx1);
        float t01 = texel(i + sy, vz && vy1 && vx0), t11 = texel(i + sy + 1, vz && vy1 && vx1);
        float top = fmaf(a, t10 - t00, t00), bot = fmaf(a, t11 - t01, t01);
        r[dz] = fmaf(b, bot - top, top);
    }
    return fmaf(c, r[1] - r[0], r[0]);
}

// trilinear between voxel centres, zero border
__device__ __forceinline__ float grid_sigma(const PtConsts& P, float3 p) {
    float gx = (p.x - P.origin.x) * P.inv_voxel - 0.5f;
    float gy = (p.y - P.origin.y) * P.inv_voxel - 0.5f;
    float gz = (p.z - P.origin.z) * P.inv_voxel - 0.5f;
    return trilinear_zero_border(P.grid, P.nx, P.ny, P.nz, gx, gy, gz) * P.density;
}

// CloudRegionIntersect (PathTracing.comp:57-75)
__device__ __forceinline__ void region(const PtConsts& P, float3 o, float3 d, float& t0, float& t1) {
    float3 inv = f3(1.f / d.x, 1.f / d.y, 1.f / d.z);
    float ax = (P.box_min.x - o.x) * inv.x, bx = (P.box_max.x - o.x) * inv.x;
    float ay = (P.box_min.y - o.y) * inv.y, by = (P.box_max.y - o.y) * inv.y;
    float az = (P.box_min.z - o.z) * inv.z, bz = (P.box_max.z - o.z) * inv.z;
    t0 = fmaxf(0.f, fmaxf(fminf(ax, bx), fmaxf(fminf(ay, by), fminf(az, bz))));
    t1 = fminf(1e7f, fminf(fmaxf(ax, bx), fminf(fmaxf(ay, by), fmaxf(az, bz))));
}

// GetSunVisibility(transmittance_texture, pos) x solar_illuminance, local frame
__device__ __forceinline__ float3 sun_illuminance(const CloudConsts& C, const AtmoConsts& A, const float4* tlut,
                                                  int tw, int th, float3 p) {
    float rho2 = fmaf(p.x, p.x, fmaf(p.y, p.y, p.z * (p.z + 2.f * C.R)));
    float r2 = fmaf(C.R, C.R, rho2);
    float inv_r = rsqrtf(r2);
    float r = r2 * inv_r;
    float h = __fdividef(rho2, r + C.R);
    float mu_s = fmaf(C.sun.x, p.x, fmaf(C.sun.y, p.y, C.sun.z * (p.z + C.R))) * inv_r;
    return sun_visibility_lut(A, tlut, tw, th, r, rho2, h, mu_s) * A.solar_illuminance;
}

__device__ __forceinline__ void onb(float3 n, float3& t0, float3& t1) {  // Common.glsl:45-50
    float s = n.z >= 0.f ? 1.f : -1.f;
    float a = -1.f / (s + n.z);
    float b = n.x * n.y * a;
    t0 = f3(1.f + s * n.x * n.x * a, s * b, -s * n.x);
    t1 = f3(b, s + n.y * n.y * a, -n.y);
}

__device__ __forceinline__ float hg_pt(float c, float g) {
    float a = 1.f - g * g;
    float b = fmaf(-2.f * g, c, 1.f + g * g);
    return (0.25f / SKYR_PI) * a / (b * sqrtf(b));
}

// Primary ray through the pixel centre at NDC z = 1 (far plane); also the
// texture coordinates of the pixel for the aerial-perspective lookup.
__device__ __forceinline__ float3 primary_dir(const CloudConsts& C, const PtConsts& P, int px, int py, float& u,
                                              float& v) {
    u = ((float)px + 0.5f) / (float)P.width;
    v = ((float)py + 0.5f) / (float)P.height;
    float x = 2.f * u - 1.f, y = 2.f * v - 1.f;
    float3 dir = C.a0 * x + C.a1 * y + C.af;
    float wv = fmaf(C.w0, x, fmaf(C.w1, y, C.wf));
    return dir * (copysignf(1.f, wv) * rsqrtf(dot3(dir, dir)));
}

}  // namespace skyr
