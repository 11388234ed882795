// surrogate.cu — the surrogate-shaded voxel cloud (include/skyr_surrogate.h):
// the feature lattice, training points and records, and the 128-step raymarch
// with the network of mlp_device.cuh evaluated inside the march.
//
// The raymarch keeps a warp on an 8x4 pixel tile.  At each step the lanes whose
// sample lies in the cloud write their feature record (interpolated from the
// lattice) to the warp's shared-memory tile, and the warp evaluates the network
// for its 32 samples on the tensor cores (mma.sync BF16, FP32 accumulation);
// single scattering of the sun uses the lattice's optical depth to the sun.
#include <cmath>
#include <cstring>

#include "../../include/skyr_surrogate.h"
#include "mlp_device.cuh"
#include "skyr_ctx.cuh"
#include "voxel_device.cuh"

namespace skyr {
namespace {

// Feature record layout (skyr_surrogate.h): kRec bf16, kRec / 8 chunks of 16 bytes.
constexpr int kRecQ = SKYR_MLP_RECORD / 8;  // chunks per record (14)
constexpr int kLatQ = 10;                   // chunks per lattice node: features 0..79 of the record
constexpr int kSun = 32;                    // samples toward the sun (features 1..32)
constexpr int kViewNbr = 33;                // features 33..40: view-oriented cube corners (per sample)
constexpr int kHeight = 41;                 // height in the grid box (lattice)
constexpr int kCos = 42;                    // cos(view, sun) (per sample)
constexpr int kFar = 43;                    // transmittance along the view ray to the box's exit (per sample)
constexpr int kStencil = 44;                // features 44..78: the sun-oriented density stencil (lattice)
constexpr int kStencilLevels = 5;           // mip levels 2..6
constexpr int kStencilFirst = 2;
constexpr int kStencilPoints = 7;           // centre and +-1 along the stencil's three axes
constexpr int kViewSt = kStencil + kStencilLevels * kStencilPoints;  // 79..102: the view-oriented stencil (per sample)
constexpr int kViewStLevels = 4;            // mip levels 3..6
constexpr int kViewStFirst = 3;
constexpr int kViewStPoints = 6;            // +-1 along the view frame's three axes (the centres are in 44..78)
constexpr int kMipLevels = 6;               // levels 1..6 of the grid, kept in the lattice's buffer
static_assert(kViewSt + kViewStLevels * kViewStPoints == SKYR_MLP_INPUTS, "network inputs");
static_assert(kLatQ * 8 == kViewSt + 1 && kRecQ >= kLatQ, "lattice nodes hold features 0..kViewSt");
constexpr int kMaxSampleTries = 64;
constexpr int kMaxTrackSteps = 1 << 16;

struct Lattice {
    const uint4* rec;  // [nodes][kLatQ] (features 0..79 of the record, the per-sample slots zero)
    const float* tau;  // [nodes]
    int nx, ny, nz;
    float3 origin;
    float inv_cell;
    float3 sun;
};

// Level l (1..6) of the grid's mip chain: each texel the mean of the (up to)
// 2 x 2 x 2 texels of level l - 1 that exist (ceil sizes), FP16.
struct MipLevel {
    const unsigned short* data;
    int nx, ny, nz;
    float inv_voxel;
};
struct Mips {
    MipLevel level[kMipLevels + 1];  // [0] is the grid itself
    float voxel;                     // the grid's voxel edge
};

__device__ __forceinline__ float u01(uint32_t& s) {
    s = pcg_hash(s);
    return (float)(s >> 8) * (1.f / 16777216.f);
}

__device__ __forceinline__ float3 uniform_dir(uint32_t& s) {
    float c = 1.f - 2.f * u01(s), ph = 2.f * SKYR_PI * u01(s);
    float r = sqrtf(fmaxf(0.f, 1.f - c * c)), sp, cp;
    sincosf(ph, &sp, &cp);
    return f3(r * cp, r * sp, c);
}

// slab intersection of the ray with [lo, hi]
__device__ __forceinline__ void box_hit(float3 lo, float3 hi, float3 o, float3 d, float& t0, float& t1) {
    float3 inv = f3(1.f / d.x, 1.f / d.y, 1.f / d.z);
    float ax = (lo.x - o.x) * inv.x, bx = (hi.x - o.x) * inv.x;
    float ay = (lo.y - o.y) * inv.y, by = (hi.y - o.y) * inv.y;
    float az = (lo.z - o.z) * inv.z, bz = (hi.z - o.z) * inv.z;
    t0 = fmaxf(0.f, fmaxf(fminf(ax, bx), fmaxf(fminf(ay, by), fminf(az, bz))));
    t1 = fminf(fmaxf(ax, bx), fminf(fmaxf(ay, by), fmaxf(az, bz)));
}

struct GridBox {
    float3 lo, hi;
    float span;  // longest edge
};

// Trilinear between texel centres of a mip level, zero border (grid_sigma's
// convention), in the grid's units (without the grid's density factor).
__device__ __forceinline__ float mip_value(const MipLevel& M, float3 origin, float3 p) {
    float gx = (p.x - origin.x) * M.inv_voxel - 0.5f, gy = (p.y - origin.y) * M.inv_voxel - 0.5f,
          gz = (p.z - origin.z) * M.inv_voxel - 0.5f;
    return trilinear_zero_border(M.data, M.nx, M.ny, M.nz, gx, gy, gz);
}

// Level l + 1 texel (x, y, z) from level l: the mean of the texels that exist.
__global__ void __launch_bounds__(256) mip_reduce_kernel(MipLevel src, MipLevel dst, unsigned short* __restrict__ out) {
    size_t n = (size_t)dst.nx * dst.ny * dst.nz;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int x = (int)(i % dst.nx), y = (int)((i / dst.nx) % dst.ny), z = (int)(i / ((size_t)dst.nx * dst.ny));
    float sum = 0.f;
    int cnt = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        int sx = 2 * x + (c & 1), sy = 2 * y + ((c >> 1) & 1), sz = 2 * z + (c >> 2);
        if (sx < src.nx && sy < src.ny && sz < src.nz) {
            sum += __half2float(__ushort_as_half(__ldg(src.data + ((size_t)sz * src.ny + sy) * src.nx + sx)));
            ++cnt;
        }
    }
    out[i] = __half_as_ushort(__float2half_rn(sum / (float)cnt));
}

// The lattice's trilinear cell at x: the 8 node indices and weights.
struct LatticeCell {
    size_t node[8];
    float w[8];
};
__device__ __forceinline__ void lattice_cell(const Lattice& L, float3 x, LatticeCell& c) {
    float gx = (x.x - L.origin.x) * L.inv_cell, gy = (x.y - L.origin.y) * L.inv_cell,
          gz = (x.z - L.origin.z) * L.inv_cell;
    int ix = min(max((int)floorf(gx), 0), L.nx - 2), iy = min(max((int)floorf(gy), 0), L.ny - 2),
        iz = min(max((int)floorf(gz), 0), L.nz - 2);
    float fx = fminf(fmaxf(gx - ix, 0.f), 1.f), fy = fminf(fmaxf(gy - iy, 0.f), 1.f),
          fz = fminf(fmaxf(gz - iz, 0.f), 1.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
        c.w[k] = (dx ? fx : 1.f - fx) * (dy ? fy : 1.f - fy) * (dz ? fz : 1.f - fz);
        c.node[k] = ((size_t)(iz + dz) * L.ny + (iy + dy)) * L.nx + (ix + dx);
    }
}

// The optical depth to the sun at x, interpolated from the lattice.
__device__ __forceinline__ float lattice_tau(const Lattice& L, const LatticeCell& c) {
    float tau = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) tau = fmaf(c.w[k], __ldg(L.tau + c.node[k]), tau);
    return tau;
}

// Features 33..40: extinction / sigma_ref at the 8 corners of a cube whose
// corners lie `dist` from x, with axes (v, u, w): v the view direction, u the
// sun's component perpendicular to v (any perpendicular when the two are
// parallel), w = v x u.  Corner j takes +dist/sqrt(3) along v, u, w where bit
// 0, 1, 2 of j is set, -dist/sqrt(3) where it is not.
// The view frame (v, u, w): u the sun's component perpendicular to v (any
// perpendicular when the two are parallel), w = v x u.
__device__ __forceinline__ void view_frame(float3 v, float3 sun, float3& u, float3& w) {
    u = sun - v * dot3(v, sun);
    float l2 = dot3(u, u);
    if (l2 < 1e-8f) {
        float3 b1;
        onb(v, u, b1);
    } else {
        u = u * rsqrtf(l2);
    }
    w = f3(v.y * u.z - v.z * u.y, v.z * u.x - v.x * u.z, v.x * u.y - v.y * u.x);
}

__device__ __forceinline__ void view_neighbours(const PtConsts& P, float3 x, float3 v, float3 u, float3 w, float dist,
                                                float inv_ref, float (&nb)[8]) {
    const float r = dist * 0.57735026918962576f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float3 o = v * ((j & 1) ? r : -r) + u * ((j & 2) ? r : -r) + w * ((j & 4) ? r : -r);
        nb[j] = grid_sigma(P, x + o) * inv_ref;
    }
}

// The feature record of a sample at x seen along v: the lattice's features
// interpolated trilinearly chunk by chunk, with the per-sample slots filled in
// (the view neighbours, cos(v, sun), the far-side transmittance `far_t`, the
// view-oriented stencil over the mip levels M), written as kRecQ 16-byte
// chunks to `row`.  Returns the sun optical depth; f0 / near_sun receive
// feature 0 and the mean of features 1..8 (the error table's bin).
__device__ __forceinline__ float write_record(const Lattice& L, const PtConsts& P, const Mips& M, float3 x, float3 v,
                                              float nbr, float inv_ref, float far_t, uint4* row, float& f0,
                                              float& near_sun) {
    LatticeCell c;
    lattice_cell(L, x, c);
    const float tau = lattice_tau(L, c);
    float3 fu, fw;
    view_frame(v, L.sun, fu, fw);
    float nb[8];
    view_neighbours(P, x, v, fu, fw, nbr, inv_ref, nb);
    const float mu = dot3(v, L.sun);
    const float k_ref = inv_ref * P.density;
    float near = 0.f;
#pragma unroll
    for (int q = 0; q < kRecQ; ++q) {
        float a[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) a[e] = 0.f;
        if (q < kLatQ) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint4 u = __ldg(L.rec + c.node[k] * kLatQ + q);
                uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&w4[h]);
                    a[2 * h] = fmaf(c.w[k], __low2float(b), a[2 * h]);
                    a[2 * h + 1] = fmaf(c.w[k], __high2float(b), a[2 * h + 1]);
                }
            }
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = q * 8 + e;
            if (i >= kViewNbr && i < kViewNbr + 8) a[e] = nb[i - kViewNbr];
            if (i == kCos) a[e] = mu;
            if (i == kFar) a[e] = far_t;
            if (i == 0) f0 = a[e];
            if (i >= 1 && i <= 8) near += a[e];
        }
        row[q] = make_uint4(mlp::pack_bf16(a[0], a[1]), mlp::pack_bf16(a[2], a[3]), mlp::pack_bf16(a[4], a[5]),
                            mlp::pack_bf16(a[6], a[7]));
    }
    // the view-oriented stencil over the chunks' zeros, one value at a time in a
    // rolled loop (unrolled, its 24 lookups crowd the instruction cache):
    // +-2^(l+1) voxels along v, u, w at mip level l = kViewStFirst + s / 6
    __nv_bfloat16* rb = reinterpret_cast<__nv_bfloat16*>(row);
#pragma unroll 1
    for (int s = 0; s < kViewStLevels * kViewStPoints; ++s) {
        const int lv = kViewStFirst + s / kViewStPoints, j = s % kViewStPoints;
        const float3 ax = j < 2 ? v : j < 4 ? fu : fw;
        const float h = M.voxel * (float)(2 << lv) * ((j & 1) ? -1.f : 1.f);
        rb[kViewSt + s] = __float2bfloat16_rn(mip_value(M.level[lv], P.origin, x + ax * h) * k_ref);
    }
    near_sun = near * 0.125f;
    return tau;
}

struct LatticeBuild {
    float dist[kSun];  // sun sample distances
    float nbr;         // neighbour radius
    float inv_sigma_ref;
    float step;        // sun optical-depth march step
    float3 axis[3];    // the stencil's axes: the sun, then two perpendiculars
    float spacing[kStencilLevels];  // stencil step at each level: 2 texels of the level
    float inv_brick;   // 1 / the brick edge (P.maj non-null)
};

// Whether the grid is empty around p: the brick majorant there is 0, so every
// trilinear sample in the brick is 0 (its one-voxel apron included).
__device__ __forceinline__ bool empty_brick(const PtConsts& P, float inv_brick, float3 p) {
    int i = min(max((int)floorf((p.x - P.origin.x) * inv_brick), 0), P.bx - 1);
    int j = min(max((int)floorf((p.y - P.origin.y) * inv_brick), 0), P.by - 1);
    int k = min(max((int)floorf((p.z - P.origin.z) * inv_brick), 0), P.bz - 1);
    return __ldg(P.maj + ((size_t)k * P.by + j) * P.bx + i) == 0.f;
}

__global__ void __launch_bounds__(128) feature_lattice_kernel(PtConsts P, GridBox B, Lattice L, LatticeBuild Q,
                                                              Mips M, int stride, uint4* __restrict__ rec,
                                                              float* __restrict__ tau) {
    size_t n = (size_t)L.nx * L.ny * L.nz;
    size_t node = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= n) return;
    int ix = (int)(node % L.nx), iy = (int)((node / L.nx) % L.ny), iz = (int)(node / ((size_t)L.nx * L.ny));
    float cell = 1.f / L.inv_cell;
    float3 x = f3(L.origin.x + ix * cell, L.origin.y + iy * cell, L.origin.z + iz * cell);
    // chunk by chunk: the features of positions q * 8 .. q * 8 + 7
    const float k_ref = Q.inv_sigma_ref * P.density;
#pragma unroll 1
    for (int q = 0; q < kLatQ; ++q) {
        float a[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int i = q * 8 + e;
            float v = 0.f;  // the per-sample slots (view neighbours, cos, far side) and the pad stay zero
            if (i == 0) {
                v = grid_sigma(P, x) * Q.inv_sigma_ref;
            } else if (i <= kSun) {
                v = grid_sigma(P, x + L.sun * Q.dist[i - 1]) * Q.inv_sigma_ref;
            } else if (i == kHeight) {
                v = fminf(fmaxf((x.z - B.lo.z) / (B.hi.z - B.lo.z), 0.f), 1.f);
            } else if (i >= kStencil && i < kStencil + kStencilLevels * kStencilPoints) {
                const int s = i - kStencil, lv = s / kStencilPoints, j = s % kStencilPoints;
                float3 p = x;
                if (j > 0) {
                    const float h = (j & 1) ? Q.spacing[lv] : -Q.spacing[lv];
                    p = x + Q.axis[(j - 1) >> 1] * h;
                }
                v = mip_value(M.level[kStencilFirst + lv], P.origin, p) * k_ref;
            }
            a[e] = v;
        }
        rec[node * kLatQ + q] = make_uint4(mlp::pack_bf16(a[0], a[1]), mlp::pack_bf16(a[2], a[3]),
                                           mlp::pack_bf16(a[4], a[5]), mlp::pack_bf16(a[6], a[7]));
    }
    // optical depth to the sun: midpoint rule to the exit of the grid box; a
    // sample in an empty brick adds exactly 0, so its lookup is skipped
    float t0, t1;
    box_hit(B.lo, B.hi, x, L.sun, t0, t1);
    float od = 0.f;
    if (t1 > 0.f) {
        int steps = min((int)ceilf(t1 / Q.step), kMaxTrackSteps);
        float h = t1 / (float)max(steps, 1);
        for (int s = 0; s < steps; ++s) {
            const float3 p = x + L.sun * ((s + 0.5f) * h);
            if (P.maj && empty_brick(P, Q.inv_brick, p)) continue;
            od += grid_sigma(P, p);
        }
        od *= h;
    }
    tau[node] = od;
}

// Transmittance from x along d to the exit of the grid box: midpoint rule at
// steps of at most `step` (the training records' far-side feature).
__device__ __forceinline__ float far_transmittance(const PtConsts& P, const GridBox& B, float3 x, float3 d,
                                                   float step) {
    float t0, t1;
    box_hit(B.lo, B.hi, x, d, t0, t1);
    float od = 0.f;
    if (t1 > 0.f) {
        int steps = min((int)ceilf(t1 / step), kMaxTrackSteps);
        float h = t1 / (float)max(steps, 1);
        for (int s = 0; s < steps; ++s) od += grid_sigma(P, x + d * ((s + 0.5f) * h));
        od *= h;
    }
    return __expf(-od);
}

__global__ void __launch_bounds__(128) sample_points_kernel(PtConsts P, GridBox B, float sigma_max, float sigma_min,
                                                            uint32_t seed_lo, uint32_t seed_hi, int n,
                                                            float* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = pcg_hash(pcg_hash(seed_lo ^ pcg_hash((uint32_t)i)) + seed_hi);
    float3 ext = B.hi - B.lo;
    float3 x = B.lo + ext * 0.5f, d = f3(0.f, 0.f, 1.f);
    bool found = false;
    if ((i & 1) == 0 && sigma_max > 0.f) {
        // first collision of a ray from outside the box aimed at a random point in it
        for (int tr = 0; tr < kMaxSampleTries && !found; ++tr) {
            float3 q = B.lo + f3(ext.x * u01(s), ext.y * u01(s), ext.z * u01(s));
            float3 dir = uniform_dir(s);
            float3 o = q - dir * (2.f * B.span);
            float t0, t1;
            box_hit(B.lo, B.hi, o, dir, t0, t1);
            float t = t0;
            for (int it = 0; it < kMaxTrackSteps; ++it) {
                t += -__logf(1.f - u01(s)) / sigma_max;
                if (!(t < t1)) break;
                float3 p = o + dir * t;
                if (u01(s) * sigma_max < grid_sigma(P, p)) {
                    x = p;
                    d = dir;
                    found = true;
                    break;
                }
            }
        }
    }
    if (!found) {
        for (int tr = 0; tr < 4 * kMaxSampleTries; ++tr) {
            x = B.lo + f3(ext.x * u01(s), ext.y * u01(s), ext.z * u01(s));
            if (grid_sigma(P, x) >= sigma_min) break;
        }
        d = uniform_dir(s);
    }
    float* o6 = out + 6 * (size_t)i;
    o6[0] = x.x; o6[1] = x.y; o6[2] = x.z;
    o6[3] = d.x; o6[4] = d.y; o6[5] = d.z;
}

__global__ void __launch_bounds__(128) records_kernel(Lattice L, PtConsts P, GridBox B, Mips M, float nbr,
                                                      float inv_ref,
                                                      float far_step, const float* __restrict__ pts, int n,
                                                      uint4* __restrict__ rec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* q = pts + 6 * (size_t)i;
    float3 x = f3(q[0], q[1], q[2]), d = f3(q[3], q[4], q[5]);
    float f0, near_sun;
    write_record(L, P, M, x, d, nbr, inv_ref, far_transmittance(P, B, x, d, far_step), rec + (size_t)i * kRecQ, f0,
                 near_sun);
}

// Sample s of the surrogate raymarch: t = t0 + (s + jitter) dt along dir from o
// (explicit fused operations, so that both loops that visit it agree bit for bit).
__device__ __forceinline__ float3 march_point(float3 o, float3 dir, float t0, float dt, float jitter, int s) {
    const float t = fmaf((float)s + jitter, dt, t0);
    return f3(fmaf(dir.x, t, o.x), fmaf(dir.y, t, o.y), fmaf(dir.z, t, o.z));
}

struct RenderConsts {
    int steps, use_network;
    float network_error, min_t;
    float g_fwd, g_back, ratio;
    const float* error_table;
    float nbr, inv_ref;  // view-neighbour distance and 1 / sigma_ref
    long long copy_wait_cycles;  // bound of the wait for the network's bulk copy
    float inv_brick;     // 1 / the brick edge (P.maj non-null)
};

// The grid's extinction at a march sample: 0 without a lookup where the brick
// majorant says the brick is empty (the lookup would return exactly 0).
__device__ __forceinline__ float march_sigma(const PtConsts& P, float inv_brick, float3 x) {
    if (P.maj && empty_brick(P, inv_brick, x)) return 0.f;
    return grid_sigma(P, x);
}

constexpr int kBins = SKYR_SURROGATE_ERROR_BINS;

// error-table bin of a sample: feature 0 and the mean of features 1..8
__device__ __forceinline__ int error_bin(float f0, float near_sun) {
    int a = min(max((int)(f0 * kBins), 0), kBins - 1), b = min(max((int)(near_sun * kBins), 0), kBins - 1);
    return a * kBins + b;
}

__global__ void __launch_bounds__(256) error_bins_kernel(const __nv_bfloat16* __restrict__ rec, int n,
                                                         int* __restrict__ bins) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const __nv_bfloat16* r = rec + (size_t)i * SKYR_MLP_RECORD;
    float s = 0.f;
    for (int k = 1; k <= 8; ++k) s += __bfloat162float(r[k]);
    bins[i] = error_bin(__bfloat162float(r[0]), s * 0.125f);
}

constexpr int kRenderWarps = 8;              // 2 blocks per SM: one network copy for 8 warps
constexpr int kSmTile = 32 * mlp::kXS * 2;    // records of one warp
constexpr int kSmOut = 32 * 4 * 4;            // network outputs of one warp
constexpr int kSmRender = mlp::kPackedBytes + kRenderWarps * (kSmTile + kSmOut);

template <class S>
__global__ void __launch_bounds__(32 * kRenderWarps, 2) surrogate_render_kernel(CloudConsts C, AtmoConsts A, PtConsts P, Lattice L, Mips M,
                                                                  RenderConsts R, const float4* __restrict__ tlut,
                                                                  int tw, int th, const S* __restrict__ apl,
                                                                  const S* __restrict__ apt,
                                                                  const unsigned char* __restrict__ packed,
                                                                  float4* __restrict__ out,
                                                                  float* __restrict__ out_err) {
    extern __shared__ __align__(16) unsigned char sm[];
    const unsigned full = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ unsigned long long net_bar;
    if (R.use_network && !mlp::load_packed_bulk(sm, packed, &net_bar, P.status, R.copy_wait_cycles)) return;
    __nv_bfloat16* tile = reinterpret_cast<__nv_bfloat16*>(sm + mlp::kPackedBytes + warp * (kSmTile + kSmOut));
    float* yout = reinterpret_cast<float*>(sm + mlp::kPackedBytes + warp * (kSmTile + kSmOut) + kSmTile);
    const int tiles_x = (P.width + 7) / 8;
    const int t_id = blockIdx.x * kRenderWarps + warp;
    const int px = (t_id % tiles_x) * 8 + (lane & 7), py = (t_id / tiles_x) * 4 + (lane >> 3);
    const bool in_view = px < P.width && py < P.height;
    float u, v;
    float3 dir = primary_dir(C, P, min(px, P.width - 1), min(py, P.height - 1), u, v);
    float t0 = 0.f, t1 = 0.f;
    region(P, C.cam, dir, t0, t1);
    bool hit = in_view && t0 < t1;
    const float dt = hit ? (t1 - t0) / (float)R.steps : 0.f;
    uint32_t js = pcg_hash((uint32_t)(py * P.width + px) * 747796405u + 2891336453u);
    const float jitter = (float)(js >> 8) * (1.f / 16777216.f);
    const float mu = dot3(dir, C.sun);
    const float ph = hg_pt(mu, R.g_back) * (1.f - R.ratio) + hg_pt(mu, R.g_fwd) * R.ratio;
    float T = 1.f, err = 0.f, wsum = 0.f, wt = 0.f;
    float3 Lum = f3(0.f);
    uint4* row = reinterpret_cast<uint4*>(tile + lane * mlp::kXS);
    // the ray's optical depth through the region at the march's own samples:
    // the far-side feature of sample s is what remains of it past the sample
    float tau_total = 0.f;
    if (R.use_network && hit) {
        for (int s = 0; s < R.steps; ++s) tau_total += march_sigma(P, R.inv_brick, march_point(C.cam, dir, t0, dt, jitter, s));
        tau_total *= dt;
    }
    float run = 0.f;  // optical depth up to and including the current sample
    for (int s = 0; s < R.steps; ++s) {
        bool live = hit && T > R.min_t;
        if (!__any_sync(full, live)) break;
        float t = fmaf((float)s + jitter, dt, t0);
        float3 x = march_point(C.cam, dir, t0, dt, jitter, s);
        float sigma = live ? march_sigma(P, R.inv_brick, x) : 0.f;
        run = fmaf(sigma, dt, run);
        bool need = live && sigma > 0.f;
        if (!__any_sync(full, need)) continue;
        float tau = 0.f, rel_err = R.network_error;
        float3 ms = f3(0.f);
        if (R.use_network) {
            if (need) {
                const float far_t = __expf(-fmaxf(tau_total - run + 0.5f * sigma * dt, 0.f));
                float f0, near_sun;
                tau = write_record(L, P, M, x, dir, R.nbr, R.inv_ref, far_t, row, f0, near_sun);
                if (R.error_table) rel_err = __ldg(R.error_table + error_bin(f0, near_sun));
            } else {
#pragma unroll
                for (int q = 0; q < kRecQ; ++q) row[q] = make_uint4(0, 0, 0, 0);
            }
            __syncwarp();
            mlp::forward_warp(sm, tile, yout);
            __syncwarp();
            ms = f3(fmaxf(yout[lane * 4], 0.f), fmaxf(yout[lane * 4 + 1], 0.f), fmaxf(yout[lane * 4 + 2], 0.f));
            __syncwarp();
        } else if (need) {
            LatticeCell c;
            lattice_cell(L, x, c);
            tau = lattice_tau(L, c);
        }
        if (need) {
            float3 ss = sun_illuminance(C, A, tlut, tw, th, x) * (ph * __expf(-tau));
            float dT = __expf(-sigma * dt);
            float w = T * (1.f - dT);
            Lum += (ss + ms) * w;
            err += w * (ms.x + ms.y + ms.z) * (1.f / 3.f) * rel_err;
            wsum += w;
            wt += w * t;
            T *= dT;
        }
    }
    if (!in_view) return;
    if (wsum > 0.f) {
        // GetAerialPerspective (VolumetricCloudCommon.glsl:81-98) at the mean depth
        float ta = wt / wsum;
        if (C.atmo_in_space != 0.f) {
            float r = C.R + C.cam.z, rm = r * dir.z;
            float cc = (C.cam.z - A.thickness) * (r + A.top);
            float disc = rm * rm - cc;
            if (dir.z < 0.f && disc >= 0.f) ta -= fmaxf(cc / (-rm + sqrtf(disc)), 0.f);
            else ta = 0.f;
        }
        float wz = sqrtf(fmaxf(ta, 0.f) * C.inv_ap_max_distance);
        float ax = u * (float)(C.ap_w - 1), ay = v * (float)(C.ap_h - 1), az = wz * (float)(C.ap_d - 1);
        float3 at = trilinear_clamp(apt, C.ap_w, C.ap_h, C.ap_d, ax, ay, az);
        float3 al = trilinear_clamp(apl, C.ap_w, C.ap_h, C.ap_d, ax, ay, az);
        al = al * froxel_visibility(C, u, v, wt / wsum);
        Lum = Lum * at + al * (1.f - T);
    }
    size_t pix = (size_t)py * P.width + px;
    out[pix] = make_float4(Lum.x, Lum.y, Lum.z, T);
    if (out_err) out_err[pix] = err;
}

// Launch constants of a grid: the PtConsts grid fields and the grid box.
int grid_setup(const skyr_density_grid* grid, PtConsts& P, GridBox& B) {
    if (!grid || !grid->data) return set_error(SKYR_EINVAL, "null density grid");
    if (grid->nx < 2 || grid->ny < 2 || grid->nz < 2 || !(grid->voxel_size > 0.f) ||
        !std::isfinite(grid->density) || grid->density < 0.f || !std::isfinite(grid->origin[0]) ||
        !std::isfinite(grid->origin[1]) || !std::isfinite(grid->origin[2]))
        return set_error(SKYR_EINVAL, "bad density grid");
    std::memset(&P, 0, sizeof(P));
    P.tracking_steps = skyr_ctx{}.limits.tracking_steps;
    P.grid = reinterpret_cast<const unsigned short*>(grid->data);
    P.nx = grid->nx;
    P.ny = grid->ny;
    P.nz = grid->nz;
    P.origin = make_float3(grid->origin[0], grid->origin[1], grid->origin[2]);
    P.inv_voxel = 1.f / grid->voxel_size;
    P.density = grid->density;
    if (grid->majorant && grid->brick >= 1) {  // the brick majorants, when the grid carries them
        P.maj = grid->majorant;
        P.bx = skyr_grid_brick_count(grid->nx, grid->brick);
        P.by = skyr_grid_brick_count(grid->ny, grid->brick);
        P.bz = skyr_grid_brick_count(grid->nz, grid->brick);
        P.brick_size = grid->voxel_size * (float)grid->brick;
    }
    B.lo = P.origin;
    B.hi = make_float3(grid->origin[0] + grid->nx * grid->voxel_size, grid->origin[1] + grid->ny * grid->voxel_size,
                       grid->origin[2] + grid->nz * grid->voxel_size);
    B.span = grid->voxel_size * (float)std::max(grid->nx, std::max(grid->ny, grid->nz));
    return SKYR_OK;
}

// Bytes of a lattice of `nodes` nodes over `grid`: the records, the sun optical
// depths, then the grid's mip levels 1..kMipLevels (each 256-byte aligned).
// With M: the levels' sizes and texel sizes, and their addresses in the buffer
// that starts at `base`; level 0 is the grid itself.
size_t lattice_bytes(const skyr_density_grid* grid, size_t nodes, Mips* M = nullptr,
                     const unsigned char* base = nullptr) {
    size_t off = nodes * (kLatQ * 16 + 4);
    int nx = grid->nx, ny = grid->ny, nz = grid->nz;
    if (M) {
        M->level[0] = MipLevel{reinterpret_cast<const unsigned short*>(grid->data), nx, ny, nz,
                               1.f / grid->voxel_size};
        M->voxel = grid->voxel_size;
    }
    for (int l = 1; l <= kMipLevels; ++l) {
        off = (off + 255) & ~(size_t)255;
        nx = (nx + 1) / 2, ny = (ny + 1) / 2, nz = (nz + 1) / 2;
        if (M)
            M->level[l] = MipLevel{reinterpret_cast<const unsigned short*>(base + off), nx, ny, nz,
                                   1.f / (grid->voxel_size * (float)(1 << l))};
        off += (size_t)nx * ny * nz * 2;
    }
    return off;
}

// The mip chain in a lattice's buffer.
Mips lattice_mips(const skyr_density_grid* grid, const skyr_feature_volume* fv) {
    Mips M;
    lattice_bytes(grid, (size_t)fv->nx * fv->ny * fv->nz, &M, reinterpret_cast<const unsigned char*>(fv->data));
    return M;
}

int lattice_setup(const skyr_density_grid* grid, const skyr_feature_volume* fv, Lattice& L) {
    if (!fv || !fv->data) return set_error(SKYR_EINVAL, "null feature lattice");
    if (fv->stride < 1 || fv->nx < 2 || fv->ny < 2 || fv->nz < 2)
        return set_error(SKYR_EINVAL, "feature lattice not sized (skyr_feature_volume_bytes)");
    if (fv->nx != (grid->nx + fv->stride - 1) / fv->stride + 1 || fv->ny != (grid->ny + fv->stride - 1) / fv->stride + 1 ||
        fv->nz != (grid->nz + fv->stride - 1) / fv->stride + 1)
        return set_error(SKYR_EINVAL, "feature lattice does not match the grid");
    if (reinterpret_cast<uintptr_t>(fv->data) & 15) return set_error(SKYR_EINVAL, "feature lattice must be 16-byte aligned");
    size_t nodes = (size_t)fv->nx * fv->ny * fv->nz;
    L.rec = reinterpret_cast<const uint4*>(fv->data);
    L.tau = reinterpret_cast<const float*>(reinterpret_cast<const unsigned char*>(fv->data) + nodes * kLatQ * 16);
    L.nx = fv->nx;
    L.ny = fv->ny;
    L.nz = fv->nz;
    L.origin = make_float3(grid->origin[0], grid->origin[1], grid->origin[2]);
    L.inv_cell = 1.f / (grid->voxel_size * (float)fv->stride);
    L.sun = make_float3(fv->sun[0], fv->sun[1], fv->sun[2]);
    return SKYR_OK;
}

int frame_consts(const skyr_atmosphere_parameters* atmosphere, const skyr_cloud_parameters* cloud,
                 const skyr_cloud_view* view, const skyr_lut_sizes* sizes, CloudConsts& C, AtmoConsts& A) {
    skyr_cloud_material mat;
    skyr_cloud_material_default(SKYR_MATERIAL_MINIMAL, &mat);
    skyr_cloud_textures tex{};
    MaterialConsts M;
    if (int st = derive_cloud_consts(*atmosphere, *cloud, mat, tex, *view, *sizes, C, M)) return st;
    derive_atmo_consts(*atmosphere, A);
    return SKYR_OK;
}

}  // namespace
}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_surrogate_parameters_default(skyr_surrogate_parameters* p) {
    if (!p) return set_error(SKYR_EINVAL, "null parameters");
    p->steps = 128;
    p->use_network = 1;
    p->network_error = 0.05f;
    p->min_transmittance = 1e-4f;
    p->error_table = nullptr;
    return SKYR_OK;
}

size_t skyr_feature_volume_bytes(const skyr_density_grid* grid, int stride, skyr_feature_volume* fv) {
    if (!grid || stride < 1 || grid->nx < 2 || grid->ny < 2 || grid->nz < 2) return 0;
    int nx = (grid->nx + stride - 1) / stride + 1, ny = (grid->ny + stride - 1) / stride + 1,
        nz = (grid->nz + stride - 1) / stride + 1;
    if (fv) {
        fv->stride = stride;
        fv->nx = nx;
        fv->ny = ny;
        fv->nz = nz;
    }
    return lattice_bytes(grid, (size_t)nx * ny * nz);
}

int skyr_feature_volume_build(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                              const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                              const skyr_cloud_view* view, skyr_feature_volume* fv) {
    if (!ctx || !atmosphere || !cloud || !grid || !view || !fv) return set_error(SKYR_EINVAL, "null argument");
    if (!(fv->sigma_ref > 0.f) || !std::isfinite(fv->sigma_ref)) return set_error(SKYR_EINVAL, "bad sigma_ref");
    PtConsts P;
    GridBox B;
    if (int e = grid_setup(grid, P, B)) return e;
    if (skyr_feature_volume_bytes(grid, fv->stride, fv) == 0) return set_error(SKYR_EINVAL, "bad lattice stride");
    skyr_lut_sizes sizes{};
    sizes.transmittance_width = sizes.transmittance_height = 2;
    sizes.aerial_perspective_width = sizes.aerial_perspective_height = sizes.aerial_perspective_depth = 2;
    CloudConsts C;
    AtmoConsts A;
    if (int e = frame_consts(atmosphere, cloud, view, &sizes, C, A)) return e;
    fv->sun[0] = C.sun.x;
    fv->sun[1] = C.sun.y;
    fv->sun[2] = C.sun.z;
    Lattice L;
    if (int e = lattice_setup(grid, fv, L)) return e;
    LatticeBuild Q;
    for (int k = 0; k < kSun; ++k) Q.dist[k] = B.span * 0.01f * (float)std::pow(1000.0, k / 31.0);
    Q.nbr = 0.1f * B.span;
    Q.inv_sigma_ref = 1.f / fv->sigma_ref;
    Q.step = 0.5f * grid->voxel_size;
    // the stencil's axes: the sun, its perpendicular in the horizontal plane
    // (sun x z; sun x x when the sun is at the zenith), and their cross product
    {
        double e1[3] = {C.sun.x, C.sun.y, C.sun.z};
        double n1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (double& v : e1) v /= n1;
        double e2[3] = {e1[1], -e1[0], 0.0};  // e1 x z
        double n2 = std::sqrt(e2[0] * e2[0] + e2[1] * e2[1]);
        if (n2 < 1e-3) {
            e2[0] = 0.0, e2[1] = e1[2], e2[2] = -e1[1];  // e1 x x
            n2 = std::sqrt(e2[1] * e2[1] + e2[2] * e2[2]);
        }
        for (double& v : e2) v /= n2;
        double e3[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        Q.axis[0] = make_float3((float)e1[0], (float)e1[1], (float)e1[2]);
        Q.axis[1] = make_float3((float)e2[0], (float)e2[1], (float)e2[2]);
        Q.axis[2] = make_float3((float)e3[0], (float)e3[1], (float)e3[2]);
    }
    for (int l = 0; l < kStencilLevels; ++l)
        Q.spacing[l] = grid->voxel_size * (float)(2 << (kStencilFirst + l));
    Q.inv_brick = P.maj ? 1.f / P.brick_size : 0.f;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    // the mip chain of the grid, in the lattice's buffer after the optical depths
    const Mips M = lattice_mips(grid, fv);
    size_t nodes = (size_t)L.nx * L.ny * L.nz;
    for (int l = 1; l <= kMipLevels; ++l) {
        size_t n = (size_t)M.level[l].nx * M.level[l].ny * M.level[l].nz;
        mip_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            M.level[l - 1], M.level[l], const_cast<unsigned short*>(M.level[l].data));
        if (int e = check_cuda(cudaGetLastError(), "mip reduce kernel")) return e;
    }
    feature_lattice_kernel<<<(unsigned)((nodes + 127) / 128), 128, 0, ctx->stream>>>(
        P, B, L, Q, M, fv->stride, reinterpret_cast<uint4*>(fv->data), const_cast<float*>(L.tau));
    return check_cuda(cudaGetLastError(), "feature lattice kernel");
}

int skyr_surrogate_sample_points(skyr_ctx* ctx, const skyr_density_grid* grid, float sigma_max, float sigma_min,
                                 uint64_t seed, int n, float* points) {
    if (!ctx || !grid || (n > 0 && !points)) return set_error(SKYR_EINVAL, "null argument");
    if (n < 0) return set_error(SKYR_EINVAL, "negative point count");
    if (!(sigma_max >= 0.f) || !std::isfinite(sigma_max) || !std::isfinite(sigma_min))
        return set_error(SKYR_EINVAL, "bad extinction bounds");
    PtConsts P;
    GridBox B;
    if (int e = grid_setup(grid, P, B)) return e;
    if (n == 0) return SKYR_OK;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    sample_points_kernel<<<(n + 127) / 128, 128, 0, ctx->stream>>>(P, B, sigma_max, sigma_min, (uint32_t)seed,
                                                                  (uint32_t)(seed >> 32), n, points);
    return check_cuda(cudaGetLastError(), "sample points kernel");
}

int skyr_surrogate_records(skyr_ctx* ctx, const skyr_density_grid* grid, const skyr_feature_volume* fv,
                           const float* points, int n, uint16_t* records) {
    if (!ctx || !grid || (n > 0 && (!points || !records))) return set_error(SKYR_EINVAL, "null argument");
    if (n < 0) return set_error(SKYR_EINVAL, "negative point count");
    if (reinterpret_cast<uintptr_t>(records) & 15) return set_error(SKYR_EINVAL, "records must be 16-byte aligned");
    PtConsts P;
    GridBox B;
    if (int e = grid_setup(grid, P, B)) return e;
    Lattice L;
    if (int e = lattice_setup(grid, fv, L)) return e;
    if (n == 0) return SKYR_OK;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    records_kernel<<<(n + 127) / 128, 128, 0, ctx->stream>>>(L, P, B, lattice_mips(grid, fv), 0.1f * B.span,
                                                           1.f / fv->sigma_ref,
                                                           0.5f * grid->voxel_size, points, n,
                                                           reinterpret_cast<uint4*>(records));
    return check_cuda(cudaGetLastError(), "records kernel");
}

int skyr_surrogate_error_bins(skyr_ctx* ctx, const uint16_t* records, int n, int* bins) {
    if (!ctx || (n > 0 && (!records || !bins))) return set_error(SKYR_EINVAL, "null argument");
    if (n < 0) return set_error(SKYR_EINVAL, "negative record count");
    if (n == 0) return SKYR_OK;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    error_bins_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(reinterpret_cast<const __nv_bfloat16*>(records), n,
                                                                bins);
    return check_cuda(cudaGetLastError(), "error bins kernel");
}

int skyr_surrogate_render(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_lut_sizes* sizes, const void* transmittance,
                          const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                          const skyr_feature_volume* fv, const void* packed, const skyr_surrogate_parameters* sp,
                          float* out_rgba, float* out_error) {
    if (!ctx || !atmosphere || !cloud || !grid || !pt || !view || !sizes || !sp || !out_rgba)
        return set_error(SKYR_EINVAL, "null argument");
    if (!transmittance || !aerial_perspective_luminance || !aerial_perspective_transmittance)
        return set_error(SKYR_EINVAL, "null LUT input");
    if (sp->steps < 1 || sp->steps > 4096) return set_error(SKYR_EINVAL, "steps must be in [1, 4096]");
    if (sp->use_network && !packed) return set_error(SKYR_EINVAL, "network requested but none given");
    if (packed && (reinterpret_cast<uintptr_t>(packed) & 15))
        return set_error(SKYR_EINVAL, "packed network must be 16-byte aligned");
    if (!(std::fabs(pt->forward_phase_g) < 1.f) || !(std::fabs(pt->back_phase_g) < 1.f) ||
        !(pt->forward_scattering_ratio >= 0.f && pt->forward_scattering_ratio <= 1.f))
        return set_error(SKYR_EINVAL, "phase parameters out of range");
    if (view->width < 1 || view->height < 1 || view->width > 16384 || view->height > 16384)
        return set_error(SKYR_EINVAL, "render size must be in [1, 16384]");
    if (sizes->aerial_perspective_width < 2 || sizes->aerial_perspective_height < 2 ||
        sizes->aerial_perspective_depth < 2 || sizes->transmittance_width < 2 || sizes->transmittance_height < 2)
        return set_error(SKYR_EINVAL, "LUT sizes must be >= 2");
    PtConsts P;
    GridBox B;
    if (int e = grid_setup(grid, P, B)) return e;
    Lattice L;
    if (int e = lattice_setup(grid, fv, L)) return e;
    CloudConsts C;
    AtmoConsts A;
    if (int e = frame_consts(atmosphere, cloud, view, sizes, C, A)) return e;
    // the region box of the path tracer, clipped to the grid
    float hw = pt->region_box_half_width;
    P.box_min = make_float3(fmaxf(-hw, B.lo.x), fmaxf(-hw, B.lo.y), fmaxf(C.bottom, B.lo.z));
    P.box_max = make_float3(fminf(hw, B.hi.x), fminf(hw, B.hi.y), fminf(C.top, B.hi.z));
    P.width = view->width;
    P.height = view->height;
    // bounded waits in the kernel (the network's bulk copy) report here
    if (int e = ensure_status(ctx)) return e;
    P.status = ctx->d_status;
    RenderConsts R;
    R.copy_wait_cycles = ctx->limits.copy_wait_cycles;
    R.steps = sp->steps;
    R.use_network = sp->use_network ? 1 : 0;
    R.network_error = sp->network_error;
    R.min_t = sp->min_transmittance;
    R.g_fwd = pt->forward_phase_g;
    R.g_back = pt->back_phase_g;
    R.ratio = pt->forward_scattering_ratio;
    R.error_table = sp->error_table;
    R.nbr = 0.1f * B.span;
    R.inv_ref = 1.f / fv->sigma_ref;
    R.inv_brick = P.maj ? 1.f / P.brick_size : 0.f;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    const Mips mips = lattice_mips(grid, fv);
    auto launch = [&](auto tag) -> int {
        using S = decltype(tag);
        auto kernel = surrogate_render_kernel<S>;
        const int use_smem = kSmRender;  // the network slot stays reserved when it is unused
        if (int e = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, use_smem),
                               "surrogate smem attribute"))
            return e;
        int tiles = ((view->width + 7) / 8) * ((view->height + 3) / 4);
        kernel<<<(tiles + kRenderWarps - 1) / kRenderWarps, 32 * kRenderWarps, use_smem, ctx->stream>>>(
            C, A, P, L, mips, R, reinterpret_cast<const float4*>(transmittance), sizes->transmittance_width,
            sizes->transmittance_height, reinterpret_cast<const S*>(aerial_perspective_luminance),
            reinterpret_cast<const S*>(aerial_perspective_transmittance),
            reinterpret_cast<const unsigned char*>(packed), reinterpret_cast<float4*>(out_rgba), out_error);
        return check_cuda(cudaGetLastError(), "surrogate render kernel");
    };
    return sizes->format == SKYR_FORMAT_RGBA16F ? launch(__half2{}) : launch(float4{});
}

}  // extern "C"
