// pathtrace.cu — the volumetric-cloud path tracer
// (VolumetricCloudPathTracing.comp) for sm_103a, the synthetic dense FP16
// density grid and its 16^3-brick majorant grid.
//
// A persistent kernel traces one path per (frame, pixel) work item with path
// regeneration.  The path logic follows the reference (delta tracking,
// ratio-tracking next-event estimation with a copied RNG context, HG importance
// sampling, the Lambert ground bounce, the environment on escape).  Two
// GB300-side changes:
//  * a dense FP16 grid with per-brick majorants walked by a 3D DDA replaces the
//    single global majorant where the caller supplies them, so empty and thin
//    regions cost few samples;
//  * the environment is the sky-view LUT + ground term evaluated per direction
//    (the math of ENVIRONMENT_LUMINANCE) instead of a pre-baked cube map.
#include <cmath>
#include <cstring>

#include "../../include/skyr_pathtrace.h"
#include "atmosphere_kernels.cuh"
#include "cloud_internal.cuh"
#include "cloud_material.cuh"
#include "environment.cuh"
#include "lut_access.cuh"
#include "noise_device.cuh"
#include "skyr_ctx.cuh"
#include "voxel_device.cuh"

namespace skyr {

// The material plug-ins' SampleSigmaT with the path tracer's flat height01.
// Kept out of line: it holds every material's texture sampling, and the dense
// grid is the path tracer's fast path.
__device__ __noinline__ float material_sigma(const CloudConsts& C, const MaterialConsts& M, float3 p) {
    float h01 = clamp01((p.z - C.bottom) * C.inv_layer);
    float3 dc = p - C.cam;
    return sigma_t(C, M, p, h01, sqrtf(dot3(dc, dc)));
}

// SampleSigmaT(vec3 P) of the path tracer (PathTracing.comp:89-91)
__device__ __forceinline__ float pt_sigma(const PtConsts& P, const CloudConsts& C, const MaterialConsts& M,
                                          float3 p) {
    if (P.grid) return grid_sigma(P, p);
    return material_sigma(C, M, p);
}

// 3D DDA over the majorant bricks
struct Walk {
    int i[3], s[3];
    float tmax[3], tdel[3];
};

__device__ __forceinline__ void walk_init(const PtConsts& P, Walk& w, float3 o, float3 d, float t) {
    float bs = P.brick_size;
    float p[3] = {o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
    float og[3] = {P.origin.x, P.origin.y, P.origin.z};
    float dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        w.i[a] = (int)floorf((p[a] - og[a]) / bs);
        if (dd[a] > 0.f) {
            w.s[a] = 1;
            w.tmax[a] = t + (og[a] + (float)(w.i[a] + 1) * bs - p[a]) / dd[a];
            w.tdel[a] = bs / dd[a];
        } else if (dd[a] < 0.f) {
            w.s[a] = -1;
            w.tmax[a] = t + (og[a] + (float)w.i[a] * bs - p[a]) / dd[a];
            w.tdel[a] = -bs / dd[a];
        } else {
            w.s[a] = 0;
            w.tmax[a] = 1e30f;
            w.tdel[a] = 1e30f;
        }
    }
}
__device__ __forceinline__ float walk_exit(const Walk& w) { return fminf(w.tmax[0], fminf(w.tmax[1], w.tmax[2])); }
__device__ __forceinline__ void walk_step(Walk& w) {
    int a = w.tmax[0] <= w.tmax[1] ? (w.tmax[0] <= w.tmax[2] ? 0 : 2) : (w.tmax[1] <= w.tmax[2] ? 1 : 2);
    // constant indices keep the walk in registers
    if (a == 0) { w.i[0] += w.s[0]; w.tmax[0] += w.tdel[0]; }
    else if (a == 1) { w.i[1] += w.s[1]; w.tmax[1] += w.tdel[1]; }
    else { w.i[2] += w.s[2]; w.tmax[2] += w.tdel[2]; }
}
// The walk runs inside the region box, which lies within the grid; an index
// one brick outside can only come from rounding at the box faces and takes the
// majorant of the boundary brick.
__device__ __forceinline__ float walk_majorant(const PtConsts& P, const Walk& w) {
    int i = min(max(w.i[0], 0), P.bx - 1), j = min(max(w.i[1], 0), P.by - 1), k = min(max(w.i[2], 0), P.bz - 1);
    return __ldg(P.maj + ((size_t)k * P.by + j) * P.bx + i);
}

// Exponential optical depth of one majorant collision: -log(1 - xi)
__device__ __forceinline__ float sample_tau(const PtConsts& P, uint32_t& seed) {
    return -logf(1.f - rand01(P, seed));
}

// free flight in [t, t_max] (delta tracking); true on a collision
__device__ __forceinline__ bool free_flight(const PtConsts& P, const CloudConsts& C, const MaterialConsts& M,
                                            uint32_t& seed, float3 o, float3 d, float& t, float t_max) {
    if (!P.use_bricks) {
        float smax = P.sigma_t_max;
        for (int it = 0; it < P.tracking_steps; ++it) {
            if (smax <= 0.f) return false;
            t += -logf(1.f - rand01(P, seed)) / smax;
            if (!(t <= t_max)) return false;
            float s = pt_sigma(P, C, M, o + d * t);
            if (rand01(P, seed) < s / smax) return true;
        }
        flag_overrun(P);
        return false;
    }
    // Piecewise-constant majorant: one exponential optical depth per tentative
    // collision, spent brick by brick (tau -= m * length), so a brick crossing
    // costs no logarithm.  The brick steps form their own inner loop, so that
    // the lanes of a warp run the density evaluation together.
    Walk w;
    walk_init(P, w, o, d, t);
    float tau = sample_tau(P, seed);
    int it = 0;
    for (;;) {
        float m;
        for (;;) {
            if (++it > P.tracking_steps) {
                flag_overrun(P);
                return false;
            }
            float te = fminf(walk_exit(w), t_max);
            m = walk_majorant(P, w);
            float seg = (te - t) * m;
            if (tau < seg) break;
            tau -= seg;
            t = te;
            if (!(t < t_max)) return false;
            walk_step(w);
        }
        t += tau / m;
        float s = pt_sigma(P, C, M, o + d * t);
        if (rand01(P, seed) < s / m) return true;
        tau = sample_tau(P, seed);
    }
}

// TransmittanceEstimation (PathTracing.comp:135-151): ratio tracking with a
// copy of the RNG state
__device__ __forceinline__ float transmittance_estimation(const PtConsts& P, const CloudConsts& C,
                                                          const MaterialConsts& M, uint32_t seed, float3 o,
                                                          float3 d) {
    float tr = 1.f;
    float t0, t1;
    region(P, o, d, t0, t1);
    if (t0 >= t1) return tr;
    float t = t0;
    if (!P.use_bricks) {
        float smax = P.sigma_t_max;
        for (int it = 0;; ++it) {
            if (it >= P.tracking_steps) {
                flag_overrun(P);
                break;
            }
            t += -logf(1.f - rand01(P, seed)) / smax;
            if (!(t <= t1)) break;
            float s = pt_sigma(P, C, M, o + d * t);
            tr *= 1.f - fmaxf(0.f, s / smax);
        }
        return clamp01(tr);
    }
    Walk w;
    walk_init(P, w, o, d, t);
    float tau = sample_tau(P, seed);
    int it = 0;
    for (;;) {
        float m;
        bool done = false;
        for (;;) {
            if (++it > P.tracking_steps) {
                flag_overrun(P);
                done = true;
                break;
            }
            float te = fminf(walk_exit(w), t1);
            m = walk_majorant(P, w);
            float seg = (te - t) * m;
            if (tau < seg) break;
            tau -= seg;
            t = te;
            if (!(t < t1)) {
                done = true;
                break;
            }
            walk_step(w);
        }
        if (done) break;
        t += tau / m;
        tr *= 1.f - fmaxf(0.f, pt_sigma(P, C, M, o + d * t) / m);
        tau = sample_tau(P, seed);
    }
    return clamp01(tr);
}

// Work items of one frame: the region in 8x4 pixel tiles, 32 items per tile
// (items past the region's right / bottom edge are skipped).
__device__ __forceinline__ bool item_pixel(const PtConsts& P, int item, int& px, int& py) {
    if (P.pixel_list) {  // out-of-range entries are skipped
        int pix = __ldg(P.pixel_list + item);
        px = pix % P.width;
        py = pix / P.width;
        return pix >= 0 && py < P.height;
    }
    int tile = item >> 5, k = item & 31;
    px = P.x0 + (tile % P.tiles_x) * 8 + (k & 7);
    py = P.y0 + (tile / P.tiles_x) * 4 + (k >> 3);
    return px < P.x1 && py < P.y1;
}

// One path of Trace (PathTracing.comp:160-249) in flight on one lane.
struct PathState {
    float3 o, d, L, thr;
    uint32_t seed;
    int px, py, istep;
    float scattered_t;
    bool scattered;
};

// Sample of a finished path: GetAerialPerspective (VolumetricCloudCommon.glsl:
// 81-98) at the first scattering distance; a = 1 when the path never scattered.
template <class S>
__device__ __forceinline__ float4 path_sample(const CloudConsts& C, const AtmoConsts& A, const PtConsts& P,
                                              const S* apl, const S* apt, const PathState& ps) {
    float u, v;
    float3 view = primary_dir(C, P, ps.px, ps.py, u, v);
    float3 L = ps.L;
    if (ps.scattered) {
        float ta = ps.scattered_t;
        float mu = view.z;
        if (C.atmo_in_space != 0.f) {
            float r = C.R + C.cam.z, rm = r * mu;
            float cc = (C.cam.z - A.thickness) * (r + A.top);
            float disc = rm * rm - cc;
            if (mu < 0.f && disc >= 0.f) ta -= fmaxf(cc / (-rm + sqrtf(disc)), 0.f);
            else ta = 0.f;
        }
        float wz = sqrtf(fmaxf(ta, 0.f) * C.inv_ap_max_distance);
        float ax = u * (float)(C.ap_w - 1), ay = v * (float)(C.ap_h - 1), az = wz * (float)(C.ap_d - 1);
        float3 at = trilinear_clamp(apt, C.ap_w, C.ap_h, C.ap_d, ax, ay, az);
        float3 al = trilinear_clamp(apl, C.ap_w, C.ap_h, C.ap_d, ax, ay, az);
        al = al * froxel_visibility(C, u, v, ps.scattered_t);  // PathTracing.comp:277
        L = L * at + al;
    }
    return make_float4(L.x, L.y, L.z, ps.scattered ? 0.f : 1.f);
}

// Start the path of pixel (px, py) for `frame`; false when it ends at once
// (the view ray misses the cloud region, or no bounces are allowed).
__device__ __forceinline__ bool start_path(const CloudConsts& C, const PtConsts& P, unsigned frame, PathState& ps) {
    ps.seed = pt_prng(P, pt_prng(P, pt_prng(P, (uint32_t)ps.px) + (uint32_t)ps.py) + frame);
    float u, v;
    ps.d = primary_dir(C, P, ps.px, ps.py, u, v);
    ps.L = f3(0.f);
    ps.thr = f3(1.f);
    ps.scattered = false;
    ps.scattered_t = 0.f;
    ps.istep = 0;
    float c0, c1;
    region(P, C.cam, ps.d, c0, c1);
    ps.o = C.cam + ps.d * c0;
    return c0 < c1 && P.max_bounces > 0;
}

// New direction after a scattering event at ps.o: GenerateHGSample
// (PathTracing.comp:98-117) with importance sampling, else a uniform sphere
// direction weighted by the phase function.
__device__ __forceinline__ void sample_scatter(const PtConsts& P, PathState& ps) {
    float3 d = ps.d;
    if (P.importance_sampling) {
        float g = rand01(P, ps.seed) < P.ratio ? P.g_fwd : P.g_back;
        float xi = rand01(P, ps.seed);
        float opg = 1.f + g * g, omg = 1.f - g * g, o2g = 0.5f / g;
        float tt = omg / (1.f - g + 2.f * g * xi);
        float ct = o2g * (opg - tt * tt);
        float st = sqrtf(clamp01(1.f - ct * ct));
        float3 b0, b1;
        onb(d, b0, b1);
        float sp, cp;
        sincosf(2.f * SKYR_PI * rand01(P, ps.seed), &sp, &cp);
        ps.d = b0 * (st * sp) + b1 * (st * cp) + d * ct;
    } else {
        float phi = 2.f * SKYR_PI * rand01(P, ps.seed);
        float c = 1.f - 2.f * rand01(P, ps.seed);
        float s = sqrtf(clamp01(1.f - c * c));
        float sp, cp;
        sincosf(phi, &sp, &cp);
        float3 nd = f3(cp * s, sp * s, c);
        float cn = dot3(d, nd);
        float val = hg_pt(cn, P.g_back) * (1.f - P.ratio) + hg_pt(cn, P.g_fwd) * P.ratio;
        ps.thr = ps.thr * (val * 4.f * SKYR_PI);
        ps.d = nd;
    }
}

// Path of a point source: it starts at points[i] with a direction drawn from
// the phase function about the point's direction, as if a path travelling
// along it had just scattered there (that event counts as the first bounce).
__device__ __forceinline__ bool start_point_path(const PtConsts& P, unsigned frame, int i, PathState& ps) {
    ps.px = i;
    ps.py = 0;
    ps.seed = pt_prng(P, pt_prng(P, pt_prng(P, (uint32_t)i) + 0x2545F491u) + frame);
    const float* q = P.points + 6 * (size_t)i;
    ps.o = f3(__ldg(q), __ldg(q + 1), __ldg(q + 2));
    ps.d = f3(__ldg(q + 3), __ldg(q + 4), __ldg(q + 5));
    ps.L = f3(0.f);
    ps.thr = f3(1.f);
    ps.scattered = true;
    ps.scattered_t = 0.f;
    ps.istep = 1;
    sample_scatter(P, ps);
    return P.max_bounces > 1;
}

// One iteration of Trace's bounce loop; false when the path ends.
template <class S>
__device__ __forceinline__ bool bounce(const CloudConsts& C, const MaterialConsts& M, const AtmoConsts& A,
                                       const PtConsts& P, const ViewConsts& E, const float4* tlut, int tw, int th,
                                       const S* svl, const S* svt, PathState& ps) {
    float t0, t1;
    region(P, ps.o, ps.d, t0, t1);
    if (t0 >= t1) return false;
    float t = t0;
    bool scatter = free_flight(P, C, M, ps.seed, ps.o, ps.d, t, t1);
    if (!scatter) {
        if (P.env == SKYR_ENV_OFF || !ps.scattered) return false;
        if (P.env == SKYR_ENV_CONST_ENVIRONMENT_MAP) {
            float3 wd = P.m_front * ps.d.x + P.m_right * ps.d.y + P.m_up * ps.d.z;
            ps.L += ps.thr * environment(A, E, tlut, tw, th, svl, svt, P.sv_w, P.sv_h, wd);
            return false;
        }
        float3 o = ps.o, d = ps.d;
        float rho2 = fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * (o.z + 2.f * C.R)));
        float r = sqrtf(fmaf(C.R, C.R, rho2));
        float mu = fmaf(d.x, o.x, fmaf(d.y, o.y, d.z * (o.z + C.R))) / r;
        if (!ray_hits_ground(r, rho2, mu)) {
            float3 wd = P.m_front * d.x + P.m_right * d.y + P.m_up * d.z;
            ps.L += ps.thr * environment(A, E, tlut, tw, th, svl, svt, P.sv_w, P.sv_h, wd);
            return false;
        }
        o = o + d * dist_to_bottom(r, rho2, mu);
        float3 n = f3(o.x, o.y, o.z + C.R);
        n = n * rsqrtf(dot3(n, n));
        float ndl = dot3(n, C.sun);
        float3 bsdf = A.ground_albedo * (1.f / SKYR_PI);
        ps.L += ps.thr * (sun_illuminance(C, A, tlut, tw, th, o) * (bsdf * ndl) *
                          transmittance_estimation(P, C, M, ps.seed, o, C.sun));
        if (P.env == SKYR_ENV_GROUND_SINGLE_BOUNCE) return false;
        // GenerateLambertSample (PathTracing.comp:119-129)
        float st = sqrtf(rand01(P, ps.seed));
        float ct = sqrtf(clamp01(1.f - st * st));
        float3 b0, b1;
        onb(n, b0, b1);
        float sp, cp;
        sincosf(2.f * SKYR_PI * rand01(P, ps.seed), &sp, &cp);
        ps.o = o;
        ps.d = b0 * (st * sp) + b1 * (st * cp) + n * ct;
        ps.thr *= A.ground_albedo;
    } else {
        if (!ps.scattered) {
            float3 dc = C.cam - ps.o;
            ps.scattered_t = sqrtf(dot3(dc, dc));
        }
        ps.scattered = true;
        ps.o = ps.o + ps.d * t;
        float3 d = ps.d;
        float cs = dot3(d, C.sun);
        float ph = hg_pt(cs, P.g_back) * (1.f - P.ratio) + hg_pt(cs, P.g_fwd) * P.ratio;
        ps.L += ps.thr * (sun_illuminance(C, A, tlut, tw, th, ps.o) *
                          (ph * transmittance_estimation(P, C, M, ps.seed, ps.o, C.sun)));
        sample_scatter(P, ps);
    }
    ++ps.istep;
    return ps.istep < P.max_bounces && fmaxf(ps.thr.x, fmaxf(ps.thr.y, ps.thr.z)) > 0.f;
}

// Persistent path tracer with path regeneration.  A work item is one path:
// (frame, pixel) in frame-major order.  A warp takes kWarpChunk items at a
// time from the call's counter, and a lane whose path has ended starts the next
// item of its warp's chunk at the top of the next bounce iteration, so lanes do
// not idle behind the warp's longest path and the SMs stay full until the
// call's items run out.  Samples are added to the accumulation buffers with
// float atomics: the frames of one call may be summed in any order (the sums
// agree to rounding, not bit for bit, between runs).
constexpr int kWarpChunk = 32;

template <class S>
__device__ __forceinline__ void deposit(const CloudConsts& C, const AtmoConsts& A, const PtConsts& P, const S* apl,
                                        const S* apt, const PathState& ps, float4* acc, float4* acc_sq) {
    if (P.points) {  // point source: the radiance of the path, no aerial perspective
        float* o = P.point_out + 3 * (size_t)ps.px;
        atomicAdd(o, ps.L.x);
        atomicAdd(o + 1, ps.L.y);
        atomicAdd(o + 2, ps.L.z);
        return;
    }
    float4 x = path_sample(C, A, P, apl, apt, ps);
    size_t pix = (size_t)ps.py * P.width + ps.px;
    atomicAdd(acc + pix, x);
    if (acc_sq) atomicAdd(acc_sq + pix, make_float4(x.x * x.x, x.y * x.y, x.z * x.z, x.w * x.w));
}

// Registers are cut for 6 resident blocks per SM (80 registers, ~200 B spilled,
// from 116 at 4 blocks): the random density fetches are latency-bound and the
// extra warps hide more of it (16 frames of 1024^2: 31.7 -> 28.9 ms on a
// GB300; 8 blocks lose, 450 B spilled).  Short jobs lose a little instead (4
// frames of 512^2: 3.10 -> 3.23 ms).  The persistent grid follows from the
// occupancy query.
template <class S>
__global__ void __launch_bounds__(128, 6) pathtrace_kernel(CloudConsts C, MaterialConsts M, AtmoConsts A,
                                                           PtConsts P, ViewConsts E,
                                                           const float4* __restrict__ tlut, int tw, int th,
                                                           const S* __restrict__ svl, const S* __restrict__ svt,
                                                           const S* __restrict__ apl, const S* __restrict__ apt,
                                                           unsigned frame_begin, int n_frames,
                                                           int* __restrict__ counter, float4* __restrict__ acc,
                                                           float4* __restrict__ acc_sq) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int n_total = P.n_items * n_frames;
    int chunk_next = 0, chunk_end = 0;  // warp-uniform
    bool exhausted = false;             // warp-uniform
    bool active = false;
    PathState ps;
    ps.px = ps.py = 0;
    for (;;) {
        // hand the warp's next items to idle lanes
        unsigned idle = __ballot_sync(full, !active);
        while (idle && !exhausted) {
            if (chunk_next >= chunk_end) {
                int base = 0;
                if (lane == 0) base = atomicAdd(counter, kWarpChunk);
                base = __shfl_sync(full, base, 0);
                if (base >= n_total) {
                    exhausted = true;
                    break;
                }
                chunk_next = base;
                chunk_end = min(base + kWarpChunk, n_total);
            }
            int take = min(__popc(idle), chunk_end - chunk_next);
            int rank = __popc(idle & ((1u << lane) - 1u));
            if (!active && rank < take) {
                int item = chunk_next + rank;
                int f = item / P.n_items;
                if (P.points) {
                    active = start_point_path(P, frame_begin + (unsigned)f, item - f * P.n_items, ps);
                } else if (item_pixel(P, item - f * P.n_items, ps.px, ps.py)) {
                    active = start_path(C, P, frame_begin + (unsigned)f, ps);
                    if (!active) deposit(C, A, P, apl, apt, ps, acc, acc_sq);
                }
            }
            chunk_next += take;
            idle = __ballot_sync(full, !active);
        }
        if (!__any_sync(full, active)) break;
        if (active && !bounce(C, M, A, P, E, tlut, tw, th, svl, svt, ps)) {
            deposit(C, A, P, apl, apt, ps, acc, acc_sq);
            active = false;
        }
    }
}

// ---------------------------------------------------------------------------
// The same estimator over the dense grid with brick majorants, as one flat
// loop per lane.  The kernel above runs a path's walks as nested loops (a free
// flight, then the ratio-tracking walk toward the sun at each event), so the
// lanes of a warp spread over different loops and wait for one another.  Here
// a lane's state says which walk it is in (free flight, or next-event ratio
// tracking with a copy of the RNG state) and every iteration advances each
// active lane's walk by one tentative collision: the brick steps up to it,
// then one trilinear density fetch at one shared call site for both kinds of
// walk.  Scattering, escape, the ground and path ends are handled where a walk
// ends.  Every walk draws the same random numbers in the same order as the
// nested form (the copied RNG state of next-event estimation is taken before
// the path's own state samples the new direction, which next-event estimation
// never reads), so the estimator and the oracle's RNG-matched paths are
// unchanged.
// ---------------------------------------------------------------------------
enum : int { kIdle = 0, kFlight = 1, kSunWalk = 2 };

struct FlatLane {
    PathState ps;
    Walk w;
    float t, t_end, tau;
    int it, mode;
    // next-event estimation in flight: RNG copy, transmittance so far, and the
    // contribution it scales, L += thr * (k * (ph * tr)); then go on (cont) or end
    uint32_t nseed;
    float tr, ph;
    float3 thr, k;
    bool cont;
};

// Begin the free flight of the next bounce from ps.o along ps.d; false when
// the ray leaves the region at once (the path ends: Trace's loop exit).
__device__ __forceinline__ bool begin_flight(const PtConsts& P, FlatLane& s) {
    float t0, t1;
    region(P, s.ps.o, s.ps.d, t0, t1);
    if (t0 >= t1) return false;
    s.t = t0;
    s.t_end = t1;
    walk_init(P, s.w, s.ps.o, s.ps.d, t0);
    s.tau = sample_tau(P, s.ps.seed);
    s.it = 0;
    s.mode = kFlight;
    return true;
}

// Begin next-event estimation from ps.o toward the sun with the RNG copy
// s.nseed (TransmittanceEstimation, PathTracing.comp:135-151); a ray that
// leaves the region at once has transmittance 1.
__device__ __forceinline__ bool begin_sun_walk(const CloudConsts& C, const PtConsts& P, FlatLane& s) {
    s.tr = 1.f;
    float t0, t1;
    region(P, s.ps.o, C.sun, t0, t1);
    if (t0 >= t1) return false;
    s.t = t0;
    s.t_end = t1;
    walk_init(P, s.w, s.ps.o, C.sun, t0);
    s.tau = sample_tau(P, s.nseed);
    s.it = 0;
    s.mode = kSunWalk;
    return true;
}

// The end of a next-event walk: its contribution, then the next bounce or the
// end of the path.  Returns whether the path goes on.
__device__ __forceinline__ bool finish_sun_walk(const PtConsts& P, FlatLane& s) {
    s.ps.L += s.thr * (s.k * (s.ph * clamp01(s.tr)));
    return s.cont && begin_flight(P, s);
}

// A free flight ended: a collision at s.t (scatter) or none (escape, the
// environment and the ground).  Returns whether the path goes on.
template <class S>
__device__ __forceinline__ bool flight_event(const CloudConsts& C, const AtmoConsts& A, const PtConsts& P,
                                             const ViewConsts& E, const float4* tlut, int tw, int th, const S* svl,
                                             const S* svt, FlatLane& s, bool collided) {
    PathState& ps = s.ps;
    if (collided) {
        if (!ps.scattered) {
            float3 dc = C.cam - ps.o;
            ps.scattered_t = sqrtf(dot3(dc, dc));
        }
        ps.scattered = true;
        ps.o = ps.o + ps.d * s.t;
        float cs = dot3(ps.d, C.sun);
        s.ph = hg_pt(cs, P.g_back) * (1.f - P.ratio) + hg_pt(cs, P.g_fwd) * P.ratio;
        s.k = sun_illuminance(C, A, tlut, tw, th, ps.o);
        s.thr = ps.thr;
        s.nseed = ps.seed;  // the copy next-event estimation draws from
        sample_scatter(P, ps);
        ++ps.istep;
        s.cont = ps.istep < P.max_bounces && fmaxf(ps.thr.x, fmaxf(ps.thr.y, ps.thr.z)) > 0.f;
        return begin_sun_walk(C, P, s) || finish_sun_walk(P, s);
    }
    if (P.env == SKYR_ENV_OFF || !ps.scattered) return false;
    auto env = [&](float3 wd) { return environment(A, E, tlut, tw, th, svl, svt, P.sv_w, P.sv_h, wd); };
    if (P.env == SKYR_ENV_CONST_ENVIRONMENT_MAP) {
        ps.L += ps.thr * env(P.m_front * ps.d.x + P.m_right * ps.d.y + P.m_up * ps.d.z);
        return false;
    }
    float3 o = ps.o, d = ps.d;
    float rho2 = fmaf(o.x, o.x, fmaf(o.y, o.y, o.z * (o.z + 2.f * C.R)));
    float r = sqrtf(fmaf(C.R, C.R, rho2));
    float mu = fmaf(d.x, o.x, fmaf(d.y, o.y, d.z * (o.z + C.R))) / r;
    if (!ray_hits_ground(r, rho2, mu)) {
        ps.L += ps.thr * env(P.m_front * d.x + P.m_right * d.y + P.m_up * d.z);
        return false;
    }
    o = o + d * dist_to_bottom(r, rho2, mu);
    float3 n = f3(o.x, o.y, o.z + C.R);
    n = n * rsqrtf(dot3(n, n));
    float ndl = dot3(n, C.sun);
    float3 bsdf = A.ground_albedo * (1.f / SKYR_PI);
    s.k = sun_illuminance(C, A, tlut, tw, th, o) * (bsdf * ndl);
    s.ph = 1.f;
    s.thr = ps.thr;
    s.nseed = ps.seed;
    ps.o = o;
    if (P.env == SKYR_ENV_GROUND_SINGLE_BOUNCE) {
        s.cont = false;
    } else {
        // GenerateLambertSample (PathTracing.comp:119-129)
        float st = sqrtf(rand01(P, ps.seed));
        float ct = sqrtf(clamp01(1.f - st * st));
        float3 b0, b1;
        onb(n, b0, b1);
        float sp, cp;
        sincosf(2.f * SKYR_PI * rand01(P, ps.seed), &sp, &cp);
        ps.d = b0 * (st * sp) + b1 * (st * cp) + n * ct;
        ps.thr *= A.ground_albedo;
        ++ps.istep;
        s.cont = ps.istep < P.max_bounces && fmaxf(ps.thr.x, fmaxf(ps.thr.y, ps.thr.z)) > 0.f;
    }
    return begin_sun_walk(C, P, s) || finish_sun_walk(P, s);
}

template <class S>
__global__ void __launch_bounds__(128, 6) pathtrace_flat_kernel(const __grid_constant__ CloudConsts C,
                                                                const __grid_constant__ MaterialConsts M,
                                                                const __grid_constant__ AtmoConsts A,
                                                                const __grid_constant__ PtConsts P,
                                                                const __grid_constant__ ViewConsts E,
                                                                const float4* __restrict__ tlut, int tw, int th,
                                                                const S* __restrict__ svl, const S* __restrict__ svt,
                                                                const S* __restrict__ apl, const S* __restrict__ apt,
                                                                unsigned frame_begin, int n_frames,
                                                                int* __restrict__ counter, float4* __restrict__ acc,
                                                                float4* __restrict__ acc_sq) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int n_total = P.n_items * n_frames;
    int chunk_next = 0, chunk_end = 0;  // warp-uniform
    bool exhausted = false;             // warp-uniform
    FlatLane s;
    s.mode = kIdle;
    s.ps.px = s.ps.py = 0;
    for (;;) {
        // hand the warp's next items to idle lanes (as pathtrace_kernel)
        unsigned idle = __ballot_sync(full, s.mode == kIdle);
        while (idle && !exhausted) {
            if (chunk_next >= chunk_end) {
                int base = 0;
                if (lane == 0) base = atomicAdd(counter, kWarpChunk);
                base = __shfl_sync(full, base, 0);
                if (base >= n_total) {
                    exhausted = true;
                    break;
                }
                chunk_next = base;
                chunk_end = min(base + kWarpChunk, n_total);
            }
            int take = min(__popc(idle), chunk_end - chunk_next);
            int rank = __popc(idle & ((1u << lane) - 1u));
            if (s.mode == kIdle && rank < take) {
                int item = chunk_next + rank;
                int f = item / P.n_items;
                bool live = false;
                if (P.points) {
                    live = start_point_path(P, frame_begin + (unsigned)f, item - f * P.n_items, s.ps) &&
                           begin_flight(P, s);
                    if (!live) deposit(C, A, P, apl, apt, s.ps, acc, acc_sq);
                } else if (item_pixel(P, item - f * P.n_items, s.ps.px, s.ps.py)) {
                    live = start_path(C, P, frame_begin + (unsigned)f, s.ps) && begin_flight(P, s);
                    if (!live) deposit(C, A, P, apl, apt, s.ps, acc, acc_sq);
                }
                if (!live) s.mode = kIdle;
            }
            chunk_next += take;
            idle = __ballot_sync(full, s.mode == kIdle);
        }
        if (!__any_sync(full, s.mode != kIdle)) break;
        if (s.mode == kIdle) continue;
        // one tentative collision of the lane's walk: brick steps up to it
        const float3 d = s.mode == kFlight ? s.ps.d : C.sun;
        bool ended = false, overrun = false;
        float m;
        for (;;) {
            if (++s.it > P.tracking_steps) {
                overrun = true;
                break;
            }
            float te = fminf(walk_exit(s.w), s.t_end);
            m = walk_majorant(P, s.w);
            float seg = (te - s.t) * m;
            if (s.tau < seg) break;
            s.tau -= seg;
            s.t = te;
            if (!(s.t < s.t_end)) {
                ended = true;
                break;
            }
            walk_step(s.w);
        }
        bool collided = false;
        if (overrun) {  // as the nested walks: a free flight counts as an escape, a sun walk keeps tr
            flag_overrun(P);
            ended = true;
        } else if (!ended) {
            // the density fetch both kinds of walk share
            s.t += s.tau / m;
            float sig = grid_sigma(P, s.ps.o + d * s.t);
            if (s.mode == kFlight) {
                if (rand01(P, s.ps.seed) < sig / m) collided = true;
                else s.tau = sample_tau(P, s.ps.seed);
            } else {
                s.tr *= 1.f - fmaxf(0.f, sig / m);
                s.tau = sample_tau(P, s.nseed);
            }
        }
        if (!ended && !collided) continue;
        bool live = s.mode == kFlight ? flight_event(C, A, P, E, tlut, tw, th, svl, svt, s, collided)
                                      : finish_sun_walk(P, s);
        if (!live) {
            deposit(C, A, P, apl, apt, s.ps, acc, acc_sq);
            s.mode = kIdle;
        }
    }
}

// ---------------------------------------------------------------------------
// Synthetic grid and brick majorants
// ---------------------------------------------------------------------------
// voxels [first, end) of the grid (the host splits the grid into short launches)
__global__ void __launch_bounds__(128) grid_generate_kernel(skyr_grid_generator g, size_t first, size_t end,
                                                            unsigned short* __restrict__ out) {
    size_t i = first + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((size_t)g.nx * g.ny));
    float3 p = f3(((float)x + 0.5f) / (float)g.nx, ((float)y + 0.5f) / (float)g.ny, ((float)z + 0.5f) / (float)g.nz);
    skyr_noise_create_info ci{g.seed, g.base_frequency, 1.f, 0.f};
    float w = fbm(SKYR_NOISE_WORLEY, p, ci, g.octaves);
    float3 q = f3((p.x - g.center[0]) / g.radii[0], (p.y - g.center[1]) / g.radii[1], (p.z - g.center[2]) / g.radii[2]);
    float dd = sqrtf(dot3(q, q));
    float env = 1.f - smoothstepf(g.inner, 1.f, dd);
    float v = clamp01(w * env - g.threshold) / (1.f - g.threshold);
    out[i] = __half_as_ushort(__float2half_rn(v));
}

// one warp per brick: max over the brick plus a one-voxel apron
__global__ void __launch_bounds__(128) grid_majorant_kernel(const unsigned short* __restrict__ grid, int nx, int ny,
                                                            int nz, int brick, int bx, int by, int bz, float density,
                                                            float* __restrict__ out) {
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid >= bx * by * bz) return;
    int i = wid % bx, j = (wid / bx) % by, k = wid / (bx * by);
    int e = brick + 2;
    float m = 0.f;
    for (int q = lane; q < e * e * e; q += 32) {
        int x = i * brick - 1 + q % e, y = j * brick - 1 + (q / e) % e, z = k * brick - 1 + q / (e * e);
        if ((unsigned)x < (unsigned)nx && (unsigned)y < (unsigned)ny && (unsigned)z < (unsigned)nz)
            m = fmaxf(m, __half2float(__ushort_as_half(grid[((size_t)z * ny + y) * nx + x])));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) out[wid] = m * density;
}

__global__ void __launch_bounds__(256) pt_resolve_kernel(const float4* __restrict__ acc, int n, float inv_frames,
                                                         const __half2* __restrict__ bg, __half2* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = acc[i];
    float3 c = f3(0.f);
    if (bg) {
        uint2 raw = reinterpret_cast<const uint2*>(bg)[i];
        float2 lo = __half22float2(*reinterpret_cast<__half2*>(&raw.x));
        float2 hi = __half22float2(*reinterpret_cast<__half2*>(&raw.y));
        c = f3(lo.x, lo.y, hi.x);
    }
    float w = a.w * inv_frames;
    float3 col = c * w + f3(a.x, a.y, a.z) * inv_frames;
    store_rgba(out, (size_t)i, col, 1.f);
}

}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_pathtrace_parameters_default(skyr_pathtrace_parameters* p) {
    if (!p) return set_error(SKYR_EINVAL, "null parameters");
    // PathTracing::InitParam defaults (src/SkyRendering/VolumetricCloud.h:104-114)
    *p = skyr_pathtrace_parameters{};
    p->max_bounces = 128;
    p->region_box_half_width = 100.f;
    p->importance_sampling = 1;
    p->forward_phase_g = 0.85f;
    p->back_phase_g = -0.15f;
    p->forward_scattering_ratio = 0.7f;
    p->prng = SKYR_PRNG_PCG_HASH;
    p->environment_lighting = SKYR_ENV_GROUND_MULTI_BOUNCE;
    p->sigma_t_max = 15.f;  // VolumetricCloudDefaultMaterialCommon::density_
    p->use_brick_majorants = 1;
    return SKYR_OK;
}

size_t skyr_grid_bytes(int nx, int ny, int nz) {
    if (nx < 1 || ny < 1 || nz < 1) return 0;
    return (size_t)nx * ny * nz * 2;
}

int skyr_grid_brick_count(int n, int brick) {
    if (n < 1 || brick < 1) return 0;
    return (n + brick - 1) / brick;
}

int skyr_grid_generate(skyr_ctx* ctx, const skyr_grid_generator* g, void* out) {
    if (!ctx || !g || !out) return set_error(SKYR_EINVAL, "null argument");
    if (g->nx < 1 || g->ny < 1 || g->nz < 1 || (size_t)g->nx * g->ny * g->nz > (size_t(1) << 33))
        return set_error(SKYR_EINVAL, "bad grid size");
    if (g->octaves < 1 || g->octaves > 16 || g->base_frequency < 1 || ((long long)g->base_frequency << (g->octaves - 1)) > (1 << 20))
        return set_error(SKYR_EINVAL, "bad grid noise frequency / octaves");
    if (!(g->radii[0] > 0.f) || !(g->radii[1] > 0.f) || !(g->radii[2] > 0.f) || !(g->threshold < 1.f) ||
        !(g->inner < 1.f))
        return set_error(SKYR_EINVAL, "bad grid envelope");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    size_t n = (size_t)g->nx * g->ny * g->nz;
    // about 16 M voxels (~0.15 s of 4-octave Worley) per launch
    const size_t chunk = (size_t)1 << 24;
    for (size_t first = 0; first < n; first += chunk) {
        size_t end = std::min(n, first + chunk);
        grid_generate_kernel<<<(unsigned)((end - first + 127) / 128), 128, 0, ctx->stream>>>(
            *g, first, end, reinterpret_cast<unsigned short*>(out));
        if (int e = check_cuda(cudaGetLastError(), "grid generator kernel")) return e;
    }
    return SKYR_OK;
}

int skyr_grid_majorants(skyr_ctx* ctx, const skyr_density_grid* gd, float* out) {
    if (!ctx || !gd || !gd->data || !out) return set_error(SKYR_EINVAL, "null argument");
    if (gd->nx < 1 || gd->ny < 1 || gd->nz < 1 || gd->brick < 1) return set_error(SKYR_EINVAL, "bad grid");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    int bx = skyr_grid_brick_count(gd->nx, gd->brick), by = skyr_grid_brick_count(gd->ny, gd->brick),
        bz = skyr_grid_brick_count(gd->nz, gd->brick);
    long long warps = (long long)bx * by * bz;
    grid_majorant_kernel<<<(unsigned)((warps * 32 + 127) / 128), 128, 0, ctx->stream>>>(
        reinterpret_cast<const unsigned short*>(gd->data), gd->nx, gd->ny, gd->nz, gd->brick, bx, by, bz,
        gd->density, out);
    return check_cuda(cudaGetLastError(), "grid majorant kernel");
}

}  // extern "C"

namespace {

// Work source of one launch: the view's region (tiles), a pixel list, or points.
struct PtSource {
    const int* region_px = nullptr;  // [x0, y0, x1, y1] or NULL (whole view)
    const int* pixel_list = nullptr;
    int n_pixels = 0;
    const float* points = nullptr;
    float* point_out = nullptr;
    int n_points = 0;
};

int pathtrace_launch(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                     const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                     const skyr_cloud_textures* textures, const skyr_density_grid* grid,
                     const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                     const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                     const void* transmittance, const void* sky_view_luminance, const void* sky_view_transmittance,
                     const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                     unsigned frame_begin, int n_frames, const PtSource& src, float* accumulation,
                     float* accumulation_sq) {
    if (!ctx || !atmosphere || !cloud || !pt || !view || !env_view || !sizes)
        return set_error(SKYR_EINVAL, "null argument");
    if (!src.points && !accumulation) return set_error(SKYR_EINVAL, "null accumulation buffer");
    if (!transmittance || !sky_view_luminance || !sky_view_transmittance || !aerial_perspective_luminance ||
        !aerial_perspective_transmittance)
        return set_error(SKYR_EINVAL, "null LUT input");
    if (n_frames < 0 || n_frames > (1 << 20)) return set_error(SKYR_EINVAL, "n_frames out of range");
    if (pt->max_bounces < 0 || pt->environment_lighting < SKYR_ENV_OFF ||
        pt->environment_lighting > SKYR_ENV_GROUND_MULTI_BOUNCE || pt->prng < 0 || pt->prng > 1)
        return set_error(SKYR_EINVAL, "bad path tracer parameters");
    if (!std::isfinite(pt->sigma_t_max) || pt->sigma_t_max < 0.f || !(std::fabs(pt->forward_phase_g) < 1.f) ||
        !(std::fabs(pt->back_phase_g) < 1.f) || !(pt->forward_scattering_ratio >= 0.f) ||
        !(pt->forward_scattering_ratio <= 1.f) || !std::isfinite(pt->region_box_half_width))
        return set_error(SKYR_EINVAL, "path tracer parameters out of range");
    if (pt->importance_sampling && (pt->forward_phase_g == 0.f || pt->back_phase_g == 0.f))
        return set_error(SKYR_EINVAL, "HG importance sampling needs g != 0 (HenyeyGreensteinInvertcdf divides by g)");
    bool use_grid = grid && grid->data;
    if (!use_grid && !material) return set_error(SKYR_EINVAL, "need a density grid or a material");
    if (use_grid && pt->use_brick_majorants && !grid->majorant)
        return set_error(SKYR_EINVAL, "brick majorants requested but the grid has none");
    if (!use_grid && pt->use_brick_majorants) return set_error(SKYR_ENOTSUP, "brick majorants need a density grid");
    skyr_cloud_material mat_default;
    skyr_cloud_textures tex_empty{};
    if (!material) {
        skyr_cloud_material_default(SKYR_MATERIAL_MINIMAL, &mat_default);
        material = &mat_default;
    }
    if (!textures) textures = &tex_empty;
    CloudConsts C;
    MaterialConsts M;
    if (int st = derive_cloud_consts(*atmosphere, *cloud, *material, *textures, *view, *sizes, C, M)) return st;
    AtmoConsts A;
    derive_atmo_consts(*atmosphere, A);
    ViewConsts E;
    derive_view_consts(*atmosphere, *env_view, E);
    PtConsts P;
    std::memset(&P, 0, sizeof(P));
    float hw = pt->region_box_half_width;
    P.box_min = make_float3(-hw, -hw, C.bottom);
    P.box_max = make_float3(hw, hw, C.top);
    P.max_bounces = pt->max_bounces;
    P.importance_sampling = pt->importance_sampling;
    P.prng = pt->prng;
    P.env = pt->environment_lighting;
    P.g_fwd = pt->forward_phase_g;
    P.g_back = pt->back_phase_g;
    P.ratio = pt->forward_scattering_ratio;
    P.sigma_t_max = pt->sigma_t_max;
    if (use_grid) {
        if (grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->voxel_size > 0.f) || grid->brick < 1 ||
            !std::isfinite(grid->density) || grid->density < 0.f || !std::isfinite(grid->origin[0]) ||
            !std::isfinite(grid->origin[1]) || !std::isfinite(grid->origin[2]))
            return set_error(SKYR_EINVAL, "bad density grid");
        P.grid = reinterpret_cast<const unsigned short*>(grid->data);
        P.nx = grid->nx;
        P.ny = grid->ny;
        P.nz = grid->nz;
        P.origin = make_float3(grid->origin[0], grid->origin[1], grid->origin[2]);
        P.inv_voxel = 1.f / grid->voxel_size;
        P.density = grid->density;
        P.maj = grid->majorant;
        P.bx = skyr_grid_brick_count(grid->nx, grid->brick);
        P.by = skyr_grid_brick_count(grid->ny, grid->brick);
        P.bz = skyr_grid_brick_count(grid->nz, grid->brick);
        P.brick_size = grid->voxel_size * (float)grid->brick;
        P.use_bricks = pt->use_brick_majorants ? 1 : 0;
        float gmax[3] = {grid->origin[0] + grid->nx * grid->voxel_size, grid->origin[1] + grid->ny * grid->voxel_size,
                         grid->origin[2] + grid->nz * grid->voxel_size};
        P.box_min = make_float3(fmaxf(P.box_min.x, grid->origin[0]), fmaxf(P.box_min.y, grid->origin[1]),
                                fmaxf(P.box_min.z, grid->origin[2]));
        P.box_max = make_float3(fminf(P.box_max.x, gmax[0]), fminf(P.box_max.y, gmax[1]), fminf(P.box_max.z, gmax[2]));
    }
    {
        // kModelMatrix3 (VolumetricCloud.cpp:188-200, 515-519): local -> world directions
        double R = atmosphere->bottom_radius;
        double c[3] = {view->camera_position[0], view->camera_position[1] + R, view->camera_position[2]};
        double cl = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        double up[3] = {c[0] / cl, c[1] / cl, c[2] / cl};
        double fr[3] = {0.0, up[2], -up[1]};  // cross(up, (1,0,0))
        double fl = std::sqrt(fr[1] * fr[1] + fr[2] * fr[2]);
        fr[1] /= fl;
        fr[2] /= fl;
        double rt[3] = {up[1] * fr[2] - up[2] * fr[1], up[2] * fr[0] - up[0] * fr[2], up[0] * fr[1] - up[1] * fr[0]};
        double rl = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
        P.m_front = make_float3((float)fr[0], (float)fr[1], (float)fr[2]);
        P.m_right = make_float3((float)(rt[0] / rl), (float)(rt[1] / rl), (float)(rt[2] / rl));
        P.m_up = make_float3((float)up[0], (float)up[1], (float)up[2]);
    }
    P.sv_w = sizes->sky_view_width;
    P.sv_h = sizes->sky_view_height;
    P.width = view->width;
    P.height = view->height;
    const int* region_px = src.region_px;
    if (region_px) {
        P.x0 = std::max(region_px[0], 0);
        P.y0 = std::max(region_px[1], 0);
        P.x1 = std::min(region_px[2], view->width);
        P.y1 = std::min(region_px[3], view->height);
    } else {
        P.x0 = P.y0 = 0;
        P.x1 = view->width;
        P.y1 = view->height;
    }
    long long items;
    if (src.points) {
        if (src.n_points < 0) return set_error(SKYR_EINVAL, "negative point count");
        if (!src.point_out) return set_error(SKYR_EINVAL, "null point output");
        if (!use_grid) return set_error(SKYR_ENOTSUP, "point sources need a density grid");
        P.points = src.points;
        P.point_out = src.point_out;
        items = src.n_points;
    } else if (src.pixel_list) {
        if (src.n_pixels < 0) return set_error(SKYR_EINVAL, "negative pixel count");
        P.pixel_list = src.pixel_list;
        items = src.n_pixels;
    } else {
        if (P.x1 <= P.x0 || P.y1 <= P.y0) return SKYR_OK;
        P.tiles_x = (P.x1 - P.x0 + 7) / 8;
        items = (long long)P.tiles_x * ((P.y1 - P.y0 + 3) / 4) * 32;
    }
    if (items == 0 || n_frames == 0) return SKYR_OK;
    if (sizes->sky_view_width < 2 || sizes->sky_view_height < 2) return set_error(SKYR_EINVAL, "bad sky-view size");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = ensure_status(ctx)) return e;
    P.status = ctx->d_status;
    P.tracking_steps = ctx->limits.tracking_steps;
    if (items * n_frames > (1LL << 30))
        return set_error(SKYR_EINVAL, "work items x frames too large for one call (2^30 paths)");
    P.n_items = (int)items;
    // the call's work counter
    if (int e = ensure_pt_scratch(ctx, sizeof(int))) return e;
    int* counter = reinterpret_cast<int*>(ctx->pt_scratch);
    if (int e = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), ctx->stream), "clear work counter")) return e;
    const float4* T = reinterpret_cast<const float4*>(transmittance);
    float4* acc = reinterpret_cast<float4*>(accumulation);
    float4* acc2 = reinterpret_cast<float4*>(accumulation_sq);
    auto launch = [&](auto tag) -> int {
        using S = decltype(tag);
        // the flat form for the dense grid with brick majorants, the nested form otherwise
        auto kernel = P.grid && P.use_bricks ? pathtrace_flat_kernel<S> : pathtrace_kernel<S>;
        int per_sm = 0, sms = 0;
        if (int e = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0), "occupancy"))
            return e;
        if (int e = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "SM count"))
            return e;
        long long blocks = std::min<long long>((long long)std::max(per_sm, 1) * sms, (items * n_frames + 127) / 128);
        kernel<<<(unsigned)blocks, 128, 0, ctx->stream>>>(
            C, M, A, P, E, T, sizes->transmittance_width, sizes->transmittance_height,
            reinterpret_cast<const S*>(sky_view_luminance), reinterpret_cast<const S*>(sky_view_transmittance),
            reinterpret_cast<const S*>(aerial_perspective_luminance),
            reinterpret_cast<const S*>(aerial_perspective_transmittance), frame_begin, n_frames, counter, acc, acc2);
        if (int e = check_cuda(cudaGetLastError(), "path tracer kernel")) return e;
        return SKYR_OK;
    };
    return sizes->format == SKYR_FORMAT_RGBA16F ? launch(__half2{}) : launch(float4{});
}

}  // namespace

extern "C" {

int skyr_pathtrace(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                   const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                   const skyr_cloud_textures* textures, const skyr_density_grid* grid,
                   const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                   const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                   const void* transmittance, const void* sky_view_luminance, const void* sky_view_transmittance,
                   const void* aerial_perspective_luminance, const void* aerial_perspective_transmittance,
                   unsigned frame_begin, int n_frames, const int* region_px, float* accumulation,
                   float* accumulation_sq) {
    PtSource src;
    src.region_px = region_px;
    return pathtrace_launch(ctx, atmosphere, cloud, material, textures, grid, pt, view, env_view, sizes,
                            transmittance, sky_view_luminance, sky_view_transmittance,
                            aerial_perspective_luminance, aerial_perspective_transmittance, frame_begin, n_frames,
                            src, accumulation, accumulation_sq);
}

int skyr_pathtrace_pixels(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_cloud_material* material,
                          const skyr_cloud_textures* textures, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, const void* aerial_perspective_luminance,
                          const void* aerial_perspective_transmittance, unsigned frame_begin, int n_frames,
                          const int* pixels, int n_pixels, float* accumulation, float* accumulation_sq) {
    if (n_pixels > 0 && !pixels) return set_error(SKYR_EINVAL, "null pixel list");
    PtSource src;
    src.pixel_list = pixels;
    src.n_pixels = n_pixels;
    return pathtrace_launch(ctx, atmosphere, cloud, material, textures, grid, pt, view, env_view, sizes,
                            transmittance, sky_view_luminance, sky_view_transmittance,
                            aerial_perspective_luminance, aerial_perspective_transmittance, frame_begin, n_frames,
                            src, accumulation, accumulation_sq);
}

int skyr_pathtrace_points(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_cloud_parameters* cloud, const skyr_density_grid* grid,
                          const skyr_pathtrace_parameters* pt, const skyr_cloud_view* view,
                          const skyr_atmosphere_render_parameters* env_view, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, const void* aerial_perspective_luminance,
                          const void* aerial_perspective_transmittance, unsigned frame_begin, int n_paths,
                          const float* points, int n_points, float* out) {
    if (n_points > 0 && (!points || !out)) return set_error(SKYR_EINVAL, "null points or output");
    if (!grid || !grid->data) return set_error(SKYR_EINVAL, "point sources need a density grid");
    PtSource src;
    src.points = points;
    src.point_out = out;
    src.n_points = n_points;
    return pathtrace_launch(ctx, atmosphere, cloud, nullptr, nullptr, grid, pt, view, env_view, sizes,
                            transmittance, sky_view_luminance, sky_view_transmittance,
                            aerial_perspective_luminance, aerial_perspective_transmittance, frame_begin, n_paths,
                            src, nullptr, nullptr);
}


int skyr_pathtrace_resolve(skyr_ctx* ctx, const float* accumulation, int width, int height, unsigned frames,
                           const void* background_rgba16f, void* out_rgba16f) {
    if (!ctx || !accumulation || !out_rgba16f) return set_error(SKYR_EINVAL, "null argument");
    if (width < 1 || height < 1 || frames < 1) return set_error(SKYR_EINVAL, "bad size or frame count");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    int n = width * height;
    pt_resolve_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
        reinterpret_cast<const float4*>(accumulation), n, 1.f / (float)frames,
        reinterpret_cast<const __half2*>(background_rgba16f), reinterpret_cast<__half2*>(out_rgba16f));
    return check_cuda(cudaGetLastError(), "path tracer resolve kernel");
}

}  // extern "C"
