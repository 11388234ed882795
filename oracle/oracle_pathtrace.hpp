// oracle_pathtrace.hpp — TEST INFRASTRUCTURE ONLY.
//
// Restatement of the volumetric-cloud path tracer of c52e/SkyRendering
// (shaders/SkyRendering/VolumetricCloudPathTracing.comp:19-296, helpers from
// VolumetricCloudCommon.glsl:58-71 and shaders/Base/Common.glsl:32-52), the
// ENVIRONMENT_LUMINANCE lookup it samples (AtmosphereRenderer.glsl:113-145,
// 250-273), the synthetic dense grid generator and the brick majorant grid.
// Random numbers follow the reference exactly: Random01 returns
// float(seed) / 2^32 in FP32 (the FP32 conversion is kept so that the GPU and
// this oracle draw identical numbers) and TransmittanceEstimation receives a
// copy of the RNG context.  Everything else is in the scalar type T.
// Parity status: unpinned (see oracle_math.hpp).
#pragma once

#include <cstring>

#include "../include/skyr_pathtrace.h"
#include "oracle_cloud.hpp"
#include "oracle_environment.hpp"
#include "oracle_noise.hpp"

namespace orc {

inline float half_to_float(uint16_t h) {
    uint32_t s = (h >> 15) & 1u, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t bits;
    if (e == 0) {
        if (m == 0) {
            bits = s << 31;
        } else {  // subnormal
            int k = -1;
            do {
                ++k;
                m <<= 1;
            } while (!(m & 0x400u));
            bits = (s << 31) | ((uint32_t)(127 - 15 - k) << 23) | ((m & 0x3ffu) << 13);
        }
    } else if (e == 31) {
        bits = (s << 31) | 0x7f800000u | (m << 13);
    } else {
        bits = (s << 31) | ((e + 127 - 15) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// Synthetic grid value at voxel (x, y, z) (skyr_grid_generator semantics).
template <class T>
T grid_value(const skyr_grid_generator& g, int x, int y, int z) {
    V3<T> p((T(x) + T(0.5)) / T(g.nx), (T(y) + T(0.5)) / T(g.ny), (T(z) + T(0.5)) / T(g.nz));
    skyr_noise_create_info ci{g.seed, g.base_frequency, 1.0f, 0.0f};
    T w = FBM<T>(SKYR_NOISE_WORLEY, p, ci, g.octaves);
    V3<T> q((p.x - T(g.center[0])) / T(g.radii[0]), (p.y - T(g.center[1])) / T(g.radii[1]),
            (p.z - T(g.center[2])) / T(g.radii[2]));
    T d = length(q);
    T env = T(1) - smoothstepg(T(g.inner), T(1), d);
    T v = clampg(w * env - T(g.threshold), T(0), T(1)) / (T(1) - T(g.threshold));
    return v;
}

// Cap on the samples of one tracking walk, as in the CUDA path tracer: the walk
// ends (free flight: no collision) when it is reached.
constexpr int kMaxTrackingSteps = 1 << 20;

// Trilinear extinction of a dense FP16 grid between voxel centres, zero border
// (the voxel material's CLAMP_TO_BORDER sampler, VolumetricCloudVoxelMaterial.cpp:25-31)
template <class T>
T grid_trilinear(const uint16_t* g, int nx, int ny, int nz, V3<T> origin, T voxel, T density, V3<T> p) {
    auto at = [&](int x, int y, int z) -> T {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return T(0);
        return T(half_to_float(g[((size_t)z * ny + y) * nx + x]));
    };
    V3<T> q = (p - origin) / voxel - V3<T>(T(0.5));
    T fx = std::floor(q.x), fy = std::floor(q.y), fz = std::floor(q.z);
    T a = q.x - fx, b = q.y - fy, c = q.z - fz;
    int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    T r = 0;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
                r += (dx ? a : T(1) - a) * (dy ? b : T(1) - b) * (dz ? c : T(1) - c) * at(x0 + dx, y0 + dy, z0 + dz);
    return r * density;
}

template <class T>
struct PathTracerOracle {
    const AtmosphereOracle<T>& O;
    const CloudOracle<T>& Cl;  // frame, material, AP LUTs, T LUT
    const ViewLutOracle<T>& Env;
    const Image<T>* svl;
    const Image<T>* svt;
    skyr_pathtrace_parameters P;
    // dense grid (nullptr = material)
    const uint16_t* grid = nullptr;
    int nx = 0, ny = 0, nz = 0;
    V3<T> origin;
    T voxel = 1, density = 0;
    const float* maj = nullptr;
    int brick = 16, bx = 0, by = 0, bz = 0;
    V3<T> box_min, box_max;
    M4<T> model3;  // kModelMatrix3 (local -> world directions)

    uint32_t prng(uint32_t s) const { return P.prng == SKYR_PRNG_WANG_HASH ? WangHash(s) : PCGHash(s); }

    // Random01 (PathTracing.comp:44-48)
    T rand(uint32_t& seed) const {
        float r = float(seed) / 4294967296.0f;
        seed = prng(seed);
        return T(r);
    }

    T voxel_at(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return T(0);
        return T(half_to_float(grid[((size_t)z * ny + y) * nx + x]));
    }

    T grid_sigma(V3<T> p) const { return grid_trilinear<T>(grid, nx, ny, nz, origin, voxel, density, p); }

    // SampleSigmaT(vec3 P) (PathTracing.comp:89-91): flat height01
    T SampleSigmaT(V3<T> p) const {
        if (grid) return grid_sigma(p);
        T h01 = clampg((p.z - Cl.F.bottom) / (Cl.F.top - Cl.F.bottom), T(0), T(1));
        return Cl.SampleSigmaT(p, h01);
    }

    T HG(T c, T g) const { return Cl.HG(c, g); }
    T GetPhase(T c) const {
        return mixg(HG(c, T(P.back_phase_g)), HG(c, T(P.forward_phase_g)), T(P.forward_scattering_ratio));
    }

    // CloudRegionIntersect (PathTracing.comp:57-75)
    void region(V3<T> o, V3<T> d, T& t0, T& t1) const {
        t0 = T(0);
        t1 = T(1e7);
        for (int i = 0; i < 3; ++i) {
            T a = (box_min[i] - o[i]) / d[i], b = (box_max[i] - o[i]) / d[i];
            t0 = std::max(t0, std::min(a, b));
            t1 = std::min(t1, std::max(a, b));
        }
    }

    // Brick walk along a ray (3D DDA over the majorant bricks, integer indices)
    struct Walk {
        int i[3], s[3];
        T tmax[3], tdel[3];
    };

    void walk_init(Walk& w, V3<T> o, V3<T> d, T t) const {
        T bs = voxel * T(brick);
        V3<T> p = o + d * t;
        for (int a = 0; a < 3; ++a) {
            T g = (p[a] - origin[a]) / bs;
            w.i[a] = (int)std::floor(g);
            if (d[a] > T(0)) {
                w.s[a] = 1;
                w.tmax[a] = t + (origin[a] + T(w.i[a] + 1) * bs - p[a]) / d[a];
                w.tdel[a] = bs / d[a];
            } else if (d[a] < T(0)) {
                w.s[a] = -1;
                w.tmax[a] = t + (origin[a] + T(w.i[a]) * bs - p[a]) / d[a];
                w.tdel[a] = -bs / d[a];
            } else {
                w.s[a] = 0;
                w.tmax[a] = T(1e30);
                w.tdel[a] = T(1e30);
            }
        }
    }
    T walk_exit(const Walk& w) const { return std::min(w.tmax[0], std::min(w.tmax[1], w.tmax[2])); }
    void walk_step(Walk& w) const {
        int a = w.tmax[0] <= w.tmax[1] ? (w.tmax[0] <= w.tmax[2] ? 0 : 2) : (w.tmax[1] <= w.tmax[2] ? 1 : 2);
        w.i[a] += w.s[a];
        w.tmax[a] += w.tdel[a];
    }
    T walk_majorant(const Walk& w) const {  // boundary brick for rounding at the box faces
        int i = std::min(std::max(w.i[0], 0), bx - 1), j = std::min(std::max(w.i[1], 0), by - 1),
            k = std::min(std::max(w.i[2], 0), bz - 1);
        return T(maj[((size_t)k * by + j) * bx + i]);
    }
    T sample_tau(uint32_t& seed) const { return -std::log(T(1) - rand(seed)); }

    bool use_bricks() const { return grid && maj && P.use_brick_majorants; }

    // free flight in [t, t_max]; returns true on a collision (t updated)
    bool free_flight(uint32_t& seed, V3<T> o, V3<T> d, T& t, T t_max) const {
        if (!use_bricks()) {
            T smax = T(P.sigma_t_max);
            for (int it = 0; it < kMaxTrackingSteps; ++it) {
                if (smax <= T(0)) return false;
                t += -std::log(T(1) - rand(seed)) / smax;
                if (t > t_max) return false;
                T s = SampleSigmaT(o + d * t);
                if (rand(seed) < s / smax) return true;
            }
            return false;
        }
        // one exponential optical depth per tentative collision, spent brick by brick
        Walk w;
        walk_init(w, o, d, t);
        T tau = sample_tau(seed);
        for (int it = 0;; ++it) {
            if (it >= kMaxTrackingSteps) return false;
            T te = std::min(walk_exit(w), t_max);
            T m = walk_majorant(w);
            T seg = (te - t) * m;
            if (tau < seg) {
                t += tau / m;
                T s = SampleSigmaT(o + d * t);
                if (rand(seed) < s / m) return true;
                tau = sample_tau(seed);
                continue;
            }
            tau -= seg;
            t = te;
            if (!(t < t_max)) return false;
            walk_step(w);
        }
    }

    // TransmittanceEstimation (PathTracing.comp:135-151), ratio tracking; the
    // context (seed) is a copy
    T TransmittanceEstimation(uint32_t seed, V3<T> o, V3<T> d) const {
        T tr = T(1);
        T t0, t1;
        region(o, d, t0, t1);
        if (t0 >= t1) return tr;
        T t = t0;
        if (!use_bricks()) {
            T smax = T(P.sigma_t_max);
            for (int it = 0; it < kMaxTrackingSteps; ++it) {
                t += -std::log(T(1) - rand(seed)) / smax;
                if (t > t1) break;
                T s = SampleSigmaT(o + d * t);
                tr *= T(1) - std::max(T(0), s / smax);
            }
            return clampg(tr, T(0), T(1));
        }
        Walk w;
        walk_init(w, o, d, t);
        T tau = sample_tau(seed);
        for (int it = 0; it < kMaxTrackingSteps; ++it) {
            T te = std::min(walk_exit(w), t1);
            T m = walk_majorant(w);
            T seg = (te - t) * m;
            if (tau < seg) {
                t += tau / m;
                tr *= T(1) - std::max(T(0), SampleSigmaT(o + d * t) / m);
                tau = sample_tau(seed);
                continue;
            }
            tau -= seg;
            t = te;
            if (!(t < t1)) break;
            walk_step(w);
        }
        return clampg(tr, T(0), T(1));
    }

    V3<T> sun_illuminance(V3<T> pos) const { return Cl.SunVisibilityAt(pos) * O.A.solar_illuminance; }

    // ENVIRONMENT_LUMINANCE (AtmosphereRenderer.glsl:250-273) for a world direction
    V3<T> environment(V3<T> w) const { return environment_luminance(O, Env.F, *Cl.tlut, *svl, *svt, w); }

    V3<T> env_local(V3<T> d) const { return environment(mul_dir(model3, d)); }

    // CreateOrthonormalBasis (Common.glsl:45-50)
    static void basis(V3<T> n, V3<T>& t0, V3<T>& t1) {
        T s = n.z >= T(0) ? T(1) : T(-1);
        T a = T(-1) / (s + n.z);
        T b = n.x * n.y * a;
        t0 = V3<T>(T(1) + s * n.x * n.x * a, s * b, -s * n.x);
        t1 = V3<T>(b, s + n.y * n.y * a, -n.y);
    }

    V3<T> uniform_sphere(uint32_t& seed) const {
        T phi = T(2) * T(kPi) * rand(seed);
        T c = T(1) - T(2) * rand(seed);
        T s = std::sqrt(clampg(T(1) - c * c, T(0), T(1)));
        return V3<T>(std::cos(phi) * s, std::sin(phi) * s, c);
    }

    // GenerateHGSample (PathTracing.comp:98-117) about d, or a uniform direction
    // weighted by the phase function
    void scatter_direction(uint32_t& seed, V3<T>& d, V3<T>& thr) const {
        if (P.importance_sampling) {
            T g = rand(seed) < T(P.forward_scattering_ratio) ? T(P.forward_phase_g) : T(P.back_phase_g);
            T xi = rand(seed);
            T opg = T(1) + g * g, omg = T(1) - g * g, o2g = T(0.5) / g;
            T tt = omg / (T(1) - g + T(2) * g * xi);
            T ct = o2g * (opg - tt * tt);
            T st = std::sqrt(clampg(T(1) - ct * ct, T(0), T(1)));
            V3<T> b0, b1;
            basis(d, b0, b1);
            T phi = T(2) * T(kPi) * rand(seed);
            d = b0 * (st * std::sin(phi)) + b1 * (st * std::cos(phi)) + d * ct;
        } else {
            V3<T> nd = uniform_sphere(seed);
            T val = GetPhase(dot(d, nd));
            thr *= val * T(4) * T(kPi);
            d = nd;
        }
    }

    // The bounce loop of Trace (PathTracing.comp:180-247) from state (o, d, thr, istep)
    void trace_from(uint32_t& seed, V3<T> o, V3<T> d, V3<T> thr, int istep, V3<T>& L, bool& has_scattered,
                    T& scattered_t) const {
        const int env = P.environment_lighting;
        while (istep < P.max_bounces && std::max(thr.x, std::max(thr.y, thr.z)) > T(0)) {
            T t0, t1;
            region(o, d, t0, t1);
            if (t0 >= t1) break;
            T t = t0;
            bool scatter = free_flight(seed, o, d, t, t1);
            if (!scatter) {
                if (env == SKYR_ENV_OFF) break;
                if (!has_scattered) break;
                if (env == SKYR_ENV_CONST_ENVIRONMENT_MAP) {
                    L += thr * env_local(d);
                    break;
                }
                V3<T> up(o.x, o.y, o.z + Cl.F.R);
                T r = length(up);
                up = up / r;
                T mu = dot(d, up);
                if (!O.RayIntersectsGround(r, mu)) {
                    L += thr * env_local(d);
                    break;
                }
                o = o + d * O.DistanceToBottomAtmosphereBoundary(r, mu);
                V3<T> n = normalize(V3<T>(o.x, o.y, o.z + Cl.F.R));
                V3<T> bsdf = O.A.ground_albedo * (T(1) / T(kPi));
                T ndl = dot(n, Cl.F.sun);
                L += thr * (sun_illuminance(o) * (bsdf * ndl) * TransmittanceEstimation(seed, o, Cl.F.sun));
                if (env == SKYR_ENV_GROUND_SINGLE_BOUNCE) break;
                // GenerateLambertSample (PathTracing.comp:119-129)
                T st = std::sqrt(rand(seed));
                T ct = std::sqrt(clampg(T(1) - st * st, T(0), T(1)));
                V3<T> b0, b1;
                basis(n, b0, b1);
                T phi = T(2) * T(kPi) * rand(seed);
                d = b0 * (st * std::sin(phi)) + b1 * (st * std::cos(phi)) + n * ct;
                thr *= O.A.ground_albedo;
            } else {
                if (!has_scattered) scattered_t = length(Cl.F.cam - o);
                has_scattered = true;
                o = o + d * t;
                T ph = GetPhase(dot(d, Cl.F.sun));
                L += thr * (sun_illuminance(o) * ph * TransmittanceEstimation(seed, o, Cl.F.sun));
                scatter_direction(seed, d, thr);
            }
            ++istep;
        }
    }

    // Trace (PathTracing.comp:160-249); returns (L, a)
    void Trace(uint32_t& seed, V3<T> view, V3<T>& L_out, T& a_out, bool& has_scattered, T& scattered_t) const {
        V3<T> L(T(0)), thr(T(1));
        has_scattered = false;
        scattered_t = T(0);
        V3<T> o = Cl.F.cam, d = view;
        T c0, c1;
        region(o, d, c0, c1);
        if (c0 >= c1) {
            L_out = L;
            a_out = thr.x;  // vec4(L, throughput) takes throughput.x
            return;
        }
        o = o + d * c0;
        trace_from(seed, o, d, thr, 0, L, has_scattered, scattered_t);
        L_out = L;
        a_out = has_scattered ? T(0) : T(1);
    }

    // Point source (skyr_pathtrace_points): a path that has just scattered at p
    // while travelling along w; its radiance (no aerial perspective)
    V3<T> PointPath(uint32_t i, uint32_t frame, V3<T> p, V3<T> w) const {
        uint32_t seed = prng(prng(prng(i) + 0x2545F491u) + frame);
        V3<T> d = w, thr(T(1)), L(T(0));
        scatter_direction(seed, d, thr);
        if (P.max_bounces <= 1) return L;
        bool sc = true;
        T st = T(0);
        trace_from(seed, p, d, thr, 1, L, sc, st);
        return L;
    }

    // main (PathTracing.comp:255-284) for one frame of one pixel
    void Pixel(int px, int py, int w, int h, uint32_t frame, T out[4]) const {
        uint32_t seed = prng(prng(prng((uint32_t)px) + (uint32_t)py) + frame);
        T u = (T(px) + T(0.5)) / T(w), v = (T(py) + T(0.5)) / T(h);
        V3<T> frag = projective_mul(Cl.F.inv_mvp, V3<T>(u * T(2) - T(1), v * T(2) - T(1), T(1)));
        V3<T> view = normalize(frag - Cl.F.cam);
        V3<T> L;
        T a, st;
        bool sc;
        Trace(seed, view, L, a, sc, st);
        if (sc) {
            T r = Cl.F.cam.z + Cl.F.R, mu = view.z;
            T ta = st;
            if (r > O.A.top_radius) {
                T disc = r * r * (mu * mu - T(1)) + O.A.top_radius * O.A.top_radius;
                if (mu < T(0) && disc >= T(0)) ta -= std::max(-r * mu - std::sqrt(std::max(disc, T(0))), T(0));
                else ta = T(0);
            }
            T wz = std::sqrt(ta / Cl.F.ap_max_distance);
            const Image<T>& al = *Cl.ap_lum;
            T uu = T(0.5) / T(al.w) + u * (T(1) - T(1) / T(al.w));
            T vv = T(0.5) / T(al.h) + v * (T(1) - T(1) / T(al.h));
            T ww = T(0.5) / T(al.d) + wz * (T(1) - T(1) / T(al.d));
            V3<T> at = sample_linear_clamp3(*Cl.ap_trans, uu, vv, ww);
            V3<T> alum = sample_linear_clamp3(al, uu, vv, ww);
            alum = alum * Cl.RayScatterVisibility(u, v, st);  // PathTracing.comp:277
            L = L * at + alum;
        }
        out[0] = L.x;
        out[1] = L.y;
        out[2] = L.z;
        out[3] = a;
    }
};

}  // namespace orc
