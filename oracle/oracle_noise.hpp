// oracle_noise.hpp — TEST INFRASTRUCTURE ONLY.
//
// Restatement of the procedural noise of c52e/SkyRendering:
//   shaders/Base/Noise.glsl:1-101 (WangHash, PCGHash, periodic Perlin,
//   Worley 3D), shaders/SkyRendering/NoiseGen.comp:12-105 (fBm, remaps and the
//   DISPLACEMENT / CLOUD_MAP / DETAIL_MAP generators), plus the UNORM8 store of
//   imageStore and a 2^n box-filter mip chain standing in for
//   glGenerateTextureMipmap.  Integer hashing is bit-exact; the noise values
//   are computed in the scalar type T.
// Parity status: unpinned (see oracle_math.hpp).
#pragma once

#include <cstdint>
#include <vector>

#include "../include/skyr_cloud.h"
#include "oracle_math.hpp"

namespace orc {

// Noise.glsl:1-8
inline uint32_t WangHash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

// Noise.glsl:10-15
inline uint32_t PCGHash(uint32_t seed) {
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// kPerlinGradients (Noise.glsl:17-22)
static const int kGrad[16][3] = {{1, 1, 0},  {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1},
                                 {1, 0, -1}, {-1, 0, -1}, {0, 1, 1}, {0, -1, 1},  {0, 1, -1}, {0, -1, -1},
                                 {1, 1, 0},  {-1, 1, 0}, {0, -1, 1}, {0, -1, -1}};

inline int perlin_gradient_index(uint32_t i, uint32_t j, uint32_t k, uint32_t seed) {
    return (int)(WangHash(seed + WangHash(i + WangHash(j + WangHash(k)))) & 0xfu);
}

// GLSL uvec3(ivec3(floor(p))) % freq with p >= 0
inline uint32_t wrap_index(double f, uint32_t freq) { return (uint32_t)(int32_t)f % freq; }

// PerlinNoise (Noise.glsl:28-60)
template <class T>
T PerlinNoise(V3<T> p, uint32_t freq, uint32_t seed) {
    p = p * T(freq);
    V3<T> fl(std::floor(p.x), std::floor(p.y), std::floor(p.z));
    V3<T> ce(std::ceil(p.x), std::ceil(p.y), std::ceil(p.z));
    uint32_t i0 = wrap_index(fl.x, freq), j0 = wrap_index(fl.y, freq), k0 = wrap_index(fl.z, freq);
    uint32_t i1 = wrap_index(ce.x, freq), j1 = wrap_index(ce.y, freq), k1 = wrap_index(ce.z, freq);
    V3<T> t = p - fl;
    auto fade = [](T x) { return x * x * x * (x * (x * T(6) - T(15)) + T(10)); };
    T u = fade(t.x), v = fade(t.y), w = fade(t.z);
    T x0 = t.x, y0 = t.y, z0 = t.z, x1 = t.x - T(1), y1 = t.y - T(1), z1 = t.z - T(1);
    auto g = [&](uint32_t i, uint32_t j, uint32_t k, T x, T y, T z) {
        const int* gr = kGrad[perlin_gradient_index(i, j, k, seed)];
        return T(gr[0]) * x + T(gr[1]) * y + T(gr[2]) * z;
    };
    return mixg(mixg(mixg(g(i0, j0, k0, x0, y0, z0), g(i1, j0, k0, x1, y0, z0), u),
                     mixg(g(i0, j1, k0, x0, y1, z0), g(i1, j1, k0, x1, y1, z0), u), v),
                mixg(mixg(g(i0, j0, k1, x0, y0, z1), g(i1, j0, k1, x1, y0, z1), u),
                     mixg(g(i0, j1, k1, x0, y1, z1), g(i1, j1, k1, x1, y1, z1), u), v),
                w);
}

// WorleyNoise, 3D (Noise.glsl:81-101)
template <class T>
T WorleyNoise(V3<T> p, uint32_t freq, uint32_t seed) {
    p = p * T(freq);
    uint32_t ijk[3] = {(uint32_t)std::floor(p.x), (uint32_t)std::floor(p.y), (uint32_t)std::floor(p.z)};
    p = p + V3<T>(T(freq));
    T min_dist = T(1e10);
    for (uint32_t di = freq - 1; di <= freq + 1; ++di)
        for (uint32_t dj = freq - 1; dj <= freq + 1; ++dj)
            for (uint32_t dk = freq - 1; dk <= freq + 1; ++dk) {
                uint32_t g[3] = {ijk[0] + di, ijk[1] + dj, ijk[2] + dk};
                uint32_t gs[3] = {g[0] % freq, g[1] % freq, g[2] % freq};
                uint32_t r0 = WangHash(seed + WangHash(gs[0] + WangHash(gs[1] + WangHash(gs[2]))));
                uint32_t r1 = WangHash(seed + WangHash(gs[0] + WangHash(gs[1] + WangHash(gs[2] + 1u))));
                uint32_t r2 = WangHash(seed + WangHash(gs[0] + WangHash(gs[1] + WangHash(gs[2] + 2u))));
                V3<T> c(T(g[0]) + T(r0) / T(4294967296.0), T(g[1]) + T(r1) / T(4294967296.0),
                        T(g[2]) + T(r2) / T(4294967296.0));
                min_dist = std::min(min_dist, length(p - c));
            }
    return min_dist;
}

// RemapTo01 / RemapFrom01 (NoiseGen.comp:12-18).  clamp is taken with IEEE
// fmin/fmax, so a 0/0 remap (remap_min == remap_max) maps to 0.
template <class T> T clamp_ieee(T x) { return std::fmin(std::fmax(x, T(0)), T(1)); }
template <class T> T RemapTo01(T x, T x0, T x1) { return clamp_ieee((x - x0) / (x1 - x0)); }
template <class T> T RemapFrom01(T x, T y0, T y1) { return clamp_ieee(y0 + x * (y1 - y0)); }

// PerlinFBM / WorleyFBM (NoiseGen.comp:20-50) with a configurable octave count
template <class T>
T FBM(int kind, V3<T> p, const skyr_noise_create_info& ci, int octaves) {
    T res = 0, a = T(0.5), sum_a = 0;
    uint32_t f = (uint32_t)ci.base_frequency;
    for (int c = 0; c < octaves; ++c) {
        T n = kind == SKYR_NOISE_PERLIN ? PerlinNoise(p, f, (uint32_t)ci.seed) * T(0.5) + T(0.5)
                                        : WorleyNoise(p, f, (uint32_t)ci.seed);
        res += RemapTo01(n, T(ci.remap_min), T(ci.remap_max)) * a;
        sum_a += a;
        f *= 2u;
        a *= T(0.5);
    }
    return res / sum_a;
}

// One channel value of a generator at texel coordinate (x, y, z) of a w x h x d
// image: coord = (index + 0.5) / size (NoiseGen.comp:62-105).
template <class T>
T channel_value(const skyr_noise_channel& ch, int x, int y, int z, int w, int h, int d, int octaves) {
    V3<T> c((T(x) + T(0.5)) / T(w), (T(y) + T(0.5)) / T(h), d > 1 ? (T(z) + T(0.5)) / T(d) : T(0));
    switch (ch.kind) {
        case SKYR_NOISE_PERLIN: return FBM<T>(SKYR_NOISE_PERLIN, c, ch.a, octaves);
        case SKYR_NOISE_WORLEY: return FBM<T>(SKYR_NOISE_WORLEY, c, ch.a, octaves);
        case SKYR_NOISE_PERLIN_WORLEY: {
            T perlin = FBM<T>(SKYR_NOISE_PERLIN, c, ch.a, octaves);
            T worley = FBM<T>(SKYR_NOISE_WORLEY, c, ch.b, octaves);
            return RemapFrom01(perlin, worley, T(1));
        }
        default: return T(0);
    }
}

// imageStore into an UNORM8 image: round to nearest of clamp(v) * 255
template <class T>
uint8_t unorm8(T v) {
    T c = clamp_ieee(v);
    return (uint8_t)std::floor(c * T(255) + T(0.5));
}

// Box-filter reduction of one level (2x2 or 2x2x2 mean, rounded to nearest).
inline void box_reduce(const uint8_t* src, int w, int h, int d, uint8_t* dst, int channels) {
    int w2 = std::max(w / 2, 1), h2 = std::max(h / 2, 1), d2 = std::max(d / 2, 1);
    int sx = w > 1 ? 2 : 1, sy = h > 1 ? 2 : 1, sz = d > 1 ? 2 : 1;
    for (int c = 0; c < channels; ++c)
        for (int z = 0; z < d2; ++z)
            for (int y = 0; y < h2; ++y)
                for (int x = 0; x < w2; ++x) {
                    unsigned sum = 0;
                    for (int dz = 0; dz < sz; ++dz)
                        for (int dy = 0; dy < sy; ++dy)
                            for (int dx = 0; dx < sx; ++dx)
                                sum += src[(size_t)c * w * h * d +
                                           ((size_t)(z * sz + dz) * h + (y * sy + dy)) * w + (x * sx + dx)];
                    unsigned n = (unsigned)(sx * sy * sz);
                    dst[(size_t)c * w2 * h2 * d2 + ((size_t)z * h2 + y) * w2 + x] = (uint8_t)((sum + n / 2) / n);
                }
}

}  // namespace orc
