// noise_device.cuh — device noise functions shared by the texture generators
// and the synthetic density-grid generator: WangHash / PCGHash, periodic
// Perlin, Worley 3D and fBm (shaders/Base/Noise.glsl:1-101,
// shaders/SkyRendering/NoiseGen.comp:12-50).
#pragma once

#include "../../include/skyr_cloud.h"
#include "skyr_internal.cuh"

namespace skyr {

__host__ __device__ __forceinline__ uint32_t wang_hash(uint32_t seed) {  // Noise.glsl:1-8
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t seed) {  // Noise.glsl:10-15
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// kPerlinGradients (Noise.glsl:17-22)
static __constant__ int8_t kGradTable[16][3] = {{1, 1, 0},  {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1},
                                         {1, 0, -1}, {-1, 0, -1}, {0, 1, 1}, {0, -1, 1},  {0, 1, -1}, {0, -1, -1},
                                         {1, 1, 0},  {-1, 1, 0}, {0, -1, 1}, {0, -1, -1}};

__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.f - t) + b * t; }

// PerlinNoise (Noise.glsl:28-60)
__device__ inline float perlin(float3 p, uint32_t freq, uint32_t seed) {
    float ff = (float)freq;
    p = p * ff;
    float3 fl = f3(floorf(p.x), floorf(p.y), floorf(p.z));
    uint32_t i0 = (uint32_t)(int)fl.x % freq, j0 = (uint32_t)(int)fl.y % freq, k0 = (uint32_t)(int)fl.z % freq;
    uint32_t i1 = (uint32_t)(int)ceilf(p.x) % freq, j1 = (uint32_t)(int)ceilf(p.y) % freq,
             k1 = (uint32_t)(int)ceilf(p.z) % freq;
    float3 t = p - fl;
    auto fade = [](float x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); };
    float u = fade(t.x), v = fade(t.y), w = fade(t.z);
    float x0 = t.x, y0 = t.y, z0 = t.z, x1 = t.x - 1.f, y1 = t.y - 1.f, z1 = t.z - 1.f;
    auto g = [&](uint32_t i, uint32_t j, uint32_t k, float x, float y, float z) {
        int idx = (int)(wang_hash(seed + wang_hash(i + wang_hash(j + wang_hash(k)))) & 0xfu);
        return (float)kGradTable[idx][0] * x + (float)kGradTable[idx][1] * y + (float)kGradTable[idx][2] * z;
    };
    return mixf(mixf(mixf(g(i0, j0, k0, x0, y0, z0), g(i1, j0, k0, x1, y0, z0), u),
                     mixf(g(i0, j1, k0, x0, y1, z0), g(i1, j1, k0, x1, y1, z0), u), v),
                mixf(mixf(g(i0, j0, k1, x0, y0, z1), g(i1, j0, k1, x1, y0, z1), u),
                     mixf(g(i0, j1, k1, x0, y1, z1), g(i1, j1, k1, x1, y1, z1), u), v),
                w);
}

// WorleyNoise, 3D (Noise.glsl:81-101)
__device__ inline float worley(float3 p, uint32_t freq, uint32_t seed) {
    float ff = (float)freq;
    p = p * ff;
    uint32_t ix = (uint32_t)floorf(p.x), iy = (uint32_t)floorf(p.y), iz = (uint32_t)floorf(p.z);
    p = p + f3(ff);
    float min_d = 1e10f;
    for (uint32_t di = freq - 1; di <= freq + 1; ++di)
        for (uint32_t dj = freq - 1; dj <= freq + 1; ++dj)
            for (uint32_t dk = freq - 1; dk <= freq + 1; ++dk) {
                uint32_t gx = ix + di, gy = iy + dj, gz = iz + dk;
                uint32_t sx = gx % freq, sy = gy % freq, sz = gz % freq;
                uint32_t base = sx;
                uint32_t r0 = wang_hash(seed + wang_hash(base + wang_hash(sy + wang_hash(sz))));
                uint32_t r1 = wang_hash(seed + wang_hash(base + wang_hash(sy + wang_hash(sz + 1u))));
                uint32_t r2 = wang_hash(seed + wang_hash(base + wang_hash(sy + wang_hash(sz + 2u))));
                const float k = 1.f / 4294967296.f;
                float3 c = f3((float)gx + (float)r0 * k, (float)gy + (float)r1 * k, (float)gz + (float)r2 * k);
                float3 dd = p - c;
                min_d = fminf(min_d, sqrtf(dot3(dd, dd)));
            }
    return min_d;
}

__device__ __forceinline__ float clamp_ieee(float x) { return fminf(fmaxf(x, 0.f), 1.f); }

__device__ inline float fbm(int kind, float3 p, const skyr_noise_create_info& ci, int octaves) {
    float res = 0.f, a = 0.5f, sum_a = 0.f;
    uint32_t f = (uint32_t)ci.base_frequency;
    for (int c = 0; c < octaves; ++c) {
        float n = kind == SKYR_NOISE_PERLIN ? perlin(p, f, (uint32_t)ci.seed) * 0.5f + 0.5f
                                            : worley(p, f, (uint32_t)ci.seed);
        res += clamp_ieee((n - ci.remap_min) / (ci.remap_max - ci.remap_min)) * a;  // RemapTo01
        sum_a += a;
        f *= 2u;
        a *= 0.5f;
    }
    return res / sum_a;
}

}  // namespace skyr
