// env_cube.cu — the environment luminance cube map (include/skyr_environment.h):
// the ENVIRONMENT_LUMINANCE program per texel and the glGenerateTextureMipmap
// box-filter chain.
//
// The reference dispatches one invocation per texel of a 128^2 x 6 RGBA16F
// cube and lets the driver build the mips (AtmosphereRenderer.cpp:234-242).
// Here one block computes a 16 x 16 tile of level 0 and reduces it in shared
// memory to levels 1-4 (each level rounded to half before its children are
// averaged, as a chain of RGBA16F levels is); a second launch, one block per
// face, finishes the levels below the tile size.
#include <cstring>

#include <cuda_fp16.h>

#include "../../include/skyr_environment.h"
#include "environment.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace {

constexpr int kTile = 16;     // level-0 texels per block side
constexpr int kMaxFace = 512;  // face sizes 1..512, powers of two

int log2i(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

__host__ __device__ inline size_t level_offset(int size, int level) {
    size_t off = 0;
    for (int l = 0; l < level; ++l) {
        size_t s = (size_t)((size >> l) > 0 ? (size >> l) : 1);
        off += 6 * s * s;
    }
    return off;
}

// ConvertCubUvToDir (shaders/Base/Common.glsl:13-30)
__device__ __forceinline__ float3 cube_dir(int face, float u, float v) {
    float uc = 2.f * u - 1.f, vc = 2.f * v - 1.f;
    float3 d;
    switch (face) {
        case 0: d = f3(1.f, vc, -uc); break;
        case 1: d = f3(-1.f, vc, uc); break;
        case 2: d = f3(uc, 1.f, -vc); break;
        case 3: d = f3(uc, -1.f, vc); break;
        case 4: d = f3(uc, vc, 1.f); break;
        default: d = f3(-uc, vc, -1.f); break;
    }
    return d * rsqrtf(dot3(d, d));
}

__device__ __forceinline__ float4 round_half4(float4 v) {
    return make_float4(__half2float(__float2half_rn(v.x)), __half2float(__float2half_rn(v.y)),
                       __half2float(__float2half_rn(v.z)), __half2float(__float2half_rn(v.w)));
}

__device__ __forceinline__ void store_half4(uint2* p, size_t i, float4 v) {
    __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, v.w);
    uint2 raw;
    raw.x = *reinterpret_cast<uint32_t*>(&lo);
    raw.y = *reinterpret_cast<uint32_t*>(&hi);
    p[i] = raw;
}

__device__ __forceinline__ float4 avg4(float4 a, float4 b, float4 c, float4 d) {
    // GL's box filter of four texels; exact in FP32 for half inputs
    return make_float4(((a.x + b.x) + (c.x + d.x)) * 0.25f, ((a.y + b.y) + (c.y + d.y)) * 0.25f,
                       ((a.z + b.z) + (c.z + d.z)) * 0.25f, ((a.w + b.w) + (c.w + d.w)) * 0.25f);
}

// Level 0 (AtmosphereRenderer.glsl:250-273) and levels 1..last_level of the block's tile.
template <class S>
__global__ void __launch_bounds__(kTile* kTile) env_cube_kernel(AtmoConsts A, ViewConsts E,
                                                                 const float4* __restrict__ tlut, int tw, int th,
                                                                 const S* __restrict__ svl,
                                                                 const S* __restrict__ svt, int sv_w, int sv_h,
                                                                 int size, int last_level, uint2* __restrict__ out) {
    __shared__ float4 tile[kTile][kTile];
    const int t = blockDim.x;  // tile side (<= kTile)
    const int face = blockIdx.z;
    const int x = blockIdx.x * t + threadIdx.x, y = blockIdx.y * t + threadIdx.y;
    float u = ((float)x + 0.5f) / (float)size;
    float v = 1.f - ((float)y + 0.5f) / (float)size;
    float3 w = cube_dir(face, u, v);
    float3 lum = environment(A, E, tlut, tw, th, svl, svt, sv_w, sv_h, w);
    float4 c = round_half4(make_float4(lum.x, lum.y, lum.z, 0.f));
    store_half4(out, ((size_t)face * size + y) * size + x, c);
    tile[threadIdx.y][threadIdx.x] = c;
    int s = t;
    for (int l = 1; l <= last_level && s > 1; ++l) {
        __syncthreads();
        s >>= 1;
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        bool active = threadIdx.x < s && threadIdx.y < s;
        if (active) {
            int ax = 2 * threadIdx.x, ay = 2 * threadIdx.y;
            r = round_half4(avg4(tile[ay][ax], tile[ay][ax + 1], tile[ay + 1][ax], tile[ay + 1][ax + 1]));
            int sl = size >> l;
            int gx = blockIdx.x * s + threadIdx.x, gy = blockIdx.y * s + threadIdx.y;
            store_half4(out, level_offset(size, l) + ((size_t)face * sl + gy) * sl + gx, r);
        }
        __syncthreads();
        if (active) tile[threadIdx.y][threadIdx.x] = r;
    }
}

// Levels first_level..last_level of one face from level first_level - 1
// (side n = size >> (first_level - 1) <= 32), one block of n x n threads.
__global__ void __launch_bounds__(1024) env_mip_kernel(int size, int first_level, int last_level,
                                                       uint2* __restrict__ out) {
    __shared__ float4 tile[32][32];
    const int face = blockIdx.x;
    int s = size >> (first_level - 1);
    const int tx = threadIdx.x, ty = threadIdx.y;
    {
        uint2 raw = out[level_offset(size, first_level - 1) + ((size_t)face * s + ty) * s + tx];
        float2 a = __half22float2(*reinterpret_cast<__half2*>(&raw.x));
        float2 b = __half22float2(*reinterpret_cast<__half2*>(&raw.y));
        tile[ty][tx] = make_float4(a.x, a.y, b.x, b.y);
    }
    for (int l = first_level; l <= last_level; ++l) {
        __syncthreads();
        s >>= 1;
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        bool active = tx < s && ty < s;
        if (active) {
            r = round_half4(avg4(tile[2 * ty][2 * tx], tile[2 * ty][2 * tx + 1], tile[2 * ty + 1][2 * tx],
                                 tile[2 * ty + 1][2 * tx + 1]));
            store_half4(out, level_offset(size, l) + ((size_t)face * s + ty) * s + tx, r);
        }
        __syncthreads();
        if (active) tile[ty][tx] = r;
    }
}

// ---------------------------------------------------------------------------
// Cube sampling with TEXTURE_CUBE_MAP_SEAMLESS (GL 4.6 sections 8.13, 8.14)
// ---------------------------------------------------------------------------
// Face and (s, t) of a direction (GL 4.6 table 8.19); ties go to x, then y.
__device__ __forceinline__ int cube_face(float3 d, float& s, float& t) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        face = d.x >= 0.f ? 0 : 1;
        sc = d.x >= 0.f ? -d.z : d.z;
        tc = -d.y;
    } else if (ay >= az) {
        ma = ay;
        face = d.y >= 0.f ? 2 : 3;
        sc = d.x;
        tc = d.y >= 0.f ? d.z : -d.z;
    } else {
        ma = az;
        face = d.z >= 0.f ? 4 : 5;
        sc = d.z >= 0.f ? d.x : -d.x;
        tc = -d.y;
    }
    s = 0.5f * (sc / ma + 1.f);
    t = 0.5f * (tc / ma + 1.f);
    return face;
}

// direction of the centre of texel (i, j) of face `face` (one texel past an edge allowed)
__device__ __forceinline__ float3 texel_dir(int face, int i, int j, int n) {
    float sc = 2.f * ((float)i + 0.5f) / (float)n - 1.f, tc = 2.f * ((float)j + 0.5f) / (float)n - 1.f;
    switch (face) {
        case 0: return f3(1.f, -tc, -sc);
        case 1: return f3(-1.f, -tc, sc);
        case 2: return f3(sc, 1.f, tc);
        case 3: return f3(sc, -1.f, -tc);
        case 4: return f3(sc, -tc, 1.f);
        default: return f3(-sc, -tc, -1.f);
    }
}

__device__ __forceinline__ float4 cube_load(const uint2* lvl, int n, int face, int i, int j) {
    uint2 raw = __ldg(lvl + ((size_t)face * n + j) * n + i);
    float2 a = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    float2 b = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

// a texel of the adjacent face through the direction of (i, j)'s centre
__device__ __forceinline__ float4 cube_neighbour(const uint2* lvl, int n, int face, int i, int j) {
    float s, t;
    int f = cube_face(texel_dir(face, i, j, n), s, t);
    int i2 = min(max((int)floorf(s * (float)n), 0), n - 1), j2 = min(max((int)floorf(t * (float)n), 0), n - 1);
    return cube_load(lvl, n, f, i2, j2);
}

__device__ __forceinline__ float4 cube_texel(const uint2* lvl, int n, int face, int i, int j) {
    bool oi = (unsigned)i >= (unsigned)n, oj = (unsigned)j >= (unsigned)n;
    if (!oi && !oj) return cube_load(lvl, n, face, i, j);
    if (oi && oj) {  // past a corner: the mean of the three texels that meet there
        int ci = min(max(i, 0), n - 1), cj = min(max(j, 0), n - 1);
        float4 a = cube_load(lvl, n, face, ci, cj), b = cube_neighbour(lvl, n, face, i, cj),
               c = cube_neighbour(lvl, n, face, ci, j);
        return make_float4((a.x + b.x + c.x) * (1.f / 3.f), (a.y + b.y + c.y) * (1.f / 3.f),
                           (a.z + b.z + c.z) * (1.f / 3.f), (a.w + b.w + c.w) * (1.f / 3.f));
    }
    return cube_neighbour(lvl, n, face, i, j);
}

__host__ __device__ inline size_t seamless_offset(int size, int level) {
    size_t off = 0;
    for (int l = 0; l < level; ++l) {
        size_t s = (size_t)((size >> l) > 0 ? (size >> l) : 1) + 2;
        off += 6 * s * s;
    }
    return off;
}

// The seamless copy: every texel of every level, apron included.
__global__ void __launch_bounds__(256) env_seamless_kernel(const uint2* __restrict__ cube, int size, int levels,
                                                           float4* __restrict__ out) {
    const size_t total = seamless_offset(size, levels);
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        int l = 0;
        while (l + 1 < levels && seamless_offset(size, l + 1) <= k) ++l;
        const int n = max(size >> l, 1), m = n + 2;
        size_t r = k - seamless_offset(size, l);
        const int face = (int)(r / ((size_t)m * m));
        r -= (size_t)face * m * m;
        const int j = (int)(r / m) - 1, i = (int)(r % m) - 1;
        out[k] = cube_texel(cube + level_offset(size, l), n, face, i, j);
    }
}

// GL LINEAR filtering of one level of the seamless copy (side n)
__device__ __forceinline__ float3 seamless_bilinear(const float4* lvl, int n, float3 d) {
    float s, t;
    const int face = cube_face(d, s, t);
    const int m = n + 2;
    float x = s * (float)n - 0.5f, y = t * (float)n - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float a = x - fx, b = y - fy;
    const float4* p = lvl + ((size_t)face * m + (int)fy + 1) * m + (int)fx + 1;  // taps i0, i0 + 1 in [-1, n]
    float4 t00 = __ldg(p), t10 = __ldg(p + 1), t01 = __ldg(p + m), t11 = __ldg(p + m + 1);
    float3 top = f3(t00.x + (t10.x - t00.x) * a, t00.y + (t10.y - t00.y) * a, t00.z + (t10.z - t00.z) * a);
    float3 bot = f3(t01.x + (t11.x - t01.x) * a, t01.y + (t11.y - t01.y) * a, t01.z + (t11.z - t01.z) * a);
    return top + (bot - top) * b;
}

struct Cube {
    const float4* base;  // the seamless copy
    int size, levels;
};

// textureLod with LINEAR / LINEAR_MIPMAP_LINEAR (magnified at lod <= 0)
__device__ __forceinline__ float3 cube_trilinear(const Cube& C, float3 d, float lod) {
    float q = (float)(C.levels - 1);
    float lam = fminf(fmaxf(lod, 0.f), q);
    int l0 = (int)floorf(lam);
    float f = lam - (float)l0;
    float3 a = seamless_bilinear(C.base + seamless_offset(C.size, l0), max(C.size >> l0, 1), d);
    if (f == 0.f || l0 + 1 > C.levels - 1) return a;
    float3 b = seamless_bilinear(C.base + seamless_offset(C.size, l0 + 1), max(C.size >> (l0 + 1), 1), d);
    return a + (b - a) * f;
}

// EnvRadianceSH.comp: block k sums coefficient k over 1024 directions in the
// shader's order (a halving tree in shared memory)
__global__ void __launch_bounds__(1024) env_sh_kernel(Cube C, float4* __restrict__ out) {
    __shared__ float3 acc[1024];
    const int k = blockIdx.x, i = threadIdx.x;
    // GetDirectionFromLocalIndex: uniform on the sphere, 32 x 32 strata
    float ut = (0.5f + (float)(i >> 5)) / 32.f, up = (0.5f + (float)(i & 31)) / 32.f;
    float ct = 1.f - 2.f * ut, st = sqrtf(fminf(fmaxf(1.f - ct * ct, 0.f), 1.f));
    float ph = 2.f * SKYR_PI * up;
    float3 d = f3(cosf(ph) * st, ct, sinf(ph) * st);
    float3 L = seamless_bilinear(C.base, C.size, d);
    float y;
    switch (k) {
        case 0: y = 0.282095f; break;
        case 1: y = 0.488603f * d.y; break;
        case 2: y = 0.488603f * d.z; break;
        case 3: y = 0.488603f * d.x; break;
        case 4: y = 1.092548f * d.x * d.y; break;
        case 5: y = 1.092548f * d.y * d.z; break;
        case 6: y = 0.315392f * (3.f * d.z * d.z - 1.f); break;
        case 7: y = 1.092548f * d.x * d.z; break;
        default: y = 0.546274f * (d.x * d.x - d.y * d.y); break;
    }
    acc[i] = L * (y * (4.f * SKYR_PI / 1024.f));
    for (int h = 512; h > 0; h >>= 1) {
        __syncthreads();
        if (i < h) acc[i] = acc[i] + acc[i + h];
    }
    if (i == 0) out[k] = make_float4(acc[0].x, acc[0].y, acc[0].z, 0.f);
}

__device__ __forceinline__ unsigned reverse_bits32(unsigned v) { return __brev(v); }

// PrefilterRadiance.comp for one level: side n, roughness r.  The level's
// Hammersley samples of a texel are spread over LANES adjacent lanes (sample i
// on lane i % LANES) and summed by shuffles, so that the coarse levels -- few
// texels, up to 64 samples each -- are not one serial chain of fetches.
template <int LANES>
__global__ void __launch_bounds__(256) env_prefilter_kernel(Cube C, int n, float roughness, uint2* __restrict__ out) {
    const int face = blockIdx.z;
    const int lane = threadIdx.x % LANES;
    const int texel = (blockIdx.x * blockDim.x + threadIdx.x) / LANES;
    const int x = texel % n, y = texel / n;
    const bool live = y < n;  // whole lane groups share this
    float u = ((float)x + 0.5f) / (float)n, v = 1.f - ((float)min(y, n - 1) + 0.5f) / (float)n;
    float3 R = cube_dir(face, u, v);
    // PrefilterEnvMap: N = V = R
    float a = roughness * roughness;
    const unsigned ns = (unsigned)(1.f + (64.f - 1.f) * powf(roughness, 0.3f));
    // CreateOrthonormalBasis (Pixar, shaders/Base/Common.glsl:45-50)
    float sg = R.z >= 0.f ? 1.f : -1.f;
    float ia = -1.f / (sg + R.z);
    float bb = R.x * R.y * ia;
    float3 t0 = f3(1.f + sg * R.x * R.x * ia, sg * bb, -sg * R.x);
    float3 t1 = f3(bb, sg + R.y * R.y * ia, -R.y);
    const float inv_sa_texel = (6.f * (float)n * (float)n) / (4.f * SKYR_PI);
    float3 col = f3(0.f, 0.f, 0.f);
    float wsum = 0.f;
    for (unsigned i = lane; live && i < ns; i += LANES) {
        // Hammersley(i, ns, 0) (shaders/Base/Noise.glsl:113-117)
        float e1 = (float)i / (float)ns;
        e1 = e1 - floorf(e1);
        float e2 = (float)__brev(i) * 2.3283064365386963e-10f;
        // ImportanceSampleGGX (shaders/Base/BRDF.glsl:48-67)
        float a2 = a * a;
        float phi = 2.f * SKYR_PI * e1;
        float cth = sqrtf((1.f - e2) / (1.f + (a2 - 1.f) * e2));
        float sth = sqrtf(1.f - cth * cth);
        float3 H = t0 * (sth * cosf(phi)) + t1 * (sth * sinf(phi)) + R * cth;
        float vh = dot3(R, H);
        float3 L = H * (2.f * vh) - R;
        float nol = fminf(fmaxf(dot3(R, L), 0.f), 1.f);
        if (nol > 0.f) {
            float noh = fminf(fmaxf(dot3(R, H), 0.f), 1.f), hov = fminf(fmaxf(vh, 0.f), 1.f);
            float dd = (noh * a2 - noh) * noh + 1.f;
            float D = a2 / (SKYR_PI * dd * dd);
            float pdf = fmaxf(D * noh / (4.f * hov), 0.0001f);
            float sa = 1.f / fmaxf((float)ns * pdf, 0.00001f);
            float lod = roughness == 0.f ? 0.f : 0.5f * log2f(sa * inv_sa_texel) + 2.5f;
            col = col + cube_trilinear(C, L, lod) * nol;
            wsum += nol;
        }
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) {
        col.x += __shfl_xor_sync(0xffffffffu, col.x, o, LANES);
        col.y += __shfl_xor_sync(0xffffffffu, col.y, o, LANES);
        col.z += __shfl_xor_sync(0xffffffffu, col.z, o, LANES);
        wsum += __shfl_xor_sync(0xffffffffu, wsum, o, LANES);
    }
    if (live && lane == 0) {
        col = col * (1.f / wsum);
        store_half4(out, ((size_t)face * n + y) * n + x, make_float4(col.x, col.y, col.z, 0.f));
    }
}

}  // namespace
}  // namespace skyr

using namespace skyr;

extern "C" {

size_t skyr_environment_cube_level_offset(int face_size, int level) {
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0) return 0;
    if (level < 0 || level > log2i(face_size) + 1) return 0;
    return level_offset(face_size, level);
}

int skyr_environment_cube(skyr_ctx* ctx, const skyr_atmosphere_parameters* atmosphere,
                          const skyr_atmosphere_render_parameters* render, const skyr_lut_sizes* sizes,
                          const void* transmittance, const void* sky_view_luminance,
                          const void* sky_view_transmittance, int face_size, int levels, void* out) {
    if (!ctx || !atmosphere || !render || !sizes) return set_error(SKYR_EINVAL, "null argument");
    if (!transmittance || !sky_view_luminance || !sky_view_transmittance || !out)
        return set_error(SKYR_EINVAL, "null LUT or output");
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0)
        return set_error(SKYR_EINVAL, "face size must be a power of two in [1, %d]", kMaxFace);
    const int max_levels = log2i(face_size) + 1;
    if (levels < 1 || levels > max_levels) return set_error(SKYR_EINVAL, "levels must be in [1, %d]", max_levels);
    if (int st = validate_atmosphere(atmosphere, 0)) return st;
    if (int st = validate_render(render, atmosphere, 0)) return st;
    if (int st = validate_sizes(sizes, true)) return st;
    AtmoConsts A;
    derive_atmo_consts(*atmosphere, A);
    ViewConsts E;
    derive_view_consts(*atmosphere, *render, E);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    cudaStream_t stream = ctx->stream;
    const int t = face_size < kTile ? face_size : kTile;
    const int tile_levels = log2i(t);  // levels 1..tile_levels come from the tile
    const int last = levels - 1;
    dim3 grid(face_size / t, face_size / t, 6), block(t, t);
    uint2* o = reinterpret_cast<uint2*>(out);
    const float4* T = reinterpret_cast<const float4*>(transmittance);
    const int tl = last < tile_levels ? last : tile_levels;
    if (sizes->format == SKYR_FORMAT_RGBA16F)
        env_cube_kernel<__half2><<<grid, block, 0, stream>>>(
            A, E, T, sizes->transmittance_width, sizes->transmittance_height,
            reinterpret_cast<const __half2*>(sky_view_luminance), reinterpret_cast<const __half2*>(sky_view_transmittance),
            sizes->sky_view_width, sizes->sky_view_height, face_size, tl, o);
    else
        env_cube_kernel<float4><<<grid, block, 0, stream>>>(
            A, E, T, sizes->transmittance_width, sizes->transmittance_height,
            reinterpret_cast<const float4*>(sky_view_luminance), reinterpret_cast<const float4*>(sky_view_transmittance),
            sizes->sky_view_width, sizes->sky_view_height, face_size, tl, o);
    if (int e = check_cuda(cudaGetLastError(), "environment cube kernel")) return e;
    if (last > tile_levels) {
        const int n = face_size >> tile_levels;  // side of the last tile-made level (<= 32)
        env_mip_kernel<<<6, dim3(n, n), 0, stream>>>(face_size, tile_levels + 1, last, o);
        if (int e = check_cuda(cudaGetLastError(), "environment mip kernel")) return e;
    }
    return SKYR_OK;
}

size_t skyr_environment_seamless_level_offset(int face_size, int level) {
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0) return 0;
    if (level < 0 || level > log2i(face_size) + 1) return 0;
    return seamless_offset(face_size, level);
}

int skyr_environment_seamless(skyr_ctx* ctx, const void* cube, int face_size, int levels, float* out) {
    if (!ctx || !cube || !out) return set_error(SKYR_EINVAL, "null argument");
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0)
        return set_error(SKYR_EINVAL, "face size must be a power of two in [1, %d]", kMaxFace);
    if (levels < 1 || levels > log2i(face_size) + 1) return set_error(SKYR_EINVAL, "bad level count %d", levels);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    const size_t total = seamless_offset(face_size, levels);
    const unsigned blocks = (unsigned)((total + 255) / 256 < 1216 ? (total + 255) / 256 : 1216);
    env_seamless_kernel<<<blocks, 256, 0, ctx->stream>>>(reinterpret_cast<const uint2*>(cube), face_size, levels,
                                                         reinterpret_cast<float4*>(out));
    return check_cuda(cudaGetLastError(), "environment seamless kernel");
}

int skyr_environment_sh(skyr_ctx* ctx, const float* cube, int face_size, int levels, float* out) {
    if (!ctx || !cube || !out) return set_error(SKYR_EINVAL, "null argument");
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0)
        return set_error(SKYR_EINVAL, "face size must be a power of two in [1, %d]", kMaxFace);
    if (levels < 1 || levels > log2i(face_size) + 1) return set_error(SKYR_EINVAL, "bad level count %d", levels);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    Cube C{reinterpret_cast<const float4*>(cube), face_size, levels};
    env_sh_kernel<<<9, 1024, 0, ctx->stream>>>(C, reinterpret_cast<float4*>(out));
    return check_cuda(cudaGetLastError(), "environment SH kernel");
}

int skyr_environment_prefilter(skyr_ctx* ctx, const float* cube, int face_size, int levels, int resolution,
                               int roughness_count, void* out) {
    if (!ctx || !cube || !out) return set_error(SKYR_EINVAL, "null argument");
    if (face_size < 1 || face_size > kMaxFace || (face_size & (face_size - 1)) != 0)
        return set_error(SKYR_EINVAL, "face size must be a power of two in [1, %d]", kMaxFace);
    if (levels < 1 || levels > log2i(face_size) + 1) return set_error(SKYR_EINVAL, "bad level count %d", levels);
    if (resolution < 1 || resolution > kMaxFace || (resolution & (resolution - 1)) != 0)
        return set_error(SKYR_EINVAL, "resolution must be a power of two in [1, %d]", kMaxFace);
    if (roughness_count < 2 || roughness_count > log2i(resolution) + 1)
        return set_error(SKYR_EINVAL, "roughness count must be in [2, %d]", log2i(resolution) + 1);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    Cube C{reinterpret_cast<const float4*>(cube), face_size, levels};
    uint2* o = reinterpret_cast<uint2*>(out);
    for (int k = 0; k < roughness_count; ++k) {
        const int n = resolution >> k;
        const float rough = (float)k / (float)(roughness_count - 1);
        // lanes per texel: enough for about 64 K threads, at most the level's sample
        // count (rounded up to a power of two) and 32
        const unsigned ns = (unsigned)(1.f + (64.f - 1.f) * powf(rough, 0.3f));
        int lanes = 1;
        while (lanes < (int)ns && lanes < 32 && (size_t)n * n * 6 * lanes < 65536) lanes <<= 1;
        const size_t threads = (size_t)n * n * lanes;
        dim3 grid((unsigned)((threads + 255) / 256), 1, 6);
        uint2* dst = o + level_offset(resolution, k);
        switch (lanes) {
            case 1: env_prefilter_kernel<1><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
            case 2: env_prefilter_kernel<2><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
            case 4: env_prefilter_kernel<4><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
            case 8: env_prefilter_kernel<8><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
            case 16: env_prefilter_kernel<16><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
            default: env_prefilter_kernel<32><<<grid, 256, 0, ctx->stream>>>(C, n, rough, dst); break;
        }
        if (int e = check_cuda(cudaGetLastError(), "environment prefilter kernel")) return e;
    }
    return SKYR_OK;
}

}  // extern "C"
