// noise.cu — procedural noise textures (NoiseGen.comp) and their mip chains,
// plus the seeded blue-noise tile generator (host).
//
// Generator semantics follow shaders/Base/Noise.glsl:1-101 and
// shaders/SkyRendering/NoiseGen.comp:12-105 of c52e/SkyRendering; one thread
// computes every channel of one texel.  Mip levels are 2^n box-filter
// reductions with round-to-nearest, one launch per level.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "../../include/skyr_cloud.h"
#include "skyr_ctx.cuh"
#include "skyr_internal.cuh"
#include "noise_device.cuh"

namespace skyr {

__global__ void __launch_bounds__(128) noise_level0_kernel(skyr_noise_texture_desc d, uint8_t* __restrict__ out) {
    size_t n = (size_t)d.width * d.height * d.depth;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int x = (int)(i % d.width), y = (int)((i / d.width) % d.height), z = (int)(i / ((size_t)d.width * d.height));
    float3 c = f3(((float)x + 0.5f) / (float)d.width, ((float)y + 0.5f) / (float)d.height,
                  d.depth > 1 ? ((float)z + 0.5f) / (float)d.depth : 0.f);
    for (int ch = 0; ch < d.channels; ++ch) {
        const skyr_noise_channel& g = d.channel[ch];
        float v = 0.f;
        if (g.kind == SKYR_NOISE_PERLIN || g.kind == SKYR_NOISE_WORLEY) {
            v = fbm(g.kind, c, g.a, d.octaves);
        } else if (g.kind == SKYR_NOISE_PERLIN_WORLEY) {
            float pe = fbm(SKYR_NOISE_PERLIN, c, g.a, d.octaves);
            float wo = fbm(SKYR_NOISE_WORLEY, c, g.b, d.octaves);
            v = clamp_ieee(wo + pe * (1.f - wo));  // RemapFrom01(perlin, worley, 1)
        }
        out[(size_t)ch * n + i] = (uint8_t)floorf(clamp_ieee(v) * 255.f + 0.5f);
    }
}

__global__ void __launch_bounds__(128) box_reduce_kernel(const uint8_t* __restrict__ src, int w, int h, int d,
                                                         uint8_t* __restrict__ dst, int channels) {
    int w2 = max(w >> 1, 1), h2 = max(h >> 1, 1), d2 = max(d >> 1, 1);
    size_t n2 = (size_t)w2 * h2 * d2;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2 * channels) return;
    int c = (int)(i / n2);
    size_t j = i % n2;
    int x = (int)(j % w2), y = (int)((j / w2) % h2), z = (int)(j / ((size_t)w2 * h2));
    int sx = w > 1 ? 2 : 1, sy = h > 1 ? 2 : 1, sz = d > 1 ? 2 : 1;
    const uint8_t* s = src + (size_t)c * w * h * d;
    unsigned sum = 0;
    for (int dz = 0; dz < sz; ++dz)
        for (int dy = 0; dy < sy; ++dy)
            for (int dx = 0; dx < sx; ++dx)
                sum += s[((size_t)(z * sz + dz) * h + (y * sy + dy)) * w + (x * sx + dx)];
    unsigned cnt = (unsigned)(sx * sy * sz);
    dst[(size_t)c * n2 + j] = (uint8_t)((sum + cnt / 2) / cnt);
}

// Level-0 corner expansion (skyr_noise_expand): REPEAT wrap, channel-planar.
__global__ void __launch_bounds__(256) expand2d_kernel(const uint8_t* __restrict__ tex, int w, int h, int channels,
                                                       uint32_t* __restrict__ out) {
    size_t n = (size_t)w * h;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * channels) return;
    int c = (int)(i / n);
    size_t j = i % n;
    int x = (int)(j % w), y = (int)(j / w);
    const uint8_t* t = tex + (size_t)c * n;
    int x1 = (x + 1) & (w - 1), y1 = (y + 1) & (h - 1);
    uint32_t v = (uint32_t)t[(size_t)y * w + x] | ((uint32_t)t[(size_t)y * w + x1] << 8) |
                 ((uint32_t)t[(size_t)y1 * w + x] << 16) | ((uint32_t)t[(size_t)y1 * w + x1] << 24);
    out[i] = v;
}

__global__ void __launch_bounds__(256) expand3d_kernel(const uint8_t* __restrict__ tex, int w, int h, int d,
                                                       int channels, unsigned long long* __restrict__ out) {
    size_t n = (size_t)w * h * d;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * channels) return;
    int c = (int)(i / n);
    size_t j = i % n;
    int x = (int)(j % w), y = (int)((j / w) % h), z = (int)(j / ((size_t)w * h));
    const uint8_t* t = tex + (size_t)c * n;
    unsigned long long v = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int xx = (x + (k & 1)) & (w - 1), yy = (y + ((k >> 1) & 1)) & (h - 1), zz = (z + (k >> 2)) & (d - 1);
        v |= (unsigned long long)t[((size_t)zz * h + yy) * w + xx] << (8 * k);
    }
    out[i] = v;
}

namespace {
bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
}  // namespace

int noise_levels(const skyr_noise_texture_desc* d) {
    int m = std::max(d->width, std::max(d->height, d->depth)), l = 1;
    while ((m >> l) > 0) ++l;
    return l;
}

size_t noise_level_offset(const skyr_noise_texture_desc* d, int level) {
    size_t off = 0;
    for (int l = 0; l < level; ++l)
        off += (size_t)std::max(d->width >> l, 1) * std::max(d->height >> l, 1) * std::max(d->depth >> l, 1) *
               d->channels;
    return off;
}

int validate_noise_desc(const skyr_noise_texture_desc* d, bool generator) {
    if (!d) return set_error(SKYR_EINVAL, "null noise texture descriptor");
    if (!pow2(d->width) || !pow2(d->height) || !pow2(d->depth) || d->width > 8192 || d->height > 8192 ||
        d->depth > 8192 || (size_t)d->width * d->height * d->depth > (size_t(1) << 31))
        return set_error(SKYR_EINVAL, "noise texture sizes must be powers of two <= 8192 (got %dx%dx%d)", d->width,
                         d->height, d->depth);
    if (d->channels < 1 || d->channels > 4) return set_error(SKYR_EINVAL, "noise texture channels must be 1..4");
    if (!generator) return SKYR_OK;
    if (d->octaves < 1 || d->octaves > 16) return set_error(SKYR_EINVAL, "fBm octaves must be 1..16");
    for (int c = 0; c < d->channels; ++c) {
        const skyr_noise_channel& g = d->channel[c];
        if (g.kind < SKYR_NOISE_PERLIN || g.kind > SKYR_NOISE_ZERO)
            return set_error(SKYR_EINVAL, "channel %d: unknown noise kind %d", c, g.kind);
        if (g.kind == SKYR_NOISE_ZERO) continue;
        int fa = g.a.base_frequency, fb = g.b.base_frequency;
        long long top_a = (long long)fa << (d->octaves - 1), top_b = (long long)fb << (d->octaves - 1);
        if (fa < 1 || top_a > (1 << 20) || (g.kind == SKYR_NOISE_PERLIN_WORLEY && (fb < 1 || top_b > (1 << 20))))
            return set_error(SKYR_EINVAL, "channel %d: base frequency must be >= 1 and its top octave <= 2^20", c);
    }
    return SKYR_OK;
}

// ---------------------------------------------------------------------------
// Void-and-cluster blue noise (Ulichney 1993): Gaussian energy (sigma 1.5) on
// a 64x64 torus; rank of insertion / removal -> (rank + 0.5) / 4096.
// ---------------------------------------------------------------------------
namespace {
struct VoidCluster {
    static constexpr int N = 64, NN = N * N;
    std::vector<float> lut;  // energy contribution by toroidal offset
    std::vector<float> energy;
    std::vector<uint8_t> on;
    VoidCluster() : lut(NN), energy(NN, 0.f), on(NN, 0) {
        const double s2 = 2.0 * 1.5 * 1.5;
        for (int dy = 0; dy < N; ++dy)
            for (int dx = 0; dx < N; ++dx) {
                int ex = std::min(dx, N - dx), ey = std::min(dy, N - dy);
                lut[dy * N + dx] = (float)std::exp(-(ex * ex + ey * ey) / s2);
            }
    }
    void add(int p, float sgn) {
        int px = p % N, py = p / N;
        for (int y = 0; y < N; ++y)
            for (int x = 0; x < N; ++x)
                energy[y * N + x] += sgn * lut[((y - py + N) % N) * N + ((x - px + N) % N)];
    }
    int tightest_cluster() const {  // max energy among ones
        int best = -1;
        for (int i = 0; i < NN; ++i)
            if (on[i] && (best < 0 || energy[i] > energy[best])) best = i;
        return best;
    }
    int largest_void() const {  // min energy among zeros
        int best = -1;
        for (int i = 0; i < NN; ++i)
            if (!on[i] && (best < 0 || energy[i] < energy[best])) best = i;
        return best;
    }
};
}  // namespace

}  // namespace skyr

using namespace skyr;

extern "C" {

int skyr_noise_texture_levels(const skyr_noise_texture_desc* desc) {
    if (validate_noise_desc(desc, false)) return 0;
    return noise_levels(desc);
}

size_t skyr_noise_level_offset(const skyr_noise_texture_desc* desc, int level) {
    if (validate_noise_desc(desc, false)) return 0;
    return noise_level_offset(desc, std::min(std::max(level, 0), noise_levels(desc)));
}

int skyr_noise_generate(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, void* out) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (int st = validate_noise_desc(desc, true)) return st;
    if (!out) return set_error(SKYR_EINVAL, "null output texture");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    uint8_t* o = reinterpret_cast<uint8_t*>(out);
    size_t n = (size_t)desc->width * desc->height * desc->depth;
    noise_level0_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(*desc, o);
    if (int e = check_cuda(cudaGetLastError(), "noise generator kernel")) return e;
    int L = noise_levels(desc);
    for (int l = 0; l + 1 < L; ++l) {
        int w = std::max(desc->width >> l, 1), h = std::max(desc->height >> l, 1), d = std::max(desc->depth >> l, 1);
        size_t n2 = (size_t)std::max(w >> 1, 1) * std::max(h >> 1, 1) * std::max(d >> 1, 1) * desc->channels;
        box_reduce_kernel<<<(unsigned)((n2 + 127) / 128), 128, 0, ctx->stream>>>(
            o + noise_level_offset(desc, l), w, h, d, o + noise_level_offset(desc, l + 1), desc->channels);
        if (int e = check_cuda(cudaGetLastError(), "mip kernel")) return e;
    }
    return SKYR_OK;
}

size_t skyr_noise_expanded_bytes(const skyr_noise_texture_desc* desc, int channels) {
    if (validate_noise_desc(desc, false) || channels < 1 || channels > desc->channels) return 0;
    size_t n = (size_t)desc->width * desc->height * desc->depth * channels;
    return n * (desc->depth > 1 ? 8 : 4);
}

int skyr_noise_expand(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, const void* tex, int channels,
                      void* out) {
    if (!ctx) return set_error(SKYR_EINVAL, "null context");
    if (int st = validate_noise_desc(desc, false)) return st;
    if (!tex || !out) return set_error(SKYR_EINVAL, "null texture");
    if (channels < 1 || channels > desc->channels) return set_error(SKYR_EINVAL, "bad channel count %d", channels);
    if (desc->depth > 1 && (desc->width < 2 || desc->height < 2))
        return set_error(SKYR_EINVAL, "3D expansion needs width and height >= 2");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    size_t n = (size_t)desc->width * desc->height * desc->depth * channels;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const uint8_t* t = reinterpret_cast<const uint8_t*>(tex);
    if (desc->depth > 1)
        expand3d_kernel<<<blocks, 256, 0, ctx->stream>>>(t, desc->width, desc->height, desc->depth, channels,
                                                         reinterpret_cast<unsigned long long*>(out));
    else
        expand2d_kernel<<<blocks, 256, 0, ctx->stream>>>(t, desc->width, desc->height, channels,
                                                         reinterpret_cast<uint32_t*>(out));
    return check_cuda(cudaGetLastError(), "texture expansion kernel");
}

}  // extern "C"

struct skyr_noise_sampler {
    int device = 0;
    cudaArray_t array = nullptr;            // level 0: LINEAR filtering (magnification)
    cudaTextureObject_t tex = 0;
    cudaMipmappedArray_t mips = nullptr;    // every level: NEAREST at an explicit level (minification)
    cudaTextureObject_t tex_nearest = 0;
    skyr_noise_texture_desc desc{};
    int channel = 0;
};

namespace {
// Channel `channel` of level 0 of `tex` (channel-planar layout) into the sampler's array.
// Channel `channel` of level `level` of `tex` (per level channel-planar) into `dst`.
int level_copy(skyr_ctx* ctx, const skyr_noise_sampler* smp, const void* tex, int level, cudaArray_t dst) {
    const skyr_noise_texture_desc& d = smp->desc;
    const int w = std::max(d.width >> level, 1), h = std::max(d.height >> level, 1),
              dp = std::max(d.depth >> level, 1);
    const size_t plane = (size_t)w * h * dp;
    cudaMemcpy3DParms cp{};
    cp.srcPtr = make_cudaPitchedPtr(const_cast<uint8_t*>(reinterpret_cast<const uint8_t*>(tex)) +
                                        noise_level_offset(&d, level) + smp->channel * plane,
                                    (size_t)w, (size_t)w, (size_t)h);
    cp.dstArray = dst;
    cp.extent = make_cudaExtent((size_t)w, (size_t)h, d.depth > 1 ? (size_t)dp : 1);
    cp.kind = cudaMemcpyDeviceToDevice;
    return check_cuda(cudaMemcpy3DAsync(&cp, ctx->stream), "copy into the noise sampler");
}

// Level 0 into the LINEAR array, every level into the mipmapped array.
int sampler_copy(skyr_ctx* ctx, skyr_noise_sampler* smp, const void* tex) {
    if (int e = level_copy(ctx, smp, tex, 0, smp->array)) return e;
    const int levels = noise_levels(&smp->desc);
    for (int l = 0; l < levels; ++l) {
        cudaArray_t a = nullptr;
        if (int e = check_cuda(cudaGetMipmappedArrayLevel(&a, smp->mips, (unsigned)l), "mipmapped array level"))
            return e;
        if (int e = level_copy(ctx, smp, tex, l, a)) return e;
    }
    return SKYR_OK;
}
}  // namespace

extern "C" {

int skyr_noise_sampler_destroy(skyr_noise_sampler* sampler) {
    if (!sampler) return SKYR_OK;
    cudaSetDevice(sampler->device);
    int st = SKYR_OK;
    if (sampler->tex) st = check_cuda(cudaDestroyTextureObject(sampler->tex), "cudaDestroyTextureObject");
    if (sampler->tex_nearest) {
        int e = check_cuda(cudaDestroyTextureObject(sampler->tex_nearest), "cudaDestroyTextureObject");
        if (!st) st = e;
    }
    if (sampler->array) {
        int e = check_cuda(cudaFreeArray(sampler->array), "cudaFreeArray");
        if (!st) st = e;
    }
    if (sampler->mips) {
        int e = check_cuda(cudaFreeMipmappedArray(sampler->mips), "cudaFreeMipmappedArray");
        if (!st) st = e;
    }
    delete sampler;
    return st;
}

int skyr_noise_sampler_create(skyr_ctx* ctx, const skyr_noise_texture_desc* desc, const void* tex, int channel,
                              skyr_noise_sampler** out) {
    if (!ctx || !out) return set_error(SKYR_EINVAL, "null argument");
    *out = nullptr;
    if (int st = validate_noise_desc(desc, false)) return st;
    if (!tex) return set_error(SKYR_EINVAL, "null texture");
    if (channel < 0 || channel >= desc->channels) return set_error(SKYR_EINVAL, "bad channel %d", channel);
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    auto* smp = new (std::nothrow) skyr_noise_sampler;
    if (!smp) return set_error(SKYR_ENOMEM, "out of host memory");
    smp->device = ctx->device;
    smp->desc = *desc;
    smp->channel = channel;
    const bool d3 = desc->depth > 1;
    cudaChannelFormatDesc fmt = cudaCreateChannelDesc<unsigned char>();
    cudaExtent ext = make_cudaExtent((size_t)desc->width, (size_t)desc->height, d3 ? (size_t)desc->depth : 0);
    const int levels = noise_levels(desc);
    int e = check_cuda(cudaMalloc3DArray(&smp->array, &fmt, ext, 0), "cudaMalloc3DArray(noise sampler)");
    if (!e)
        e = check_cuda(cudaMallocMipmappedArray(&smp->mips, &fmt, ext, (unsigned)levels, 0),
                       "cudaMallocMipmappedArray(noise sampler)");
    if (!e) e = sampler_copy(ctx, smp, tex);
    if (!e) {
        cudaResourceDesc rd{};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = smp->array;
        cudaTextureDesc td{};
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;  // GL REPEAT
        td.filterMode = cudaFilterModeLinear;                                              // GL LINEAR
        td.readMode = cudaReadModeNormalizedFloat;                                         // UNORM8
        td.normalizedCoords = 1;
        e = check_cuda(cudaCreateTextureObject(&smp->tex, &rd, &td, nullptr), "cudaCreateTextureObject");
    }
    if (!e) {
        // GL NEAREST_MIPMAP_NEAREST at a level the caller chooses (tex*Lod with an integer level)
        cudaResourceDesc rd{};
        rd.resType = cudaResourceTypeMipmappedArray;
        rd.res.mipmap.mipmap = smp->mips;
        cudaTextureDesc td{};
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;  // GL REPEAT
        td.filterMode = cudaFilterModePoint;
        td.mipmapFilterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;                                             // the byte itself
        td.normalizedCoords = 1;
        td.minMipmapLevelClamp = 0.f;
        td.maxMipmapLevelClamp = (float)(levels - 1);
        e = check_cuda(cudaCreateTextureObject(&smp->tex_nearest, &rd, &td, nullptr), "cudaCreateTextureObject");
    }
    if (e) {
        skyr_noise_sampler_destroy(smp);
        return e;
    }
    *out = smp;
    return SKYR_OK;
}

int skyr_noise_sampler_update(skyr_ctx* ctx, skyr_noise_sampler* sampler, const void* tex) {
    if (!ctx || !sampler || !tex) return set_error(SKYR_EINVAL, "null argument");
    if (sampler->device != ctx->device) return set_error(SKYR_EINVAL, "sampler of another device");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    return sampler_copy(ctx, sampler, tex);
}

uint64_t skyr_noise_sampler_handle(const skyr_noise_sampler* sampler) {
    return sampler ? (uint64_t)sampler->tex : 0;
}

uint64_t skyr_noise_sampler_nearest_handle(const skyr_noise_sampler* sampler) {
    return sampler ? (uint64_t)sampler->tex_nearest : 0;
}

int skyr_blue_noise_generate(uint32_t seed, float* out) {
    if (!out) return set_error(SKYR_EINVAL, "null output");
    VoidCluster vc;
    const int NN = VoidCluster::NN;
    std::mt19937 rng(seed);
    // initial pattern: 10% of the pixels, then relax by swapping the tightest
    // cluster into the largest void until they coincide
    int ones = NN / 10;
    std::vector<int> perm(NN);
    for (int i = 0; i < NN; ++i) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng);
    for (int i = 0; i < ones; ++i) {
        vc.on[perm[i]] = 1;
        vc.add(perm[i], 1.f);
    }
    for (int iter = 0; iter < 4 * NN; ++iter) {
        int c = vc.tightest_cluster();
        vc.on[c] = 0;
        vc.add(c, -1.f);
        int v = vc.largest_void();
        vc.on[v] = 1;
        vc.add(v, 1.f);
        if (v == c) break;
    }
    std::vector<int> rank(NN, -1);
    std::vector<uint8_t> proto = vc.on;
    std::vector<float> proto_e = vc.energy;
    // phase 1: ranks below `ones` by removing tightest clusters
    for (int r = ones - 1; r >= 0; --r) {
        int c = vc.tightest_cluster();
        vc.on[c] = 0;
        vc.add(c, -1.f);
        rank[c] = r;
    }
    // phase 2/3: ranks from `ones` up by filling the largest voids
    vc.on = proto;
    vc.energy = proto_e;
    for (int r = ones; r < NN; ++r) {
        int v = vc.largest_void();
        vc.on[v] = 1;
        vc.add(v, 1.f);
        rank[v] = r;
    }
    for (int i = 0; i < NN; ++i) out[i] = ((float)rank[i] + 0.5f) / (float)NN;
    return SKYR_OK;
}

}  // extern "C"
