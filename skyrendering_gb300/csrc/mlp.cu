// mlp.cu — the surrogate network's kernels: packing, batched inference, the
// tensor-core gradient of the relative-L2 loss and the Adam update.
//
// Training step = two launches:
//  1. mlp_grad_kernel: one block of 4 warps per 128 samples.  The forward pass
//     stores every hidden activation (BF16) in shared memory; the backward pass
//     forms dZ per layer (BF16, shared memory) and computes the block's weight
//     gradient dW = dZ^T H as a 64x64x128 tensor-core product split over the
//     warps (ldmatrix.trans supplies the transposed operands), and dX = dZ W
//     with W read transposed.  Each block writes its partial gradient vector.
//  2. mlp_adam_kernel: sums the block partials in a fixed order (deterministic),
//     applies Adam to the FP32 master parameters and re-packs the BF16 weights.
#include <cmath>
#include <cstring>
#include <new>

#include "mlp_device.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace mlp {

constexpr int kWarps = 4;
constexpr int kTile = 32 * kWarps;  // samples per gradient block
constexpr int kMaxBatch = 65536;
constexpr int kMaxBlocks = kMaxBatch / kTile;

// shared memory of the gradient kernel
constexpr int kSmX = kPackedBytes;                   // X0 [128][kXS] bf16
constexpr int kSmH = kSmX + kTile * kXS * 2;         // H1..H4 [4][128][kSH] bf16
constexpr int kSmD = kSmH + 4 * kTile * kSH * 2;     // D0, D1 [2][128][kSH] bf16 (dZ)
constexpr int kBiasSlots = 4 * kW + 8;                        // bias gradients of one warp (f32)
constexpr int kSmBias = kSmD + 2 * kTile * kSH * 2;           // [kWarps][kBiasSlots] f32
constexpr int kSmLoss = kSmBias + kWarps * kBiasSlots * 4;    // [kWarps] f32
constexpr int kSmGrad = kSmLoss + 16;                         // 166208 bytes

// shared memory of the inference kernel: packed network + per warp a record
// tile [32][kXS] bf16 and its outputs [32][4] f32
constexpr int kSmInferWarp = 32 * kXS * 2 + 32 * 4 * 4;
constexpr int kSmInfer = kPackedBytes + kWarps * kSmInferWarp;

__device__ __forceinline__ float bias_at(const unsigned char* sw, int l, int j) {
    return reinterpret_cast<const float*>(sw + kOffB)[l * kW + j];
}

// byte address of parameter i in the packed network (bf16 weight or f32 bias)
__device__ __forceinline__ void pack_one(unsigned char* packed, int i, float val) {
    int l = 0;
#pragma unroll 1
    while (l < kLayers - 1 && i >= b_offset(l) + fan_out(l)) ++l;
    if (i < b_offset(l)) {
        int idx = i - w_offset(l), row = idx / fan_in(l), col = idx % fan_in(l);
        reinterpret_cast<__nv_bfloat16*>(packed + packed_w_offset(l))[row * packed_stride(l) + col] =
            __float2bfloat16_rn(val);
    } else {
        reinterpret_cast<float*>(packed + kOffB)[l * kW + (i - b_offset(l))] = val;
    }
}

__global__ void __launch_bounds__(256) mlp_pack_kernel(const float* __restrict__ params, float out_scale,
                                                       unsigned char* __restrict__ packed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < SKYR_MLP_PARAMS) pack_one(packed, i, params[i]);
    if (i == 0) *reinterpret_cast<float*>(packed + kOffScale) = out_scale;
}

__global__ void __launch_bounds__(128) mlp_infer_kernel(const unsigned char* __restrict__ packed,
                                                        const uint4* __restrict__ x, int n,
                                                        float* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char sm[];
    load_packed(sm, packed);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* xt = reinterpret_cast<__nv_bfloat16*>(sm + kPackedBytes + warp * kSmInferWarp);
    float* yt = reinterpret_cast<float*>(sm + kPackedBytes + warp * kSmInferWarp + 32 * kXS * 2);
    int tiles = (n + 31) / 32;
    for (int tile = blockIdx.x * kWarps + warp; tile < tiles; tile += gridDim.x * kWarps) {
        int s = tile * 32 + lane;
        // one record (6 x 16 B) per lane
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            uint4 v = s < n ? __ldg(x + (size_t)s * 6 + q) : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(xt + lane * kXS + q * 8) = v;
        }
        __syncwarp();
        forward_warp(sm, xt, yt);
        __syncwarp();
        if (s < n) {
            y[(size_t)s * 3 + 0] = yt[lane * 4 + 0];
            y[(size_t)s * 3 + 1] = yt[lane * 4 + 1];
            y[(size_t)s * 3 + 2] = yt[lane * 4 + 2];
        }
        __syncwarp();
    }
}

// Reduce a per-thread FP32 value over the 8 lanes sharing lane % 4.
__device__ __forceinline__ float sum_over_rows(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

__global__ void __launch_bounds__(128) mlp_grad_kernel(const unsigned char* __restrict__ packed,
                                                       const uint4* __restrict__ x, const float* __restrict__ tgt,
                                                       int n, float inv_scale, float loss_eps, float inv_count,
                                                       float* __restrict__ partial,
                                                       float* __restrict__ loss_partial) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int base = blockIdx.x * kTile;
    __nv_bfloat16* X0 = reinterpret_cast<__nv_bfloat16*>(sm + kSmX);
    __nv_bfloat16* H = reinterpret_cast<__nv_bfloat16*>(sm + kSmH);  // H[l] at H + l * kTile * kSH
    __nv_bfloat16* D = reinterpret_cast<__nv_bfloat16*>(sm + kSmD);  // D[b] at D + b * kTile * kSH
    // per-warp bias-gradient and loss slots, summed over the warps in a fixed
    // order at the end (no float atomics: the gradient is deterministic)
    float* sbias = reinterpret_cast<float*>(sm + kSmBias) + warp * kBiasSlots;
    float* sloss = reinterpret_cast<float*>(sm + kSmLoss);
    auto Hl = [&](int l) { return H + l * kTile * kSH; };
    auto Db = [&](int b) { return D + b * kTile * kSH; };
    auto W = [&](int l) { return reinterpret_cast<const __nv_bfloat16*>(sm + packed_w_offset(l)); };

    load_packed(sm, packed);
    for (int i = threadIdx.x; i < kTile * 6; i += blockDim.x) {
        int r = i / 6, q = i % 6, s = base + r;
        uint4 v = s < n ? __ldg(x + (size_t)s * 6 + q) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4*>(X0 + r * kXS + q * 8) = v;
    }
    for (int i = threadIdx.x; i < kWarps * kBiasSlots; i += blockDim.x)
        reinterpret_cast<float*>(sm + kSmBias)[i] = 0.f;
    if (threadIdx.x < kWarps) sloss[threadIdx.x] = 0.f;
    __syncthreads();

    const int row_w = warp * 32;
    // ---- forward: hidden layers, activations to shared memory ----
#pragma unroll 1
    for (int l = 0; l < 4; ++l) {
        const __nv_bfloat16* in = l == 0 ? X0 : Hl(l - 1);
        const int in_stride = l == 0 ? kXS : kSH, kts = l == 0 ? 3 : 4;
#pragma unroll 1
        for (int mt = 0; mt < 2; ++mt) {
            float acc[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float b0 = bias_at(sm, l, nt * 8 + 2 * t), b1 = bias_at(sm, l, nt * 8 + 2 * t + 1);
                acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
            }
#pragma unroll 1
            for (int kt = 0; kt < kts; ++kt) {
                uint32_t a[4];
                load_a(a, in, in_stride, row_w + mt * 16, kt * 16);
#pragma unroll
                for (int np = 0; np < 4; ++np) {
                    uint32_t b[4];
                    load_b_pair(b, W(l), packed_stride(l), np * 16, kt * 16);
                    mma(acc[2 * np], a, b[0], b[1]);
                    mma(acc[2 * np + 1], a, b[2], b[3]);
                }
            }
            __nv_bfloat16* out = Hl(l);
            int r = row_w + mt * 16 + g;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                int c = nt * 8 + 2 * t;
                *reinterpret_cast<uint32_t*>(out + r * kSH + c) =
                    pack_bf16(fmaxf(acc[nt][0], 0.f), fmaxf(acc[nt][1], 0.f));
                *reinterpret_cast<uint32_t*>(out + (r + 8) * kSH + c) =
                    pack_bf16(fmaxf(acc[nt][2], 0.f), fmaxf(acc[nt][3], 0.f));
            }
        }
        __syncwarp();
    }
    // ---- output layer, loss and dY ----
    {
        const __nv_bfloat16* w5 = W(4);
        float db0 = 0.f, db1 = 0.f, loss = 0.f;
#pragma unroll 1
        for (int mt = 0; mt < 2; ++mt) {
            float o[4];
            o[0] = bias_at(sm, 4, 2 * t); o[1] = bias_at(sm, 4, 2 * t + 1); o[2] = o[0]; o[3] = o[1];
#pragma unroll
            for (int kp = 0; kp < 2; ++kp) {
                uint32_t a0[4], a1[4], b[4];
                load_a(a0, Hl(3), kSH, row_w + mt * 16, kp * 32);
                load_a(a1, Hl(3), kSH, row_w + mt * 16, kp * 32 + 16);
                ldsm_x4(b, smem_u32(w5 + (lane & 7) * kSH + kp * 32 + (lane >> 3) * 8));
                mma(o, a0, b[0], b[1]);
                mma(o, a1, b[2], b[3]);
            }
            float dy[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int r = row_w + mt * 16 + g + (e >> 1) * 8, c = 2 * t + (e & 1), s = base + r;
                dy[e] = 0.f;
                if (c < kOut && s < n) {
                    float d = o[e] - __ldg(tgt + (size_t)s * 3 + c) * inv_scale;
                    float w = 1.f / (o[e] * o[e] + loss_eps);
                    loss += d * d * w * inv_count;
                    dy[e] = 2.f * d * w * inv_count;
                }
            }
            db0 += dy[0] + dy[2];
            db1 += dy[1] + dy[3];
            int r = row_w + mt * 16 + g;
            *reinterpret_cast<uint32_t*>(Db(0) + r * kSH + 2 * t) = pack_bf16(dy[0], dy[1]);
            *reinterpret_cast<uint32_t*>(Db(0) + (r + 8) * kSH + 2 * t) = pack_bf16(dy[2], dy[3]);
        }
        db0 = sum_over_rows(db0);
        db1 = sum_over_rows(db1);
        if (g == 0 && t < 2) {
            sbias[4 * kW + 2 * t] = db0;
            sbias[4 * kW + 2 * t + 1] = db1;
        }
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if (lane == 0) sloss[warp] = loss;
    }
    __syncthreads();

    float* pg = partial + (size_t)blockIdx.x * SKYR_MLP_PARAMS;
    // ---- backward ----
#pragma unroll 1
    for (int l = 4; l >= 0; --l) {
        const __nv_bfloat16* dz = Db(l & 1);
        const __nv_bfloat16* hin = l == 0 ? X0 : Hl(l - 1);
        const int hin_stride = l == 0 ? kXS : kSH;
        // (a) dW_l = dZ_l^T H_{l-1} over the block's 128 samples
        if (l == 4) {
            // rows = the 3 (of 8) outputs, warp w takes input columns 16w .. 16w + 15
            float acc[2][4] = {};
            const int n0 = warp * 16;
#pragma unroll 1
            for (int kt = 0; kt < 8; ++kt) {
                uint32_t a[4], b[4];
                ldsm_x4_t(a, smem_u32(dz + (kt * 16 + (lane & 7) + ((lane >> 4) << 3)) * kSH + ((lane >> 3) & 1) * 8));
                a[1] = 0u;
                a[3] = 0u;
                ldsm_x4_t(b, smem_u32(hin + (kt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8) * hin_stride + n0 +
                                      (lane >> 4) * 8));
                mma(acc[0], a, b[0], b[1]);
                mma(acc[1], a, b[2], b[3]);
            }
            if (g < kOut) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    int c = n0 + h * 8 + 2 * t;
                    pg[w_offset(4) + g * kW + c] = acc[h][0];
                    pg[w_offset(4) + g * kW + c + 1] = acc[h][1];
                }
            }
        } else {
            // rows n_out 16w .. 16w + 15, all input columns
            const int fi = fan_in(l), nps = l == 0 ? 3 : 4;
            float acc[8][4] = {};
#pragma unroll 1
            for (int kt = 0; kt < 8; ++kt) {
                uint32_t a[4];
                ldsm_x4_t(a, smem_u32(dz + (kt * 16 + (lane & 7) + ((lane >> 4) << 3)) * kSH + warp * 16 +
                                      ((lane >> 3) & 1) * 8));
#pragma unroll
                for (int np = 0; np < 4; ++np) {
                    if (np < nps) {
                        uint32_t b[4];
                        ldsm_x4_t(b, smem_u32(hin + (kt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8) * hin_stride +
                                              np * 16 + (lane >> 4) * 8));
                        mma(acc[2 * np], a, b[0], b[1]);
                        mma(acc[2 * np + 1], a, b[2], b[3]);
                    }
                }
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                int c = nt * 8 + 2 * t, r = warp * 16 + g;
                if (c < fi) {
                    pg[w_offset(l) + r * fi + c] = acc[nt][0];
                    pg[w_offset(l) + (r + 8) * fi + c] = acc[nt][2];
                }
                if (c + 1 < fi) {
                    pg[w_offset(l) + r * fi + c + 1] = acc[nt][1];
                    pg[w_offset(l) + (r + 8) * fi + c + 1] = acc[nt][3];
                }
            }
        }
        // (b) dZ_{l-1} = (dZ_l W_l) * (H_{l-1} > 0) for the warp's own rows
        if (l > 0) {
            const __nv_bfloat16* w = W(l);
            const int ws = packed_stride(l);
            __nv_bfloat16* dzo = Db((l - 1) & 1);
            const __nv_bfloat16* hp = Hl(l - 1);
            float db[8][2] = {};
#pragma unroll 1
            for (int mt = 0; mt < 2; ++mt) {
                const int r0 = row_w + mt * 16;
                float acc[8][4] = {};
                if (l == 4) {
                    uint32_t a[4];
                    load_a(a, dz, kSH, r0, 0);
                    a[2] = 0u;
                    a[3] = 0u;
#pragma unroll
                    for (int np = 0; np < 4; ++np) {
                        uint32_t b[4];
                        ldsm_x4_t(b, smem_u32(w + (lane & 7) * ws + np * 16 + (lane >> 4) * 8));
                        mma(acc[2 * np], a, b[0], 0u);
                        mma(acc[2 * np + 1], a, b[2], 0u);
                    }
                } else {
#pragma unroll 1
                    for (int kt = 0; kt < 4; ++kt) {
                        uint32_t a[4];
                        load_a(a, dz, kSH, r0, kt * 16);
#pragma unroll
                        for (int np = 0; np < 4; ++np) {
                            uint32_t b[4];
                            ldsm_x4_t(b, smem_u32(w + (kt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8) * ws +
                                                  np * 16 + (lane >> 4) * 8));
                            mma(acc[2 * np], a, b[0], b[1]);
                            mma(acc[2 * np + 1], a, b[2], b[3]);
                        }
                    }
                }
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) {
                    int c = nt * 8 + 2 * t;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        int r = r0 + g + h * 8;
                        __nv_bfloat162 hv = *reinterpret_cast<const __nv_bfloat162*>(hp + r * kSH + c);
                        float z0 = __low2float(hv) > 0.f ? acc[nt][2 * h] : 0.f;
                        float z1 = __high2float(hv) > 0.f ? acc[nt][2 * h + 1] : 0.f;
                        db[nt][0] += z0;
                        db[nt][1] += z1;
                        *reinterpret_cast<uint32_t*>(dzo + r * kSH + c) = pack_bf16(z0, z1);
                    }
                }
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float s0 = sum_over_rows(db[nt][0]), s1 = sum_over_rows(db[nt][1]);
                if (g == 0) {
                    sbias[(l - 1) * kW + nt * 8 + 2 * t] = s0;
                    sbias[(l - 1) * kW + nt * 8 + 2 * t + 1] = s1;
                }
            }
        }
        __syncthreads();
    }
    const float* sb = reinterpret_cast<const float*>(sm + kSmBias);
    for (int l = 0; l < kLayers; ++l)
        for (int j = threadIdx.x; j < fan_out(l); j += blockDim.x) {
            float v = 0.f;
            for (int w = 0; w < kWarps; ++w) v += sb[w * kBiasSlots + l * kW + j];
            pg[b_offset(l) + j] = v;
        }
    if (threadIdx.x == 0) loss_partial[blockIdx.x] = ((sloss[0] + sloss[1]) + sloss[2]) + sloss[3];
}

// grad[i] = sum over blocks of partial[b][i] (fixed order); optional Adam
// update of params / moments and re-pack; loss: sum of the loss partials.
__global__ void __launch_bounds__(256) mlp_reduce_kernel(const float* __restrict__ partial, int nblk,
                                                         const float* __restrict__ loss_partial,
                                                         float* __restrict__ grad_out, float* __restrict__ loss_out,
                                                         int loss_accumulate, float* __restrict__ params,
                                                         float* __restrict__ m, float* __restrict__ v, float lr,
                                                         float b1, float b2, float eps, float c1, float c2,
                                                         unsigned char* __restrict__ packed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && loss_out) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += loss_partial[b];
        *loss_out = loss_accumulate ? *loss_out + s : s;
    }
    if (i >= SKYR_MLP_PARAMS) return;
    float gsum = 0.f;
    for (int b = 0; b < nblk; ++b) gsum += partial[(size_t)b * SKYR_MLP_PARAMS + i];
    if (grad_out) grad_out[i] = gsum;
    if (params) {
        float mi = b1 * m[i] + (1.f - b1) * gsum;
        float vi = b2 * v[i] + (1.f - b2) * gsum * gsum;
        m[i] = mi;
        v[i] = vi;
        float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        params[i] = p;
        pack_one(packed, i, p);
    }
}

// The dynamic shared-memory opt-in of both kernels, once per device.
int ensure_grad_attr() {
    static bool done[64] = {};
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    if (dev >= 0 && dev < 64 && done[dev]) return SKYR_OK;
    if (int e = check_cuda(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmGrad),
                           "mlp gradient smem attribute"))
        return e;
    if (int e = check_cuda(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmInfer),
                           "mlp inference smem attribute"))
        return e;
    if (dev >= 0 && dev < 64) done[dev] = true;
    return SKYR_OK;
}

int validate_hparams(const skyr_mlp_hparams* h) {
    if (!h) return set_error(SKYR_EINVAL, "null hyper-parameters");
    if (!(h->learning_rate > 0.f) || !(h->beta1 >= 0.f && h->beta1 < 1.f) || !(h->beta2 >= 0.f && h->beta2 < 1.f) ||
        !(h->epsilon > 0.f) || !(h->label_scale > 0.f) || !(h->loss_epsilon > 0.f) ||
        !std::isfinite(h->learning_rate) || !std::isfinite(h->label_scale))
        return set_error(SKYR_EINVAL, "MLP hyper-parameters out of range");
    return SKYR_OK;
}

int launch_grad(skyr_ctx* ctx, const void* packed, const skyr_mlp_hparams* h, const uint16_t* x, const float* t,
                int n, float* partial, float* loss_partial) {
    if (int e = ensure_grad_attr()) return e;
    int nblk = (n + kTile - 1) / kTile;
    mlp_grad_kernel<<<nblk, kTile, kSmGrad, ctx->stream>>>(
        reinterpret_cast<const unsigned char*>(packed), reinterpret_cast<const uint4*>(x), t, n, 1.f / h->label_scale,
        h->loss_epsilon, 1.f / (3.f * (float)n), partial, loss_partial);
    return check_cuda(cudaGetLastError(), "mlp gradient kernel");
}

}  // namespace mlp
}  // namespace skyr

struct skyr_mlp_trainer {
    skyr_ctx* ctx = nullptr;
    skyr_mlp_hparams h{};
    float* params = nullptr;  // [P] FP32 master
    float* m = nullptr;
    float* v = nullptr;
    unsigned char* packed = nullptr;
    float* partial = nullptr;  // [kMaxBlocks][P]
    float* loss_partial = nullptr;
    int steps = 0;
};

using namespace skyr;

extern "C" {

int skyr_mlp_hparams_default(skyr_mlp_hparams* h) {
    if (!h) return set_error(SKYR_EINVAL, "null hyper-parameters");
    h->learning_rate = 1e-3f;
    h->beta1 = 0.9f;
    h->beta2 = 0.999f;
    h->epsilon = 1e-8f;
    h->label_scale = 1.f;
    h->loss_epsilon = 1e-2f;
    return SKYR_OK;
}

size_t skyr_mlp_param_count(void) { return SKYR_MLP_PARAMS; }
size_t skyr_mlp_packed_bytes(void) { return mlp::kPackedBytes; }

int skyr_mlp_init_params(uint64_t seed, float* params) {
    if (!params) return set_error(SKYR_EINVAL, "null parameters");
    // splitmix64 stream -> uniform [0, 1)
    uint64_t s = seed;
    auto next = [&]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < mlp::kLayers; ++l) {
        double a = std::sqrt(6.0 / mlp::fan_in(l));
        for (int i = 0; i < mlp::fan_in(l) * mlp::fan_out(l); ++i)
            params[mlp::w_offset(l) + i] = (float)((2.0 * next() - 1.0) * a);
        for (int i = 0; i < mlp::fan_out(l); ++i) params[mlp::b_offset(l) + i] = 0.f;
    }
    return SKYR_OK;
}

int skyr_mlp_pack(skyr_ctx* ctx, const float* params, float out_scale, void* packed) {
    if (!ctx || !params || !packed) return set_error(SKYR_EINVAL, "null argument");
    if (!(out_scale > 0.f) || !std::isfinite(out_scale)) return set_error(SKYR_EINVAL, "bad output scale");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = check_cuda(cudaMemsetAsync(packed, 0, mlp::kPackedBytes, ctx->stream), "clear packed network"))
        return e;
    mlp::mlp_pack_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        params, out_scale, reinterpret_cast<unsigned char*>(packed));
    return check_cuda(cudaGetLastError(), "mlp pack kernel");
}

int skyr_mlp_infer(skyr_ctx* ctx, const void* packed, const uint16_t* x, int n, float* y) {
    if (!ctx || !packed || (n > 0 && (!x || !y))) return set_error(SKYR_EINVAL, "null argument");
    if (n < 0) return set_error(SKYR_EINVAL, "negative sample count");
    if (n == 0) return SKYR_OK;
    if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(packed) & 15))
        return set_error(SKYR_EINVAL, "records and packed network must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = mlp::ensure_grad_attr()) return e;
    int sms = 0;
    if (int e = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device),
                           "multiprocessor count"))
        return e;
    int tiles = (n + 31) / 32;
    int blocks = std::min((tiles + mlp::kWarps - 1) / mlp::kWarps, sms * 8);
    mlp::mlp_infer_kernel<<<blocks, 32 * mlp::kWarps, mlp::kSmInfer, ctx->stream>>>(
        reinterpret_cast<const unsigned char*>(packed), reinterpret_cast<const uint4*>(x), n, y);
    return check_cuda(cudaGetLastError(), "mlp inference kernel");
}

int skyr_mlp_gradient(skyr_ctx* ctx, const void* packed, const skyr_mlp_hparams* h, const uint16_t* x,
                      const float* t, int n, float* grad, float* loss) {
    if (!ctx || !packed || !x || !t || !grad) return set_error(SKYR_EINVAL, "null argument");
    if (int e = mlp::validate_hparams(h)) return e;
    if (n < 1 || n > mlp::kMaxBatch) return set_error(SKYR_EINVAL, "batch size must be in [1, 65536]");
    if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(packed) & 15))
        return set_error(SKYR_EINVAL, "records and packed network must be 16-byte aligned");
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    int nblk = (n + mlp::kTile - 1) / mlp::kTile;
    size_t need = ((size_t)nblk * SKYR_MLP_PARAMS + nblk) * sizeof(float);
    if (int e = ensure_pt_scratch(ctx, need)) return e;  // shared per-context scratch
    float* partial = reinterpret_cast<float*>(ctx->pt_scratch);
    float* lp = partial + (size_t)nblk * SKYR_MLP_PARAMS;
    if (int e = mlp::launch_grad(ctx, packed, h, x, t, n, partial, lp)) return e;
    mlp::mlp_reduce_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        partial, nblk, lp, grad, loss, 0, nullptr, nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, nullptr);
    return check_cuda(cudaGetLastError(), "mlp reduce kernel");
}

int skyr_mlp_trainer_create(skyr_ctx* ctx, const float* host_params, const skyr_mlp_hparams* h,
                            skyr_mlp_trainer** out) {
    if (!ctx || !host_params || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = mlp::validate_hparams(h)) return e;
    *out = nullptr;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    auto* tr = new (std::nothrow) skyr_mlp_trainer;
    if (!tr) return set_error(SKYR_ENOMEM, "out of host memory");
    tr->ctx = ctx;
    tr->h = *h;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    int e = SKYR_OK;
    if (!e) e = check_cuda(cudaMalloc(&tr->params, pb), "cudaMalloc(mlp params)");
    if (!e) e = check_cuda(cudaMalloc(&tr->m, pb), "cudaMalloc(mlp m)");
    if (!e) e = check_cuda(cudaMalloc(&tr->v, pb), "cudaMalloc(mlp v)");
    if (!e) e = check_cuda(cudaMalloc(&tr->packed, mlp::kPackedBytes), "cudaMalloc(mlp packed)");
    if (!e) e = check_cuda(cudaMalloc(&tr->partial, (size_t)mlp::kMaxBlocks * pb), "cudaMalloc(mlp partials)");
    if (!e) e = check_cuda(cudaMalloc(&tr->loss_partial, mlp::kMaxBlocks * sizeof(float)), "cudaMalloc(mlp loss)");
    if (!e) e = check_cuda(cudaMemcpyAsync(tr->params, host_params, pb, cudaMemcpyHostToDevice, ctx->stream), "upload");
    if (!e) e = check_cuda(cudaMemsetAsync(tr->m, 0, pb, ctx->stream), "clear m");
    if (!e) e = check_cuda(cudaMemsetAsync(tr->v, 0, pb, ctx->stream), "clear v");
    if (!e) e = skyr_mlp_pack(ctx, tr->params, h->label_scale, tr->packed);
    if (!e) e = check_cuda(cudaStreamSynchronize(ctx->stream), "synchronize");  // host_params may go away
    if (e) {
        skyr_mlp_trainer_destroy(tr);
        return e;
    }
    *out = tr;
    return SKYR_OK;
}

int skyr_mlp_trainer_destroy(skyr_mlp_trainer* tr) {
    if (!tr) return SKYR_OK;
    if (tr->ctx) cudaSetDevice(tr->ctx->device);
    cudaFree(tr->params);
    cudaFree(tr->m);
    cudaFree(tr->v);
    cudaFree(tr->packed);
    cudaFree(tr->partial);
    cudaFree(tr->loss_partial);
    delete tr;
    return SKYR_OK;
}

int skyr_mlp_train_step(skyr_mlp_trainer* tr, const uint16_t* x, const float* t, int n, float* loss_accum) {
    if (!tr || !x || !t) return set_error(SKYR_EINVAL, "null argument");
    if (n < 1 || n > mlp::kMaxBatch) return set_error(SKYR_EINVAL, "batch size must be in [1, 65536]");
    if (reinterpret_cast<uintptr_t>(x) & 15) return set_error(SKYR_EINVAL, "records must be 16-byte aligned");
    skyr_ctx* ctx = tr->ctx;
    if (int e = check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice")) return e;
    if (int e = mlp::launch_grad(ctx, tr->packed, &tr->h, x, t, n, tr->partial, tr->loss_partial)) return e;
    int step = tr->steps + 1;
    double c1 = 1.0 - std::pow((double)tr->h.beta1, step), c2 = 1.0 - std::pow((double)tr->h.beta2, step);
    int nblk = (n + mlp::kTile - 1) / mlp::kTile;
    mlp::mlp_reduce_kernel<<<(SKYR_MLP_PARAMS + 255) / 256, 256, 0, ctx->stream>>>(
        tr->partial, nblk, tr->loss_partial, nullptr, loss_accum, 1, tr->params, tr->m, tr->v, tr->h.learning_rate,
        tr->h.beta1, tr->h.beta2, tr->h.epsilon, (float)c1, (float)c2, tr->packed);
    if (int e = check_cuda(cudaGetLastError(), "mlp adam kernel")) return e;
    tr->steps = step;
    return SKYR_OK;
}

const float* skyr_mlp_trainer_params(const skyr_mlp_trainer* tr) { return tr ? tr->params : nullptr; }
const void* skyr_mlp_trainer_packed(const skyr_mlp_trainer* tr) { return tr ? tr->packed : nullptr; }
int skyr_mlp_trainer_steps(const skyr_mlp_trainer* tr) { return tr ? tr->steps : -1; }

int skyr_mlp_trainer_set_learning_rate(skyr_mlp_trainer* tr, float learning_rate) {
    if (!tr) return set_error(SKYR_EINVAL, "null trainer");
    if (!(learning_rate > 0.f) || !std::isfinite(learning_rate)) return set_error(SKYR_EINVAL, "bad learning rate");
    tr->h.learning_rate = learning_rate;
    return SKYR_OK;
}

int skyr_mlp_trainer_copy_params(const skyr_mlp_trainer* tr, float* out) {
    if (!tr || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaMemcpyAsync(out, tr->params, SKYR_MLP_PARAMS * sizeof(float), cudaMemcpyDeviceToDevice,
                                      tr->ctx->stream),
                      "copy parameters");
}

int skyr_mlp_trainer_copy_packed(const skyr_mlp_trainer* tr, void* out) {
    if (!tr || !out) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    return check_cuda(cudaMemcpyAsync(out, tr->packed, mlp::kPackedBytes, cudaMemcpyDeviceToDevice, tr->ctx->stream),
                      "copy packed network");
}

int skyr_mlp_trainer_save_state(const skyr_mlp_trainer* tr, float* params, float* m, float* v, int* steps) {
    if (!tr || !params || !m || !v || !steps) return set_error(SKYR_EINVAL, "null argument");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    cudaStream_t st = tr->ctx->stream;
    if (int e = check_cuda(cudaMemcpyAsync(params, tr->params, pb, cudaMemcpyDeviceToDevice, st), "save parameters"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(m, tr->m, pb, cudaMemcpyDeviceToDevice, st), "save first moments"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(v, tr->v, pb, cudaMemcpyDeviceToDevice, st), "save second moments"))
        return e;
    *steps = tr->steps;
    return SKYR_OK;
}

int skyr_mlp_trainer_load_state(skyr_mlp_trainer* tr, const float* params, const float* m, const float* v,
                                int steps) {
    if (!tr || !params || !m || !v) return set_error(SKYR_EINVAL, "null argument");
    if (steps < 0) return set_error(SKYR_EINVAL, "negative step count");
    if (int e = check_cuda(cudaSetDevice(tr->ctx->device), "cudaSetDevice")) return e;
    const size_t pb = SKYR_MLP_PARAMS * sizeof(float);
    cudaStream_t st = tr->ctx->stream;
    if (int e = check_cuda(cudaMemcpyAsync(tr->params, params, pb, cudaMemcpyDeviceToDevice, st), "load parameters"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(tr->m, m, pb, cudaMemcpyDeviceToDevice, st), "load first moments"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync(tr->v, v, pb, cudaMemcpyDeviceToDevice, st), "load second moments"))
        return e;
    if (int e = skyr_mlp_pack(tr->ctx, tr->params, tr->h.label_scale, tr->packed)) return e;
    tr->steps = steps;
    return SKYR_OK;
}

}  // extern "C"
