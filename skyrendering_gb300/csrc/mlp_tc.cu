// mlp_tc.cu — batched inference of the surrogate network on tcgen05
// (skyr_mlp_infer).  A persistent grid of 4-warp CTAs walks 128-sample tiles;
// see mlp_tc.cuh for the tile scheme.
#include <algorithm>

#include "mlp_tc.cuh"
#include "skyr_ctx.cuh"

namespace skyr {
namespace mlp {

// Waits of this kernel that ran out set bit 2 of the status word.
constexpr int kTcStatusBit = 4;

__global__ void __launch_bounds__(128) mlp_infer_tc_kernel(const unsigned char* __restrict__ packed,
                                                           const uint4* __restrict__ x, int n,
                                                           float* __restrict__ y, int* __restrict__ status,
                                                           long long wait_cycles) {
    extern __shared__ unsigned char sm_raw[];
    unsigned char* s = tc_base(sm_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t bar = tc05::smem_addr(s + kTcBar);
    tc_load_network(s, packed);
    if (tid == 0) tc05::mbar_init(bar, 1);
    if (warp == 0) tc05::alloc(tc05::smem_addr(s + kTcHold), kTcCols);
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(s + kTcHold);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
    const float* bias = reinterpret_cast<const float*>(s + kTcBias);
    const float scale = bias[4 * kW + 8];
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + 127) / 128;
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int smp = tile * 128 + tid;
        // the record of sample tid: kRec bf16 = kRec / 8 chunks of the A row
#pragma unroll
        for (int q = 0; q < kRec / 8; ++q) {
            uint4 v = smp < n ? __ldg(x + (size_t)smp * (kRec / 8) + q) : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(s + kTcA + tc05::sw128_offset(tid, q * 8, 128)) = v;
        }
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            tc05::fence_smem_to_async();
            tc05::fence_before_sync();
            __syncthreads();
            tc05::fence_after_sync();
            if (tid == 0) tc_layer_mma(s, l, tmem, bar);
            ok = __syncthreads_and(tc05::mbar_wait(bar, phase, wait_cycles));
            if (!ok) break;
            phase ^= 1;
            tc05::fence_after_sync();
            if (l < kLayers - 1) {
                tc_hidden_epilogue(s, bias + l * kW, lane_addr, tid, kTcA);
            } else {
                float v[16];
                tc05::ld16(lane_addr, v);
                if (smp < n) {
#pragma unroll
                    for (int c = 0; c < kOut; ++c) y[(size_t)smp * 3 + c] = (v[c] + bias[4 * kW + c]) * scale;
                }
            }
        }
    }
    if (!ok) {
        // a wait ran out: report, let the MMAs in flight land (bounded), then free the tensor memory
        if (tid == 0 && status) atomicOr(status, kTcStatusBit);
        tc05::mbar_wait(bar, phase, kBulkWaitCycles);
    }
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    if (warp == 0) tc05::dealloc(tmem, kTcCols);
}

// ---------------------------------------------------------------------------
// The training gradient of one 128-sample tile per CTA
// ---------------------------------------------------------------------------
// Shared memory (offsets from a 1024-byte aligned base): the network image of
// mlp_tc.cuh, the transposed weights W2^T..W5^T (B operands of dZ W), the input
// X0, the hidden activations H1..H4 (A operands forward, ReLU masks and dW
// operands backward), two dZ tiles used in turn, biases and reduction slots.
constexpr int kGWT = kTcNet;                      // W2^T, W3^T, W4^T, W5^T: [64 in][64 out] each
constexpr int kGX = kGWT + 4 * kTcWTile;          // X0 [128][128] (two tiles, kRec columns used)
constexpr int kGH = kGX + 2 * kTcABlock;          // H1..H4 [128][64]
constexpr int kGD = kGH + 4 * 128 * 128;          // D0, D1 [128][64]
constexpr int kGBias = kGD + 2 * 128 * 128;       // b1..b5 f32, then the output scale
constexpr int kGSlot = kGBias + 1088;             // [4 warps][64] f32 column sums
constexpr int kGLoss = kGSlot + 4 * 64 * 4;       // [4 warps] loss, [4 warps][4] output-bias sums
constexpr int kGBar = kGLoss + 16 + 64;
constexpr int kGHold = kGBar + 8;
constexpr int kGSmem = kGHold + 8 + 1024;
static_assert(kGX % 1024 == 0 && kGH % 1024 == 0 && kGD % 1024 == 0 && kGWT % 1024 == 0, "tile alignment");
static_assert(kGSmem <= 232448, "shared memory of one CTA");

__device__ __forceinline__ uint32_t gh(int l) { return l == 0 ? (uint32_t)kGX : (uint32_t)(kGH + (l - 1) * 128 * 128); }
__device__ __forceinline__ uint32_t gd(int b) { return (uint32_t)(kGD + b * 128 * 128); }

// Sum of v[0..63] over the 32 lanes of the warp by a halving butterfly: lane L
// ends with the sums of columns 2L and 2L + 1 in v[0], v[1] (fixed order).
__device__ __forceinline__ void butterfly_column_sums(float (&v)[64]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int st = 16, w = 32; st >= 1; st >>= 1, w >>= 1) {
        const bool upper = (lane & st) != 0;
#pragma unroll
        for (int j = 0; j < w; ++j) {
            float send = upper ? v[j] : v[j + w];
            float keep = upper ? v[j + w] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, st);
        }
    }
}

// Sample i of the batch is record idx[i] of x / tgt (i itself without idx);
// an index outside [0, n_all) counts as an empty sample.
__global__ void __launch_bounds__(128, 1) mlp_grad_tc_kernel(const unsigned char* __restrict__ packed,
                                                             const uint4* __restrict__ x,
                                                             const float* __restrict__ tgt,
                                                             const int* __restrict__ idx, int n_all, int n,
                                                             float inv_scale,
                                                             float loss_eps, float inv_count,
                                                             float* __restrict__ partial,
                                                             float* __restrict__ loss_partial,
                                                             int* __restrict__ status, long long wait_cycles) {
    extern __shared__ unsigned char sm_raw[];
    unsigned char* s = tc_base(sm_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    int smp = blockIdx.x * 128 + tid;
    if (smp < n) {
        smp = idx ? __ldg(idx + smp) : smp;
        if ((unsigned)smp >= (unsigned)n_all) smp = -1;
    } else {
        smp = -1;
    }
    const uint32_t bar = tc05::smem_addr(s + kGBar);
    // network image, biases (+ scale) and this tile's records
    tc_load_network(s, packed);
    {
        const float* pb = reinterpret_cast<const float*>(packed + kOffB);
        float* sb = reinterpret_cast<float*>(s + kGBias);
        for (int i = tid; i < 4 * kW + 8 + 1; i += blockDim.x) sb[i] = __ldg(pb + i);
    }
#pragma unroll
    for (int q = 0; q < kRec / 8; ++q) {
        uint4 v = smp >= 0 ? __ldg(x + (size_t)smp * (kRec / 8) + q) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4*>(s + kGX + tc05::sw128_offset(tid, q * 8, 128)) = v;
    }
    if (tid == 0) tc05::mbar_init(bar, 1);
    if (warp == 0) tc05::alloc(tc05::smem_addr(s + kGHold), kTcCols);
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    // transposed weights from the image: W^T[l][i][o] = W[l][o][i] (W5^T: 3 outputs, zero beyond)
    for (int k = tid; k < 4 * 64 * 8; k += blockDim.x) {
        const int l = 1 + k / 512, i = (k >> 3) & 63, c = k & 7;
        const int rows = l < 4 ? 64 : 16;
        uint32_t p[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int o0 = c * 8 + 2 * e, o1 = o0 + 1;
            uint16_t lo = 0, hi = 0;
            if (l < 4 || o0 < kOut)
                lo = *reinterpret_cast<const uint16_t*>(s + tc_weight_tile(l) + tc05::sw128_offset(o0, i, rows));
            if (l < 4 || o1 < kOut)
                hi = *reinterpret_cast<const uint16_t*>(s + tc_weight_tile(l) + tc05::sw128_offset(o1, i, rows));
            p[e] = (uint32_t)lo | ((uint32_t)hi << 16);
        }
        *reinterpret_cast<uint4*>(s + kGWT + (l - 1) * kTcWTile + tc05::sw128_offset(i, c * 8, 64)) =
            make_uint4(p[0], p[1], p[2], p[3]);
    }
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(s + kGHold);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    const float* bias = reinterpret_cast<const float*>(s + kGBias);
    float* slot = reinterpret_cast<float*>(s + kGSlot);
    float* sloss = reinterpret_cast<float*>(s + kGLoss);
    float* sdb5 = sloss + 4;
    float* pg = partial + (size_t)blockIdx.x * SKYR_MLP_PARAMS;
    uint32_t phase = 0;
    bool ok = true;
    auto sync_for_mma = [&]() {
        tc05::fence_smem_to_async();
        tc05::fence_before_sync();
        __syncthreads();
        tc05::fence_after_sync();
    };
    auto wait_mma = [&]() {
        ok = __syncthreads_and(tc05::mbar_wait(bar, phase, wait_cycles));
        if (ok) {
            phase ^= 1;
            tc05::fence_after_sync();
        }
        return ok;
    };
    // ---- forward: H[l + 1] = relu(H[l] W[l]^T + b[l]), H[0] = X0 ----
#pragma unroll 1
    for (int l = 0; l < 4 && ok; ++l) {
        sync_for_mma();
        if (tid == 0) tc_layer_mma(s, l, gh(l), tmem, bar);
        if (!wait_mma()) break;
        tc_hidden_epilogue(s, bias + l * kW, lane_addr, tid, gh(l + 1));
    }
    // ---- output layer, loss and dY (into D0, 16 columns, 3 used) ----
    if (ok) {
        sync_for_mma();
        if (tid == 0) tc_layer_mma(s, 4, gh(4), tmem, bar);
        if (wait_mma()) {
            float v[16];
            tc05::ld16(lane_addr, v);
            float dy[4] = {0.f, 0.f, 0.f, 0.f}, loss = 0.f;
#pragma unroll
            for (int c = 0; c < kOut; ++c) {
                if (smp >= 0) {
                    float o = v[c] + bias[4 * kW + c];
                    float d = o - __ldg(tgt + (size_t)smp * 3 + c) * inv_scale;
                    float w = 1.f / (o * o + loss_eps);
                    loss += d * d * w * inv_count;
                    dy[c] = 2.f * d * w * inv_count;
                }
            }
            *reinterpret_cast<uint4*>(s + gd(0) + tc05::sw128_offset(tid, 0, 128)) =
                make_uint4(pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], 0.f), 0u, 0u);
            *reinterpret_cast<uint4*>(s + gd(0) + tc05::sw128_offset(tid, 8, 128)) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                loss += __shfl_xor_sync(0xffffffffu, loss, o);
#pragma unroll
                for (int c = 0; c < kOut; ++c) dy[c] += __shfl_xor_sync(0xffffffffu, dy[c], o);
            }
            if (lane == 0) {
                sloss[warp] = loss;
                for (int c = 0; c < kOut; ++c) sdb5[warp * 4 + c] = dy[c];
            }
        }
    }
    // ---- backward: dW[l] = dZ[l]^T H[l]; dZ[l - 1] = (dZ[l] W[l]) * (H[l] > 0) ----
#pragma unroll 1
    for (int l = 4; l >= 0 && ok; --l) {
        sync_for_mma();
        const uint32_t dz = gd(l & 1), hin = gh(l);
        if (l > 0 && tid == 0)
            tc_mma(tc05::smem_addr(s + dz), 0, tc05::smem_addr(s + kGWT + (l - 1) * kTcWTile), 0, l == 4 ? 1 : 4, 64,
                   tmem, bar);
        // dW[l] on the warp-level tensor path while the tcgen05 product runs
        if (l == 4) {
            float acc[2][4] = {};
            const int n0 = warp * 16;
#pragma unroll 1
            for (int kt = 0; kt < 8; ++kt) {
                uint32_t a[4], b[4];
                ldsm_x4_t(a, tc05::smem_addr(s + dz + tc05::sw128_offset(kt * 16 + (lane & 7) + ((lane >> 4) << 3),
                                                                         ((lane >> 3) & 1) * 8, 128)));
                a[1] = 0u;
                a[3] = 0u;
                ldsm_x4_t(b, tc05::smem_addr(s + hin + tc05::sw128_offset(kt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8,
                                                                          n0 + (lane >> 4) * 8, 128)));
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
            const int fi = fan_in(l), nps = l == 0 ? kKT : 4;  // 16-column pairs of dW's columns
            float acc[2 * kKT > 8 ? 2 * kKT : 8][4] = {};
#pragma unroll 1
            for (int kt = 0; kt < 8; ++kt) {
                uint32_t a[4];
                ldsm_x4_t(a, tc05::smem_addr(s + dz + tc05::sw128_offset(kt * 16 + (lane & 7) + ((lane >> 4) << 3),
                                                                         warp * 16 + ((lane >> 3) & 1) * 8, 128)));
#pragma unroll
                for (int np = 0; np < (kKT > 4 ? kKT : 4); ++np) {
                    if (np < nps) {
                        uint32_t b[4];
                        ldsm_x4_t(b, tc05::smem_addr(
                                         s + hin + tc05::sw128_offset(kt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8,
                                                                      np * 16 + (lane >> 4) * 8, 128)));
                        mma(acc[2 * np], a, b[0], b[1]);
                        mma(acc[2 * np + 1], a, b[2], b[3]);
                    }
                }
            }
#pragma unroll
            for (int nt = 0; nt < 2 * (kKT > 4 ? kKT : 4); ++nt) {
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
        if (l == 0) break;
        // dZ[l - 1] for this thread's row, the ReLU mask from H[l], and its column sums (bias gradient)
        if (!wait_mma()) break;
        float z[64];
#pragma unroll
        for (int cb = 0; cb < 4; ++cb) {
            float v[16];
            tc05::ld16(lane_addr + cb * 16, v);
            uint4 h0 = *reinterpret_cast<const uint4*>(s + hin + tc05::sw128_offset(tid, cb * 16, 128));
            uint4 h1 = *reinterpret_cast<const uint4*>(s + hin + tc05::sw128_offset(tid, cb * 16 + 8, 128));
            uint32_t hw[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
            uint32_t p[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                __nv_bfloat162 hv = *reinterpret_cast<__nv_bfloat162*>(&hw[j]);
                float z0 = __low2float(hv) > 0.f ? v[2 * j] : 0.f;
                float z1 = __high2float(hv) > 0.f ? v[2 * j + 1] : 0.f;
                z[cb * 16 + 2 * j] = z0;
                z[cb * 16 + 2 * j + 1] = z1;
                p[j] = pack_bf16(z0, z1);
            }
            const uint32_t dst = gd((l - 1) & 1);
            *reinterpret_cast<uint4*>(s + dst + tc05::sw128_offset(tid, cb * 16, 128)) =
                make_uint4(p[0], p[1], p[2], p[3]);
            *reinterpret_cast<uint4*>(s + dst + tc05::sw128_offset(tid, cb * 16 + 8, 128)) =
                make_uint4(p[4], p[5], p[6], p[7]);
        }
        butterfly_column_sums(z);
        slot[warp * 64 + 2 * lane] = z[0];
        slot[warp * 64 + 2 * lane + 1] = z[1];
        __syncthreads();
        if (tid < 64) pg[b_offset(l - 1) + tid] = ((slot[tid] + slot[64 + tid]) + slot[128 + tid]) + slot[192 + tid];
    }
    if (ok) {
        __syncthreads();
        if (tid < kOut) pg[b_offset(4) + tid] = ((sdb5[tid] + sdb5[4 + tid]) + sdb5[8 + tid]) + sdb5[12 + tid];
        if (tid == 0) loss_partial[blockIdx.x] = ((sloss[0] + sloss[1]) + sloss[2]) + sloss[3];
    } else {
        if (tid == 0 && status) atomicOr(status, kTcStatusBit);
        tc05::mbar_wait(bar, phase, kBulkWaitCycles);
    }
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    if (warp == 0) tc05::dealloc(tmem, kTcCols);
}

int launch_grad_tc(skyr_ctx* ctx, const void* packed, const uint16_t* x, const float* t, const int* idx, int n_all,
                   int n, float inv_scale, float loss_eps, float* partial, float* loss_partial) {
    static bool attr_done[64] = {};
    int dev = ctx->device;
    if (dev < 0 || dev >= 64) return set_error(SKYR_ENOTSUP, "device index %d beyond 64", dev);
    if (!attr_done[dev]) {
        if (int e = check_cuda(cudaFuncSetAttribute(mlp_grad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    kGSmem),
                               "mlp tensor-core gradient smem attribute"))
            return e;
        attr_done[dev] = true;
    }
    if (int e = ensure_status(ctx)) return e;
    int nblk = (n + 127) / 128;
    mlp_grad_tc_kernel<<<nblk, 128, kGSmem, ctx->stream>>>(
        reinterpret_cast<const unsigned char*>(packed), reinterpret_cast<const uint4*>(x), t, idx, n_all, n,
        inv_scale, loss_eps,
        1.f / (3.f * (float)n), partial, loss_partial, ctx->d_status, ctx->limits.copy_wait_cycles);
    return check_cuda(cudaGetLastError(), "mlp tensor-core gradient kernel");
}

int launch_infer_tc(skyr_ctx* ctx, const void* packed, const uint16_t* x, int n, float* y) {
    static bool attr_done[64] = {};
    int dev = ctx->device;
    if (dev < 0 || dev >= 64) return set_error(SKYR_ENOTSUP, "device index %d beyond 64", dev);
    if (!attr_done[dev]) {
        if (int e = check_cuda(cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    kTcSmem),
                               "mlp tensor-core inference smem attribute"))
            return e;
        attr_done[dev] = true;
    }
    if (int e = ensure_status(ctx)) return e;
    int sms = 0, per_sm = 0;
    if (int e = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count")) return e;
    if (int e = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_infer_tc_kernel, 128, kTcSmem),
                           "occupancy"))
        return e;
    // tensor memory: per_sm CTAs x kTcCols columns stay within the SM's 512
    per_sm = std::min(std::max(per_sm, 1), (int)(512 / kTcCols));
    int tiles = (n + 127) / 128;
    int blocks = std::min(tiles, sms * per_sm);
    mlp_infer_tc_kernel<<<blocks, 128, kTcSmem, ctx->stream>>>(reinterpret_cast<const unsigned char*>(packed),
                                                               reinterpret_cast<const uint4*>(x), n, y, ctx->d_status,
                                                               ctx->limits.copy_wait_cycles);
    return check_cuda(cudaGetLastError(), "mlp tensor-core inference kernel");
}

}  // namespace mlp
}  // namespace skyr
