// mlp_tc.cuh — the surrogate network on the 5th-generation tensor cores
// (tcgen05): the shared-memory image of the packed network in the tensor
// core's operand layout, and the forward pass of a 128-sample tile with the
// accumulator in tensor memory.  Used by batched inference (mlp_tc.cu) and by
// the forward half of the training step.
//
// A CTA of 4 warps owns one 128-sample tile at a time: thread t holds sample
// t (tensor-memory lane t), so a layer's epilogue (bias, ReLU, BF16) runs on
// the thread's own accumulator row and writes the next layer's A operand row.
// One elected thread issues each layer's MMAs (M = 128, N = 64, K = the record
// width (112) or 64) and commits them to an mbarrier the CTA waits on (bounded).
#pragma once

#include <cuda_bf16.h>

#include "mlp_device.cuh"
#include "tc05.cuh"

namespace skyr {
namespace mlp {

// Shared-memory image (offsets from a 1024-byte aligned base).  The first
// layer's K (the record, kRec <= 128 columns) spans two 64-column tiles.
constexpr int kTcWTile = 64 * 128;                  // one 64 x 64 K-major SWIZZLE_128B weight tile (8 KB)
constexpr int kTcW2 = 2 * kTcWTile;                 // W2..W4 (W1, 64 rows x 128 columns with kIn used, at 0)
constexpr int kTcW5 = kTcW2 + 3 * kTcWTile;         // W5: 16 rows (3 used) x 64
constexpr int kTcA = kTcW5 + 16 * 128;              // activations: 128 rows x 128 columns (two tiles)
constexpr int kTcNet = kTcA;                        // bytes of the weight image
constexpr int kTcABlock = 128 * 128;                // bytes of one 64-column tile of 128 rows
constexpr int kTcBias = kTcA + 2 * kTcABlock;       // b1..b4 [4][64], b5 [8], output scale (f32)
constexpr int kTcBar = kTcBias + (4 * kW + 8 + 4) * 4;
constexpr int kTcHold = kTcBar + 8;
constexpr int kTcSmem = kTcHold + 8 + 1024;         // + the alignment slack of the dynamic base
constexpr uint32_t kTcCols = 64;                    // tensor-memory columns of the accumulator

static_assert(kTcA % 1024 == 0 && kTcW5 % 1024 == 0, "swizzled tiles start on 1024-byte boundaries");

__device__ __forceinline__ unsigned char* tc_base(unsigned char* raw) {
    uint32_t a = tc05::smem_addr(raw);
    return raw + ((1024u - (a & 1023u)) & 1023u);
}

__device__ __forceinline__ uint32_t tc_weight_tile(int l) {
    return l == 0 ? 0u : l < 4 ? (uint32_t)(kTcW2 + (l - 1) * kTcWTile) : (uint32_t)kTcW5;
}

// The packed network (global, skyr_mlp_packed_bytes layout) into the tensor
// core's operand image; every thread of the block takes part, caller syncs.
__device__ __forceinline__ void tc_load_network(unsigned char* s, const unsigned char* packed) {
    constexpr int kW1Chunks = 64 * 16, kHChunks = 64 * 8;  // 16-byte chunks of W1 (128 columns), of W2..W4
    for (int i = threadIdx.x; i < kW1Chunks + 3 * kHChunks + 16 * 8; i += blockDim.x) {
        int l, j;
        if (i < kW1Chunks) {
            l = 0, j = i;
        } else if (i < kW1Chunks + 3 * kHChunks) {
            l = 1 + (i - kW1Chunks) / kHChunks, j = (i - kW1Chunks) % kHChunks;
        } else {
            l = 4, j = i - kW1Chunks - 3 * kHChunks;
        }
        const int cpr = l == 0 ? 16 : 8;  // chunks per row
        int r = j / cpr, c = j % cpr, rows = l < 4 ? 64 : 16;
        // packed rows: W1 kS1 bf16 (kIn used), W2..W4 72 (64 used), W5 8 rows (3 used) of 72
        bool valid = (l == 0 && c * 8 < kS1) || (l > 0 && l < 4) || (l == 4 && r < 8);
        uint4 v = make_uint4(0, 0, 0, 0);
        if (valid)
            v = __ldg(reinterpret_cast<const uint4*>(packed + packed_w_offset(l) + r * packed_stride(l) * 2 + c * 16));
        *reinterpret_cast<uint4*>(s + tc_weight_tile(l) + tc05::sw128_offset(r, c * 8, rows)) = v;
    }
    const float* pb = reinterpret_cast<const float*>(packed + kOffB);
    float* sb = reinterpret_cast<float*>(s + kTcBias);
    for (int i = threadIdx.x; i < 4 * kW + 8 + 1; i += blockDim.x) sb[i] = __ldg(pb + i);  // biases, then the scale
}

// D[tmem] = A[128 x 16 ksteps] * B[n x 16 ksteps]^T from K-major SWIZZLE_128B
// operands whose 64-column tiles lie a_block / b_block bytes apart (elected
// thread), committed to `bar`.
__device__ __forceinline__ void tc_mma(uint32_t a, uint32_t a_block, uint32_t b, uint32_t b_block, int ksteps, int n,
                                       uint32_t tmem, uint32_t bar) {
    const uint32_t idesc = tc05::idesc_bf16(128, n);
#pragma unroll 1
    for (int kk = 0; kk < ksteps; ++kk)
        tc05::mma_bf16(tmem, tc05::sw128_desc(a + (kk >> 2) * a_block + (kk & 3) * 32),
                       tc05::sw128_desc(b + (kk >> 2) * b_block + (kk & 3) * 32), idesc, kk > 0);
    tc05::commit(bar);
}

// One forward layer's MMAs: D[tmem] = A[128 x K] * W_l^T (K = kRec for layer 0,
// its A a 128-row, two-tile operand at a_off).
__device__ __forceinline__ void tc_layer_mma(const unsigned char* s, int l, uint32_t a_off, uint32_t tmem,
                                             uint32_t bar) {
    tc_mma(tc05::smem_addr(s + a_off), kTcABlock, tc05::smem_addr(s + tc_weight_tile(l)), kTcWTile,
           l == 0 ? kKT : 4, l == 4 ? 16 : 64, tmem, bar);
}
__device__ __forceinline__ void tc_layer_mma(const unsigned char* s, int l, uint32_t tmem, uint32_t bar) {
    tc_layer_mma(s, l, kTcA, tmem, bar);
}

// Epilogue of a hidden layer on this thread's row: bias (64 f32), ReLU, BF16,
// written as row `row` of the 128-row operand tile at s + dst (64 columns).
__device__ __forceinline__ void tc_hidden_epilogue(unsigned char* s, const float* bias, uint32_t lane_addr, int row,
                                                   uint32_t dst) {
#pragma unroll
    for (int cb = 0; cb < 4; ++cb) {
        float v[16];
        tc05::ld16(lane_addr + cb * 16, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            p[j] = pack_bf16(fmaxf(v[2 * j] + bias[cb * 16 + 2 * j], 0.f),
                             fmaxf(v[2 * j + 1] + bias[cb * 16 + 2 * j + 1], 0.f));
        *reinterpret_cast<uint4*>(s + dst + tc05::sw128_offset(row, cb * 16, 128)) = make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(s + dst + tc05::sw128_offset(row, cb * 16 + 8, 128)) =
            make_uint4(p[4], p[5], p[6], p[7]);
    }
}

}  // namespace mlp
}  // namespace skyr
