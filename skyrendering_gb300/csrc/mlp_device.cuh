// mlp_device.cuh — device side of the surrogate network (include/skyr_mlp.h):
// the packed layout, BF16 tensor-core fragments (mma.sync m16n8k16, FP32
// accumulation, ldmatrix) and the warp-level forward pass that the inference
// kernel and the surrogate raymarch share.
//
// A warp evaluates 32 samples as two 16-row tiles.  The activations never leave
// registers between layers: the FP32 accumulator fragment of two adjacent
// 8-column tiles of layer l is, after bias, ReLU and BF16 packing, exactly the
// A-operand fragment of one 16-column k-tile of layer l + 1.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "../../include/skyr_mlp.h"

namespace skyr {
namespace mlp {

constexpr int kIn = SKYR_MLP_INPUTS;    // 103
constexpr int kRec = SKYR_MLP_RECORD;   // 112
constexpr int kKT = kRec / 16;          // k-tiles of the first layer (7)
constexpr int kW = SKYR_MLP_WIDTH;      // 64
constexpr int kOut = SKYR_MLP_OUTPUTS;  // 3
constexpr int kLayers = 5;
static_assert(kRec % 16 == 0 && kIn < kRec && kRec <= 128, "record: whole k-tiles, at most two 64-column tiles");

// Row strides (bf16) of the packed weight matrices: rows of an odd number of
// 16-byte units (240 B, 144 B) put the 8 rows an ldmatrix phase reads in 8
// different 16-byte bank groups.
constexpr int kS1 = kRec + 8;  // W1 [64][kS1], columns kIn.. zero
constexpr int kSH = 72;        // W2..W4 [64][kSH], W5 [8][kSH] (rows 3..7 zero)
// Byte offsets in the packed network
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kW * kS1 * 2;
constexpr int kOffW3 = kOffW2 + kW * kSH * 2;
constexpr int kOffW4 = kOffW3 + kW * kSH * 2;
constexpr int kOffW5 = kOffW4 + kW * kSH * 2;
constexpr int kOffB = kOffW5 + 8 * kSH * 2;          // b1..b4 [4][64] f32, b5 [8] f32
constexpr int kOffScale = kOffB + (4 * kW + 8) * 4;
constexpr int kPackedBytes = kOffScale + 16;

// Row stride (bf16) of a feature-record tile in shared memory (240 B rows)
constexpr int kXS = kRec + 8;

__host__ __device__ constexpr int fan_in(int l) { return l == 0 ? kIn : kW; }
__host__ __device__ constexpr int fan_out(int l) { return l == kLayers - 1 ? kOut : kW; }
__host__ __device__ constexpr int w_offset(int l) {  // in the FP32 parameter vector
    return l == 0 ? 0 : (kIn * kW + kW) + (l - 1) * (kW * kW + kW);
}
__host__ __device__ constexpr int b_offset(int l) { return w_offset(l) + fan_in(l) * fan_out(l); }
static_assert(b_offset(kLayers - 1) + kOut == SKYR_MLP_PARAMS, "parameter count");

__host__ __device__ constexpr int packed_w_offset(int l) {
    return l == 0 ? kOffW1 : l == 1 ? kOffW2 : l == 2 ? kOffW3 : l == 3 ? kOffW4 : kOffW5;
}
__host__ __device__ constexpr int packed_stride(int l) { return l == 0 ? kS1 : kSH; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Copy the packed network (global) into shared memory; all threads of the
// block take part, caller synchronises.
// The packed network into shared memory `s` by one bulk copy on the TMA
// engine (cp.async.bulk, completion counted in bytes on the mbarrier `bar`),
// for every thread of the block.  `g` and `s` are 16-byte aligned and
// kPackedBytes is a multiple of 16.  The wait is bounded by `budget` SM cycles
// (skyr_device_limits::copy_wait_cycles, default 2^31, about a second; 0 never waits); if any
// thread's wait expires, the status word gets bit 1, the block waits once more
// for its copy in flight, bounded by kBulkWaitCycles whatever `budget` is (the
// copy must land before the block's shared memory is released), and every
// thread gets false: the caller leaves without touching the shared copy.
constexpr long long kBulkWaitCycles = 1ll << 31;

// Waits for phase 0 of the mbarrier at most `budget` SM cycles (the clock is
// read before every try, so a budget of 0 never waits); true if it completed.
__device__ __forceinline__ bool bulk_wait(uint32_t bar, long long budget) {
    const long long t0 = clock64();
    uint32_t done = 0;
    while (!done && clock64() - t0 < budget) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar)
            : "memory");
    }
    return done != 0;
}

__device__ __forceinline__ bool load_packed_bulk(unsigned char* s, const unsigned char* g, unsigned long long* bar,
                                                 int* status, long long budget = kBulkWaitCycles) {
    static_assert(kPackedBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
    const uint32_t b = smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"((uint32_t)kPackedBytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(s)),
                     "l"(g), "r"((uint32_t)kPackedBytes), "r"(b)
                     : "memory");
    }
    // one decision for the whole block: a thread that gave up makes every thread leave
    if (__syncthreads_and(bulk_wait(b, budget))) return true;
    if (status && threadIdx.x == 0) atomicOr(status, 2);
    bulk_wait(b, kBulkWaitCycles);
    return false;
}

__device__ __forceinline__ void load_packed(unsigned char* s, const unsigned char* g) {
    const uint4* src = reinterpret_cast<const uint4*>(g);
    uint4* dst = reinterpret_cast<uint4*>(s);
    for (int i = threadIdx.x; i < kPackedBytes / 16; i += blockDim.x) dst[i] = __ldg(src + i);
}

// A fragment (16 rows x 16 columns) of a row-major bf16 tile in shared memory
// (rows `row0`.., columns `col0`.., row stride `stride` bf16).
__device__ __forceinline__ void load_a(uint32_t (&a)[4], const __nv_bfloat16* base, int stride, int row0, int col0) {
    int lane = threadIdx.x & 31;
    ldsm_x4(a, smem_u32(base + (row0 + (lane & 15)) * stride + col0 + (lane >> 4) * 8));
}

// B fragments of two adjacent 8-column tiles (n0, n0 + 8) for k-tile k0 of a
// weight matrix stored [out][in] (Y = X W^T): b[0], b[1] for n0; b[2], b[3] for n0 + 8.
__device__ __forceinline__ void load_b_pair(uint32_t (&b)[4], const __nv_bfloat16* w, int stride, int n0, int k0) {
    int lane = threadIdx.x & 31;
    ldsm_x4(b, smem_u32(w + (n0 + (lane >> 4) * 8 + (lane & 7)) * stride + k0 + ((lane >> 3) & 1) * 8));
}

// Output tile of one 16-row slab: the C fragment holds rows g / g + 8 and
// columns 2t, 2t + 1 (g = lane / 4, t = lane % 4).
struct OutTile {
    float c[4];
};

// Forward of one 16-row slab: rows row0.. of the record tile x (stride kXS),
// its kKT k-tiles loaded one at a time.  Returns the FP32 output fragment of
// the final layer (columns 0..2 valid, before the output scale).
__device__ __forceinline__ OutTile forward_slab(const unsigned char* sw, const __nv_bfloat16* x, int row0) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    const float* bias = reinterpret_cast<const float*>(sw + kOffB);
    uint32_t a[4][4];
    float acc[8][4];
    // layer 1: K = kRec
    {
        const __nv_bfloat16* w = reinterpret_cast<const __nv_bfloat16*>(sw + kOffW1);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float b0 = bias[nt * 8 + 2 * t], b1 = bias[nt * 8 + 2 * t + 1];
            acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        }
#pragma unroll
        for (int kt = 0; kt < kKT; ++kt) {
            uint32_t xa[4];
            load_a(xa, x, kXS, row0, kt * 16);
#pragma unroll
            for (int np = 0; np < 4; ++np) {
                uint32_t b[4];
                load_b_pair(b, w, kS1, np * 16, kt * 16);
                mma(acc[2 * np], xa, b[0], b[1]);
                mma(acc[2 * np + 1], xa, b[2], b[3]);
            }
        }
    }
    // layers 2..4: K = 64, A from the previous accumulators
#pragma unroll 1
    for (int l = 1; l < 4; ++l) {
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            a[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0], 0.f), fmaxf(acc[2 * kt][1], 0.f));
            a[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2], 0.f), fmaxf(acc[2 * kt][3], 0.f));
            a[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0], 0.f), fmaxf(acc[2 * kt + 1][1], 0.f));
            a[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2], 0.f), fmaxf(acc[2 * kt + 1][3], 0.f));
        }
        const __nv_bfloat16* w = reinterpret_cast<const __nv_bfloat16*>(sw + packed_w_offset(l));
        const float* bl = bias + l * kW;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float b0 = bl[nt * 8 + 2 * t], b1 = bl[nt * 8 + 2 * t + 1];
            acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        }
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int np = 0; np < 4; ++np) {
                uint32_t b[4];
                load_b_pair(b, w, kSH, np * 16, kt * 16);
                mma(acc[2 * np], a[kt], b[0], b[1]);
                mma(acc[2 * np + 1], a[kt], b[2], b[3]);
            }
    }
    // layer 5: N = 8 (3 valid)
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0], 0.f), fmaxf(acc[2 * kt][1], 0.f));
        a[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2], 0.f), fmaxf(acc[2 * kt][3], 0.f));
        a[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0], 0.f), fmaxf(acc[2 * kt + 1][1], 0.f));
        a[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2], 0.f), fmaxf(acc[2 * kt + 1][3], 0.f));
    }
    const __nv_bfloat16* w5 = reinterpret_cast<const __nv_bfloat16*>(sw + kOffW5);
    const float* b5 = bias + 4 * kW;
    OutTile o;
    o.c[0] = b5[2 * t]; o.c[1] = b5[2 * t + 1]; o.c[2] = o.c[0]; o.c[3] = o.c[1];
#pragma unroll
    for (int kp = 0; kp < 2; ++kp) {
        // two k-tiles of the 8-row W5 at once: b[0], b[1] for k-tile 2kp, b[2], b[3] for 2kp + 1
        uint32_t b[4];
        ldsm_x4(b, smem_u32(w5 + (lane & 7) * kSH + kp * 32 + (lane >> 3) * 8));
        mma(o.c, a[2 * kp], b[0], b[1]);
        mma(o.c, a[2 * kp + 1], b[2], b[3]);
    }
    return o;
}

// Forward of the warp's 32 samples whose records sit in shared memory rows
// [0, 32) of `x` (stride kXS); the three outputs of sample r are written to
// y[r * 4 + c] (shared memory, c < 3) scaled by the packed output scale.  All
// 32 lanes must take part; the caller syncs the warp before reading y.
__device__ __forceinline__ void forward_warp(const unsigned char* sw, const __nv_bfloat16* x, float* y) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const float scale = *reinterpret_cast<const float*>(sw + kOffScale);
#pragma unroll 1
    for (int mt = 0; mt < 2; ++mt) {
        OutTile o = forward_slab(sw, x, mt * 16);
        if (t < 2) {
            int r = mt * 16 + g;
            int c = 2 * t;
            y[r * 4 + c] = o.c[0] * scale;
            if (c + 1 < 4) y[r * 4 + c + 1] = o.c[1] * scale;
            y[(r + 8) * 4 + c] = o.c[2] * scale;
            y[(r + 8) * 4 + c + 1] = o.c[3] * scale;
        }
    }
}

}  // namespace mlp
}  // namespace skyr
