// tc05.cuh — inline-PTX helpers for the 5th-generation tensor cores of sm_103a
// (tcgen05): tensor-memory allocation, shared-memory matrix descriptors in the
// 128-byte-swizzled K-major layout, the BF16 MMA with an FP32 accumulator in
// tensor memory, its commit to an mbarrier, and the accumulator loads.
//
// Operand layout (K-major, SWIZZLE_128B): a tile of R rows x 64 bf16 columns is
// R rows of 128 bytes; the 16-byte chunk c of row r sits at chunk position
// c ^ (r % 8), and the tile starts on a 1024-byte boundary (8-row atoms of
// 1024 bytes).  Wider K is a sequence of such 64-column tiles.  One MMA takes
// K = 16 columns (32 bytes of every row): its descriptor starts 32 bytes into
// the row for each further step, and the tensor core applies the swizzle to
// the addresses it forms.
#pragma once

#include <cstdint>

namespace skyr {
namespace tc05 {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row r, column k) in a K-major SWIZZLE_128B tile of
// `rows` rows (bf16 elements; columns beyond 63 go to the following 64-column tiles).
__host__ __device__ __forceinline__ uint32_t sw128_offset(int r, int k, int rows) {
    return (uint32_t)((k >> 6) * rows * 128 + r * 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row atoms 1024 bytes
// apart (stride byte offset), start address `addr` (shared window).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);       // bits 0-13: start address >> 4
    d |= (uint64_t)1 << 16;                         // bits 16-29: leading byte offset (unused when swizzled)
    d |= (uint64_t)(1024u >> 4) << 32;              // bits 32-45: stride byte offset >> 4
    d |= (uint64_t)1 << 46;                         // bits 46-48: fixed 0b001
    d |= (uint64_t)2 << 61;                         // bits 61-63: 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 D,
// an M x N tile.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4)                      // D format: F32
           | (1u << 7)                    // A format: BF16
           | (1u << 10)                   // B format: BF16
           | ((uint32_t)(n >> 3) << 17)   // N >> 3
           | ((uint32_t)(m >> 4) << 24);  // M >> 4
}

// Tensor-memory allocation of `cols` columns (a power of two >= 32) by one
// whole warp; the base address is written to shared memory at `holder`.
__device__ __forceinline__ void alloc(uint32_t holder, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(holder), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes made visible to the tensor core's reads.
__device__ __forceinline__ void fence_smem_to_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// The MMAs issued so far by this thread arrive on the mbarrier when complete.
__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for the phase with parity `parity` of the mbarrier, at most `budget`
// SM cycles; true if it completed.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long budget) {
    const long long t0 = clock64();
    uint32_t done = 0;
    while (!done && clock64() - t0 < budget) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    }
    return done != 0;
}

// 16 consecutive FP32 accumulator columns of this thread's tensor-memory lane
// (a warp reads its own 32 lanes: lane base 32 x (warp % 4) in taddr bits 16-31).
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc05
}  // namespace skyr
