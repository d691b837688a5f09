// Fifth-generation tensor core (tcgen05) building blocks for sm_103a, as
// inline PTX: tensor-memory allocation, shared-memory matrix descriptors,
// the kind::f16 MMA (BF16 x BF16 -> FP32 accumulators in tensor memory),
// commit to an mbarrier, bounded mbarrier waits and tensor-memory loads.
//
// Operand layout used throughout (no swizzle, "interleaved" core matrices):
// a tile of R rows x K bf16 values is stored as K/8 column chunks, each chunk
// holding the R rows' 8 values (16 bytes) back to back:
//     byte(r, k) = (k / 8) * (R * 16) + r * 16 + (k % 8) * 2
// so the 8x8 core matrix of rows 8g..8g+7 and chunk c is 128 contiguous
// bytes at c * R * 16 + g * 128.  For a K-major operand the descriptor's
// leading-dimension byte offset is then the chunk stride (R * 16) and its
// stride-dimension byte offset the 8-row stride (128).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in the layout above.
__host__ __device__ __forceinline__ uint32_t tile_offset(uint32_t rows, uint32_t r, uint32_t k) {
    return (k >> 3) * (rows * 16u) + r * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor (64 bits): start address, leading and
// stride byte offsets (all >> 4), descriptor version 1 at bits 46-47,
// base offset 0, swizzle mode 0 (none) at bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both
// operands K-major unless a_mn / b_mn select MN-major; M and N as given.
__host__ __device__ __forceinline__ uint32_t idesc_bf16(uint32_t m, uint32_t n, bool a_mn = false,
                                                        bool b_mn = false) {
    uint32_t d = 0;
    d |= 1u << 4;                 // D format: F32
    d |= 1u << 7;                 // A format: BF16
    d |= 1u << 10;                // B format: BF16
    d |= (a_mn ? 1u : 0u) << 15;  // A major
    d |= (b_mn ? 1u : 0u) << 16;  // B major
    d |= (n >> 3) << 17;          // N / 8
    d |= (m >> 4) << 24;          // M / 16
    return d;
}

// ---- tensor memory ------------------------------------------------------------
// Allocation by one whole warp; the TMEM address is written to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes generic-proxy writes to shared memory visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T for one K=16 step.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
        "}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}

// Arrives once on the mbarrier when all previously issued MMAs of this
// thread have completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(mbar))
                 : "memory");
}

// ---- mbarrier ------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t"
        "}\n"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for the phase with the given parity to complete, giving up after
// `limit` polls (each poll itself returns after a bounded time).
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}

// ---- tensor memory -> registers ---------------------------------------------------
// 32 lanes x 32 columns of 32-bit values: thread t of the warp receives lane
// (warp's lane base + t), columns col .. col+31.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// TMEM address of (lane, column).
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, uint32_t lane, uint32_t col) {
    return base + (lane << 16) + col;
}

}  // namespace tc
