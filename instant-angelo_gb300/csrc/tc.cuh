// Blackwell 5th-generation tensor-core helpers (tcgen05, inline PTX, sm_100a+
// family): tensor-memory allocation, shared-memory matrix descriptors for the
// no-swizzle K-major layout, the bf16 MMA with fp32 accumulation in tensor
// memory, completion through an mbarrier with a bounded wait, and loads of
// the accumulator back to registers.
//
// Shared-memory operand layout (no swizzle): the operand is a grid of "core
// matrices" of 128 contiguous bytes.  K-major: 8 rows x 16 bytes (8 bf16
// along K); core matrices adjacent along K are LBO bytes apart, groups of 8
// rows SBO bytes apart:
//   byte(r, k) = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2,
// here with LBO = 128 and SBO = 16 * K; one MMA consumes K = 16 (two chunks)
// and the next K step starts 256 bytes further.  MN-major: 8 K-rows x 16
// bytes (8 bf16 along M); LBO is again the stride along K (between groups of
// 8 K-rows) and SBO the stride along M (between 8-element chunks).
//
// Accumulator (M = 128, cta_group::1): row i of D is tensor-memory lane i,
// column j is the allocation's column base + j (fp32).  M = 64: row i is lane
// 32 (i / 16) + i % 16 (lanes 16 .. 31 of each quarter are not written).
// Warp w may read only lanes 32 (w % 4) .. 32 (w % 4) + 31.
#pragma once

#include <stdint.h>

namespace angelo {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) of a bf16 K-major operand with K columns
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (16 * K) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Core-matrix strides of an operand with `rows` M (or N) rows and K columns,
// staged K-major (kmajor_offset(r, k, K)) or MN-major (kmajor_offset(k, r,
// rows): the same 128-byte core matrices with M contiguous).  The descriptor
// takes the stride along K in LBO and the stride along M/N in SBO for both.
__host__ __device__ __forceinline__ uint32_t k_stride(int mn_major, int rows, int K) {
    return mn_major ? (uint32_t)(16 * rows) : 128u;
}
__host__ __device__ __forceinline__ uint32_t mn_stride(int mn_major, int rows, int K) {
    return mn_major ? 128u : (uint32_t)(16 * K);
}

// 64-bit shared-memory matrix descriptor: start address, LBO, SBO (all >> 4),
// descriptor version 1 (bits 46-48 = 0b001), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D fp32, A and B bf16,
// dense, M x N; a_mn / b_mn select the MN-major operand layout (0: K-major).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N, int a_mn = 0, int b_mn = 0) {
    return (1u << 4)                       // D format: f32
           | (1u << 7)                     // A format: bf16
           | (1u << 10)                    // B format: bf16
           | ((uint32_t)(a_mn & 1) << 15)  // A major
           | ((uint32_t)(b_mn & 1) << 16)  // B major
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// The same for A and B in fp16 (format field 0).  A and B always share one
// type in a kind::f16 product.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N, int a_mn = 0, int b_mn = 0) {
    return (1u << 4)                       // D format: f32
           | ((uint32_t)(a_mn & 1) << 15)  // A major
           | ((uint32_t)(b_mn & 1) << 16)  // B major
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}
__host__ __device__ constexpr uint32_t idesc_f32(int M, int N, bool fp16) {
    return fp16 ? idesc_f16_f32(M, N) : idesc_bf16_f32(M, N);
}

// ---- tensor memory allocation (one full warp)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 ::"r"(smem_addr(slot_smem)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// ---- ordering
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// ---- MMA (single thread): D[tmem] (+)= A[smem] x B[smem]^T
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on the mbarrier once every MMA this thread issued so far completed
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_addr(mbar))
                 : "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred P1;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
        "selp.b32 %0, 1, 0, P1;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false when the phase did not complete within max_iters polls
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t max_iters) {
    for (uint32_t i = 0; i < max_iters; ++i)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}

// ---- accumulator loads: this thread's lane, 16 consecutive fp32 columns.
// The load and tcgen05.wait::ld are one asm statement: the destination
// registers are undefined until the wait, and the compiler must not move
// their uses above it.
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// this thread's lane, 8 (or 4) consecutive fp32 columns
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld4(uint32_t taddr, float (&v)[4]) {
    uint32_t r[4];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ldn(uint32_t taddr, float (&v)[8]) { ld8(taddr, v); }
__device__ __forceinline__ void ldn(uint32_t taddr, float (&v)[4]) { ld4(taddr, v); }

// ---- accumulator stores: zeros into this thread's lane, 16 consecutive
// columns (completed by tcgen05.wait::st in the same statement)
__device__ __forceinline__ void st16_zero(uint32_t taddr) {
    const uint32_t z = 0u;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};\n"
        "tcgen05.wait::st.sync.aligned;\n" ::"r"(taddr),
        "r"(z)
        : "memory");
}

}  // namespace tc
}  // namespace angelo
