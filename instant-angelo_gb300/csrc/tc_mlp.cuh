// Building blocks of the tcgen05 MLP kernels (fused VolumeSDF and fused
// radiance): a CTA of kTcThreads threads owns 128 rows; one thread issues the
// tensor-core products of a round and commits them to an mbarrier; every
// thread waits (bounded), reads a 16-column slice of its row back from tensor
// memory and stages the next operand in shared memory as bf16 hi/lo.
//
// Operands are staged as bf16 [rows][C] in the no-swizzle core-matrix layout
// (tc::kmajor_offset(r, c, C)), the hi half and the lo half `half` bytes
// apart.  The same bytes are read K-major (K = C, M or N = rows: a layer's
// input) or, transposed, MN-major (M or N = C, K = rows: the operand of a
// weight-gradient product whose reduction runs over the rows).
#pragma once

#include <stdint.h>

#include "mma.cuh"
#include "tc.cuh"

namespace angelo {

constexpr uint32_t kTcWaitPolls = 1u << 24;   // bounded mbarrier waits
constexpr int kTcThreads = 512;

// Every thread waits for the mbarrier phase; false (the same in every thread)
// when some thread gave up.
__device__ __forceinline__ bool tc_wait_all(uint64_t *bar, uint32_t phase) {
    const bool ok = tc::mbar_wait(bar, phase, kTcWaitPolls);
    const int failed = __syncthreads_or(!ok);
    tc::fence_after_sync();
    return failed == 0;
}

// Operand writes of every thread visible to the tensor cores, then thread 0
// may issue (after this, all threads have also finished their tensor-memory
// reads of the previous phase).
__device__ __forceinline__ void tc_publish() {
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// 16 consecutive columns c0 .. c0 + 15 (c0 % 16 == 0) of row r of an operand
// staged with K columns, split into bf16 hi and lo
__device__ __forceinline__ void stage16(char *hi, char *lo, int r, int c0, int K, const float (&v)[16]) {
    uint32_t h[8], l[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const Split sp = split2(v[2 * i], v[2 * i + 1]);
        h[i] = sp.hi;
        l[i] = sp.lo;
    }
    const uint32_t o0 = tc::kmajor_offset(r, c0, K), o1 = tc::kmajor_offset(r, c0 + 8, K);
    *reinterpret_cast<uint4 *>(hi + o0) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(hi + o1) = make_uint4(h[4], h[5], h[6], h[7]);
    *reinterpret_cast<uint4 *>(lo + o0) = make_uint4(l[0], l[1], l[2], l[3]);
    *reinterpret_cast<uint4 *>(lo + o1) = make_uint4(l[4], l[5], l[6], l[7]);
}

// stage16 in the operand format of the forward kernels: bf16 or fp16, with
// the lo part (three products) or the hi part alone (one pass: the lo half
// is not written and not read)
template <bool FP16>
__device__ __forceinline__ void stage16f(char *hi, char *lo, int r, int c0, int K, const float (&v)[16],
                                         bool with_lo) {
    const uint32_t o0 = tc::kmajor_offset(r, c0, K), o1 = tc::kmajor_offset(r, c0 + 8, K);
    if (!with_lo) {
        uint32_t h[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) h[i] = pack2<FP16>(v[2 * i], v[2 * i + 1]);
        *reinterpret_cast<uint4 *>(hi + o0) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(hi + o1) = make_uint4(h[4], h[5], h[6], h[7]);
        return;
    }
    if (!FP16) {
        stage16(hi, lo, r, c0, K, v);
        return;
    }
    uint32_t h[8], l[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const Split sp = split2h(v[2 * i], v[2 * i + 1]);
        h[i] = sp.hi;
        l[i] = sp.lo;
    }
    *reinterpret_cast<uint4 *>(hi + o0) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(hi + o1) = make_uint4(h[4], h[5], h[6], h[7]);
    *reinterpret_cast<uint4 *>(lo + o0) = make_uint4(l[0], l[1], l[2], l[3]);
    *reinterpret_cast<uint4 *>(lo + o1) = make_uint4(l[4], l[5], l[6], l[7]);
}

// descriptor fields of one staged operand for one K step of 16
struct TcOp {
    uint32_t hi, lo, lbo, sbo, step;
};
// read K-major: K = C, M (or N) = rows
__device__ __forceinline__ TcOp op_k(uint32_t hi, uint32_t half, int C) {
    return TcOp{hi, hi + half, 128u, 16u * (uint32_t)C, 256u};
}
// read as the transposed operand (MN-major): M (or N) = C, K = rows
__device__ __forceinline__ TcOp op_t(uint32_t hi, uint32_t half, int C) {
    return TcOp{hi, hi + half, 16u * (uint32_t)C, 128u, 32u * (uint32_t)C};
}

// hi and lo side by side in one [rows][C] staging: the hi part in columns
// [0, w), the lo part in [w, 2 w) (a weight-gradient product then reads both
// as one operand of 2 w rows: op_t(base, 0, C) with M or N = 2 w)
__device__ __forceinline__ TcOp op_k2(uint32_t base, int w, int C) {
    return TcOp{base, base + (uint32_t)(w / 8) * 128u, 128u, 16u * (uint32_t)C, 256u};
}
__device__ __forceinline__ TcOp op_t2(uint32_t base, int w, int C) {
    return TcOp{base, base + (uint32_t)(w / 8) * 128u, 16u * (uint32_t)C, 128u, 32u * (uint32_t)C};
}

// 16 columns c0 .. c0 + 15 of row r, hi part at column c0 and lo part at
// column w + c0 of a staging with C columns
__device__ __forceinline__ void stage16_2(char *base, int r, int c0, int w, int C, const float (&v)[16]) {
    uint32_t h[8], l[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const Split sp = split2(v[2 * i], v[2 * i + 1]);
        h[i] = sp.hi;
        l[i] = sp.lo;
    }
    *reinterpret_cast<uint4 *>(base + tc::kmajor_offset(r, c0, C)) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(base + tc::kmajor_offset(r, c0 + 8, C)) = make_uint4(h[4], h[5], h[6], h[7]);
    *reinterpret_cast<uint4 *>(base + tc::kmajor_offset(r, w + c0, C)) = make_uint4(l[0], l[1], l[2], l[3]);
    *reinterpret_cast<uint4 *>(base + tc::kmajor_offset(r, w + c0 + 8, C)) = make_uint4(l[4], l[5], l[6], l[7]);
}

// D (+)= A B^T over KSTEPS steps of 16, one product per step (operands
// whose rows already stack the hi and lo parts).  One thread.
template <int KSTEPS>
__device__ __forceinline__ void tc_mma1(uint32_t d, const TcOp &a, const TcOp &b, uint32_t idesc, bool acc) {
#pragma unroll
    for (int ks = 0; ks < KSTEPS; ++ks)
        tc::mma_bf16(d, tc::smem_desc(a.hi + ks * a.step, a.lbo, a.sbo),
                     tc::smem_desc(b.hi + ks * b.step, b.lbo, b.sbo), idesc, (acc || ks > 0) ? 1u : 0u);
}

// D (+)= A B^T over KSTEPS steps of 16 in bf16x3 (lo*hi + hi*lo + hi*hi); with
// b_exact, B is exact in bf16 and its lo product is left out.  One thread.
template <int KSTEPS>
__device__ __forceinline__ void tc_mma(uint32_t d, const TcOp &a, const TcOp &b, uint32_t idesc, bool acc,
                                       bool b_exact = false) {
#pragma unroll
    for (int ks = 0; ks < KSTEPS; ++ks) {
        const uint64_t ah = tc::smem_desc(a.hi + ks * a.step, a.lbo, a.sbo);
        const uint64_t al = tc::smem_desc(a.lo + ks * a.step, a.lbo, a.sbo);
        const uint64_t bh = tc::smem_desc(b.hi + ks * b.step, b.lbo, b.sbo);
        tc::mma_bf16(d, al, bh, idesc, (acc || ks > 0) ? 1u : 0u);
        if (!b_exact) tc::mma_bf16(d, ah, tc::smem_desc(b.lo + ks * b.step, b.lbo, b.sbo), idesc, 1u);
        tc::mma_bf16(d, ah, bh, idesc, 1u);
    }
}

// D (+)= A B^T with `passes` products per K step: 3 = bf16x3 (tc_mma), 1 =
// the hi parts alone (a single bf16 pass).  One thread.
template <int KSTEPS>
__device__ __forceinline__ void tc_mma_p(uint32_t d, const TcOp &a, const TcOp &b, uint32_t idesc, bool acc,
                                         int passes) {
    if (passes == 1) tc_mma1<KSTEPS>(d, a, b, idesc, acc);
    else tc_mma<KSTEPS>(d, a, b, idesc, acc);
}

// The constant operand [rows = 128][16] with column 0 = 1 (bf16, hi only):
// dZ^T times it is the column sum of dZ (a bias gradient) in column 0.
__device__ __forceinline__ void fill_ones_operand(uint16_t *ones, int tid, int nthreads) {
    for (int i = tid; i < 128 * 16; i += nthreads)
        ones[tc::kmajor_offset(i >> 4, i & 15, 16) >> 1] = (i & 15) == 0 ? (uint16_t)0x3F80u : (uint16_t)0u;
}

// Zero 16-column blocks [c0, c1) of this warp's tensor-memory lanes; the
// four warps of a lane quarter (slice 0..3) share the blocks.
__device__ __forceinline__ void tmem_zero(uint32_t tmem_lane, uint32_t c0, uint32_t c1, int slice) {
    for (uint32_t c = c0 + 16u * (uint32_t)slice; c < c1; c += 64u) tc::st16_zero(tmem_lane + c);
}

// Column sums over the warp's 32 lanes of v[0..15] (lane = row): afterwards
// lanes 2c and 2c + 1 hold the sum of column col(2c), 16 shuffles.
__device__ __forceinline__ float warp_colsum16(const float (&v)[16], int lane, int *col) {
    float a[8], b[4], c[2];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const bool up = lane & 16;
        const float keep = up ? v[j + 8] : v[j], send = up ? v[j] : v[j + 8];
        a[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const bool up = lane & 8;
        const float keep = up ? a[j + 4] : a[j], send = up ? a[j] : a[j + 4];
        b[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const bool up = lane & 4;
        const float keep = up ? b[j + 2] : b[j], send = up ? b[j] : b[j + 2];
        c[j] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    const bool up = lane & 2;
    float r = (up ? c[1] : c[0]) + __shfl_xor_sync(0xffffffffu, up ? c[0] : c[1], 2);
    r += __shfl_xor_sync(0xffffffffu, r, 1);
    *col = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    return r;
}

}  // namespace angelo
