// Warp-level tensor-core building blocks of the fused kernels.
//
// Precision: every operand x is split into bf16 hi = rn(x) and lo = rn(x -
// hi); a product is accumulated as hi*hi + lo*hi + hi*lo in fp32 ("bf16x3"),
// which carries ~16 mantissa bits per operand.  A single bf16 pass would add
// ~2^-9 relative noise to every activation; the finite-difference stencil of
// the SDF divides differences of such values by eps = 1/2048, so the noise
// would dominate the gradient.
//
// Fragment layouts (m16n8k16, row.col), r = lane/4, c = 2*(lane%4):
//   A (16x16): a0 = (r, c..c+1), a1 = (r+8, c..), a2 = (r, c+8..), a3 = (r+8, c+8..)
//   B (16x8) : b0 = (k = c..c+1, n = r), b1 = (k = c+8.., n = r)
//   C (16x8) : c0,c1 = (r, c), (r, c+1); c2,c3 = (r+8, c), (r+8, c+1)
// Two C tiles (n-tiles 2j, 2j+1) of a layer output are exactly the A
// fragment of k-tile j of the next layer.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace angelo {

struct Split {
    uint32_t hi, lo;
};

// (x0 at the lower column, x1 at the upper) -> packed bf16x2 hi and lo parts
__device__ __forceinline__ Split split2(float x0, float x1) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    Split s;
    s.hi = *reinterpret_cast<const uint32_t *>(&h);
    s.lo = *reinterpret_cast<const uint32_t *>(&l);
    return s;
}

// the same split into fp16 hi and lo parts (11 significant bits each: the
// operand format of the fp16 precision form)
__device__ __forceinline__ Split split2h(float x0, float x1) {
    const __half2 h = __floats2half2_rn(x0, x1);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
    Split s;
    s.hi = *reinterpret_cast<const uint32_t *>(&h);
    s.lo = *reinterpret_cast<const uint32_t *>(&l);
    return s;
}

// packed fp16x2 or bf16x2 of (x0, x1) alone (a single-pass operand)
template <bool FP16>
__device__ __forceinline__ uint32_t pack2(float x0, float x1) {
    if (FP16) {
        const __half2 h = __floats2half2_rn(x0, x1);
        return *reinterpret_cast<const uint32_t *>(&h);
    }
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// d += A * B with both operands split (three passes, small terms first)
__device__ __forceinline__ void mma_x3(float (&d)[4], const uint32_t (&ah)[4],
                                       const uint32_t (&al)[4], uint2 bh, uint2 bl) {
    mma_bf16(d, al, bh.x, bh.y);
    mma_bf16(d, ah, bl.x, bl.y);
    mma_bf16(d, ah, bh.x, bh.y);
}

// Transpose of an 8x8 b16 matrix held one bf16x2 per lane (row lane/4,
// columns 2*(lane%4)..+1) into the same layout of the transposed matrix.
__device__ __forceinline__ uint32_t movmatrix_t(uint32_t x) {
    uint32_t y;
    asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;\n" : "=r"(y) : "r"(x));
    return y;
}

__device__ __forceinline__ float softplus100(float z) {
    // torch.nn.Softplus(beta=100, threshold=20): z when 100 z > 20, else
    // log(1 + e^(100 z)) / 100.  For 100 z < -15 the result is e^(100 z)/100
    // to fp32 precision; otherwise lg2/ex2 (MUFU) are accurate to a few ulp
    // on 1 + e^x in [1, e^20].
    const float x = 100.0f * z;
    if (x > 20.0f) return z;
    const float e = __expf(x);
    return (x < -15.0f ? e : __logf(1.0f + e)) * 0.01f;
}

__device__ __forceinline__ float softplus100_grad(float z) {
    const float x = 100.0f * z;
    return x > 20.0f ? 1.0f : __fdividef(1.0f, 1.0f + __expf(-x));
}

// softplus100(z) and its derivative from one exponential: the derivative as
// e / (1 + e), e = e^(100 z), the form of torch's softplus backward.
__device__ __forceinline__ void softplus100_both(float z, float *sp, float *grad) {
    const float x = 100.0f * z;
    const float e = __expf(fminf(x, 20.0f));
    const float q = 1.0f + e;
    *sp = x > 20.0f ? z : (x < -15.0f ? e : __logf(q)) * 0.01f;
    *grad = x > 20.0f ? 1.0f : __fdividef(e, q);
}

}  // namespace angelo
