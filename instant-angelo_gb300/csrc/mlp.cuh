// Warp-level MLP layers on mma.sync (bf16x3, fp32 accumulation) shared by the
// fused kernels: forward layers chained in registers, activations, the
// backward products dX = dZ W and dW += dZ^T X (operands transposed 8x8
// blockwise with movmatrix, reduced into shared memory).
#pragma once

#include "mma.cuh"

namespace angelo {

__host__ __device__ inline int64_t frag_count(int kt, int nt) { return (int64_t)kt * nt * 32; }

template <int KT>
__device__ __forceinline__ void hidden_layer(const uint32_t (&ah)[KT][4], const uint32_t (&al)[KT][4],
                                             const uint2 *wf, const float *bias, int lane,
                                             float (&D)[8][4]) {
    const int c = (lane & 3) * 2;
    const int64_t n_frag = frag_count(KT, 8);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = bias[nt * 8 + c], b1 = bias[nt * 8 + c + 1];
        D[nt][0] = 0.f;
        D[nt][1] = 0.f;
        D[nt][2] = 0.f;
        D[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            const int64_t i = (int64_t)(kt * 8 + nt) * 32 + lane;
            mma_x3(D[nt], ah[kt], al[kt], wf[i], wf[n_frag + i]);
        }
        D[nt][0] += b0;
        D[nt][1] += b1;
        D[nt][2] += b0;
        D[nt][3] += b1;
    }
}

__device__ __forceinline__ void activate(const float (&Z)[8][4], uint32_t (&hh)[4][4],
                                         uint32_t (&hl)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const float(&z)[4] = Z[2 * kt + half];
            const Split s0 = split2(softplus100(z[0]), softplus100(z[1]));
            const Split s1 = split2(softplus100(z[2]), softplus100(z[3]));
            hh[kt][2 * half] = s0.hi;
            hl[kt][2 * half] = s0.lo;
            hh[kt][2 * half + 1] = s1.hi;
            hl[kt][2 * half + 1] = s1.lo;
        }
    }
}

__device__ __forceinline__ void red_add(float *p, float v) {
    asm volatile("red.shared.add.f32 [%0], %1;\n" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v)
                 : "memory");
}

__device__ __forceinline__ void c_to_a(const float (&C)[8][4], uint32_t (&h)[4][4], uint32_t (&l)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const float(&z)[4] = C[2 * kt + half];
            const Split s0 = split2(z[0], z[1]), s1 = split2(z[2], z[3]);
            h[kt][2 * half] = s0.hi;
            l[kt][2 * half] = s0.lo;
            h[kt][2 * half + 1] = s1.hi;
            l[kt][2 * half + 1] = s1.lo;
        }
}

template <int KTN, int KTK>
__device__ __forceinline__ void accumulate_dw(const uint32_t (&zh)[KTN][4], const uint32_t (&zl)[KTN][4],
                                              const uint32_t (&xh)[KTK][4], const uint32_t (&xl)[KTK][4],
                                              float *dW, int ld, int lane) {
    const int r = lane >> 2, c = (lane & 3) * 2;
#pragma unroll
    for (int mt = 0; mt < KTN; ++mt) {
        uint32_t ah[4], al[4];
        ah[0] = movmatrix_t(zh[mt][0]);
        ah[1] = movmatrix_t(zh[mt][2]);
        ah[2] = movmatrix_t(zh[mt][1]);
        ah[3] = movmatrix_t(zh[mt][3]);
        al[0] = movmatrix_t(zl[mt][0]);
        al[1] = movmatrix_t(zl[mt][2]);
        al[2] = movmatrix_t(zl[mt][1]);
        al[3] = movmatrix_t(zl[mt][3]);
#pragma unroll
        for (int ntp = 0; ntp < 2 * KTK; ++ntp) {
            const int kt = ntp >> 1, hf = (ntp & 1) * 2;
            const uint2 bh = make_uint2(movmatrix_t(xh[kt][hf]), movmatrix_t(xh[kt][hf + 1]));
            const uint2 bl = make_uint2(movmatrix_t(xl[kt][hf]), movmatrix_t(xl[kt][hf + 1]));
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma_x3(d, ah, al, bh, bl);
            float *row0 = dW + (mt * 16 + r) * ld + ntp * 8 + c;
            float *row1 = row0 + 8 * ld;
            red_add(row0, d[0]);
            red_add(row0 + 1, d[1]);
            red_add(row1, d[2]);
            red_add(row1 + 1, d[3]);
        }
    }
}

template <int NT>
__device__ __forceinline__ void accumulate_db(const float (&C)[NT][4], float *db, int lane) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        float a = C[nt][0] + C[nt][2], b = C[nt][1] + C[nt][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane < 4) {
            red_add(db + nt * 8 + lane * 2, a);
            red_add(db + nt * 8 + lane * 2 + 1, b);
        }
    }
}

template <int KT, int NTO>
__device__ __forceinline__ void mm_nobias(const uint32_t (&ah)[KT][4], const uint32_t (&al)[KT][4],
                                          const uint2 *wf, int NT, int lane, float (&D)[NTO][4]) {
    const int64_t n_frag = frag_count(KT, NT);
#pragma unroll
    for (int nt = 0; nt < NTO; ++nt) {
        D[nt][0] = D[nt][1] = D[nt][2] = D[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            const int64_t i = (int64_t)(kt * NT + nt) * 32 + lane;
            mma_x3(D[nt], ah[kt], al[kt], wf[i], wf[n_frag + i]);
        }
    }
}

__device__ __forceinline__ void normalize_bwd(const float x[3], float xn, const float y[3],
                                              const float dy[3], float dx[3]) {
    if (xn >= 1e-12f) {
        const float yd = y[0] * dy[0] + y[1] * dy[1] + y[2] * dy[2];
        for (int d = 0; d < 3; ++d) dx[d] = (dy[d] - y[d] * yd) / xn;
    } else {
        for (int d = 0; d < 3; ++d) dx[d] = dy[d] / 1e-12f;
    }
}

// ReLU variant of activate() for the radiance networks (models/network_utils.py:136-140)
__device__ __forceinline__ void activate_relu(const float (&Z)[8][4], uint32_t (&hh)[4][4],
                                              uint32_t (&hl)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const float(&z)[4] = Z[2 * kt + half];
            const Split s0 = split2(fmaxf(z[0], 0.f), fmaxf(z[1], 0.f));
            const Split s1 = split2(fmaxf(z[2], 0.f), fmaxf(z[3], 0.f));
            hh[kt][2 * half] = s0.hi;
            hl[kt][2 * half] = s0.lo;
            hh[kt][2 * half + 1] = s1.hi;
            hl[kt][2 * half + 1] = s1.lo;
        }
    }
}

}  // namespace angelo
