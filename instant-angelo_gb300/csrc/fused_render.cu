// Fused radiance network and fused compositing.
//
// Radiance (models/texture.py:23-58): per 128-sample tile the input rows
// [feature, SH4((d+1)/2), normalize(grad)] are staged in shared memory as
// bf16 hi/lo operands, the ReLU MLP runs on the tcgen05 tensor cores (bf16x3,
// fp32 accumulation in tensor memory), and the output sigmoid (plus
// sigmoid(feature[1:4]) for the dual-colour network) is applied in the
// epilogue.  The backward recomputes the activations from the same inputs (no
// stash) and returns dL/dfeature, dL/dgrad and dL/dW.
//
// Compositing (models/neus.py:117-139, 234-248 with nerfacc 0.3.3 weights):
// one warp per ray walks the ray's samples in chunks of 32: NeuS alpha from
// the SDF, normal, direction and interval (in fp64 when inv_s exceeds the
// gate, where the sigmoid difference cancels), log-space transmittance by a
// warp prefix sum of log(1 - alpha) carried across chunks, weights (zero
// once T < early_stop_eps), and the per-ray sums of w, w*t, w*rgb, w*n.  The
// backward walks the chunks in reverse with an affine warp scan
// R_{j-1} = (1 - a_j) R_j + g_j a_j, so dL/dalpha_j = T_j (g_j - R_j) needs no
// division.
#include <math.h>

#include "common.cuh"
#include "mlp.cuh"
#include "sh.cuh"
#include "tc.cuh"
#include "tc_mlp.cuh"

using namespace angelo;

namespace {

constexpr int kXCols = 96;           // widest staged input (6 k-tiles)

struct RadLayout {
    int k_tiles1;   // input k-tiles (ceil(in_dim / 16))
    int in_dim;
    int feat_dim;   // width of the feature input
    // tensor-core operands, bf16 hi then lo, K-major [n][k] (Y = X W^T): W1
    // 64 x 16 k_tiles1, W2 64 x 64, W3 16 x 64 (rows 3 .. 15 zero); fp32 b1,
    // b2, b3 (16) and W3 (3 x 64)
    int64_t off_tw1, off_tw2, off_tw3, off_b1, off_b2, off_b3, off_w3, bytes;
};

RadLayout rad_layout(int feat_dim) {
    RadLayout L{};
    L.feat_dim = feat_dim;
    L.in_dim = feat_dim + 16 + 3;
    L.k_tiles1 = (L.in_dim + 15) / 16;
    int64_t o = 0;
    auto take = [&](int64_t b) { const int64_t r = o; o += (b + 15) / 16 * 16; return r; };
    L.off_tw1 = take(2 * 64 * 16 * L.k_tiles1 * 2);
    L.off_tw2 = take(2 * 64 * 64 * 2);
    L.off_tw3 = take(2 * 16 * 64 * 2);
    L.off_b1 = take(64 * 4);
    L.off_b2 = take(64 * 4);
    L.off_b3 = take(16 * 4);
    L.off_w3 = take(3 * 64 * 4);
    L.bytes = o;
    return L;
}

__device__ __forceinline__ float rad_w(int layer, int n, int k, const float *W1, const float *W2,
                                       const float *W3, int in_dim) {
    if (layer == 1) return (n < 64 && k < in_dim) ? W1[n * in_dim + k] : 0.f;
    if (layer == 2) return (n < 64 && k < 64) ? W2[n * 64 + k] : 0.f;
    return (n < 3 && k < 64) ? W3[n * 64 + k] : 0.f;
}

__global__ void rad_prep_kernel(const float *W1, const float *b1, const float *W2, const float *b2,
                                const float *W3, const float *b3, RadLayout L, int fp16, char *net) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int K1 = 16 * L.k_tiles1;
    const int n1 = 64 * K1, n2 = 64 * 64, n3 = 16 * 64;
    int layer, n, k, K;
    int64_t off, half;
    if (i < n1) {
        layer = 1, K = K1, n = i / K1, k = i % K1, off = L.off_tw1, half = (int64_t)n1 * 2;
    } else if ((i -= n1) < n2) {
        layer = 2, K = 64, n = i / 64, k = i % 64, off = L.off_tw2, half = (int64_t)n2 * 2;
    } else if ((i -= n2) < n3) {
        layer = 3, K = 64, n = i / 64, k = i % 64, off = L.off_tw3, half = (int64_t)n3 * 2;
    } else {
        i -= n3;
        float *fb1 = reinterpret_cast<float *>(net + L.off_b1);
        float *fb2 = reinterpret_cast<float *>(net + L.off_b2);
        float *fb3 = reinterpret_cast<float *>(net + L.off_b3);
        float *fw3 = reinterpret_cast<float *>(net + L.off_w3);
        if (i < 64) fb1[i] = b1[i];
        else if (i < 128) fb2[i - 64] = b2[i - 64];
        else if (i < 144) fb3[i - 128] = i - 128 < 3 ? b3[i - 128] : 0.f;
        else if (i < 144 + 192) fw3[i - 144] = W3[i - 144];
        return;
    }
    const float w = rad_w(layer, n, k, W1, W2, W3, L.in_dim);
    const Split sp = fp16 ? split2h(w, 0.0f) : split2(w, 0.0f);
    const uint32_t o = tc::kmajor_offset(n, k, K);
    *reinterpret_cast<uint16_t *>(net + off + o) = (uint16_t)(sp.hi & 0xFFFFu);
    *reinterpret_cast<uint16_t *>(net + off + half + o) = (uint16_t)(sp.lo & 0xFFFFu);
}

int rad_prep_threads(const RadLayout &L) { return 64 * 16 * L.k_tiles1 + 64 * 64 + 16 * 64 + 144 + 192; }

struct RadParams {
    RadLayout L;
    const char *net;
    const float *feature;
    int64_t feat_stride;
    const float *grad;
    const int32_t *ray_idx;
    const float *rays_d;
    int64_t S;
    int dual;
    int passes;   // forward tensor-core products per layer: 3 (hi/lo x3) or 1 (hi parts alone)
    int fp16;     // forward operands fp16 (the buffer prepared in fp16) instead of bf16
    int vec4;     // feature / d_feature rows start 16-byte aligned: 4-float accesses
    float *rgb;
    const float *g_rgb;
    float *d_feature;
    float *d_grad;
    float *d_net;
};

__device__ unsigned int g_rad_tc_timeouts;   // CTAs that stopped waiting for the tensor cores

__device__ __forceinline__ float sigm(float v) { return 1.0f / (1.0f + __expf(-v)); }

// SH4 of the viewing direction as the reference feeds it ((d + 1) / 2, then
// the encoder's 2 x - 1) and the unit normal of the SDF gradient, for sample s
__device__ __forceinline__ void rad_sh_normal(const RadParams &P, int64_t s, float sh[16], float nrm[3]) {
    const float *d = P.rays_d + (int64_t)P.ray_idx[s] * 3;
    const float x = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[0], 1.f), 2.f), 2.f), 1.f);
    const float y = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[1], 1.f), 2.f), 2.f), 1.f);
    const float z = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[2], 1.f), 2.f), 2.f), 1.f);
    sh4_eval(x, y, z, sh);
    if (!P.grad) {
        // a radiance network without a normal input (VolumeRadiance of the
        // learned background): the normal columns stay zero
        nrm[0] = nrm[1] = nrm[2] = 0.f;
        return;
    }
    const float *g = P.grad + s * 3;
    const float gn = fmaxf(sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12f);
#pragma unroll
    for (int k = 0; k < 3; ++k) nrm[k] = g[k] / gn;
}

// The input row [feature (F), SH (16), normal (3), 0 ...] of sample s, the
// 16-column blocks slice, slice + 4, ... of it staged K-major (16 KT1 columns)
template <int KT1, bool FP16 = false>
__device__ __forceinline__ void rad_stage_x(const RadParams &P, int64_t s, bool v, int row, int slice, char *xh,
                                            char *xl, bool with_lo = true) {
    const int F = P.L.feat_dim;
    for (int b = slice; b < KT1; b += 4) {
        const int c0 = 16 * b;
        float x[16];
        const float *frow = P.feature + (v ? s : 0) * P.feat_stride;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = c0 + 4 * q;
            if (v && P.vec4 && c + 3 < F) {
                const float4 f = __ldg(reinterpret_cast<const float4 *>(frow + c));
                x[4 * q] = f.x;
                x[4 * q + 1] = f.y;
                x[4 * q + 2] = f.z;
                x[4 * q + 3] = f.w;
            } else {
#pragma unroll
                for (int t = 0; t < 4; ++t) x[4 * q + t] = (v && c + t < F) ? frow[c + t] : 0.f;
            }
        }
        if (v && c0 + 16 > F && c0 < F + 19) {
            float sh[16], nrm[3];
            rad_sh_normal(P, s, sh, nrm);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int c = c0 + j - F;
                if (c >= 0 && c < 16) x[j] = sh[c];
                else if (c >= 16 && c < 19) x[j] = nrm[c - 16];
            }
        }
        stage16f<FP16>(xh, xl, row, c0, 16 * KT1, x, with_lo);
    }
}

template <int KT1>
struct RadShape {
    static constexpr int K1 = 16 * KT1;
    // bytes of one (hi or lo) half
    static constexpr uint32_t w1 = 64 * K1 * 2, w2 = 64 * 64 * 2, w3 = 16 * 64 * 2;
    static constexpr uint32_t x = 128 * K1 * 2, h = 128 * 64 * 2, y = 128 * 16 * 2, ones = 128 * 16 * 2;
    static constexpr uint32_t off_w1 = 0, off_w2 = 2 * w1, off_w3 = off_w2 + 2 * w2, off_x = off_w3 + 2 * w3;
    // forward: one activation staging (H1, then H2)
    static constexpr uint32_t f_h = off_x + 2 * x, f_vec = f_h + 2 * h, f_bar = f_vec + 144 * 4,
                              f_bytes = f_bar + 16;
    // backward
    static constexpr uint32_t b_h1 = off_x + 2 * x,   // H1, then dZ1
        b_h2 = b_h1 + 2 * h, b_z = b_h2 + 2 * h, b_y = b_z + 2 * h, b_ones = b_y + 2 * y,
                              b_vec = b_ones + ones,                 // b1, b2, b3 (16), W3 (3 x 64)
        b_db3 = b_vec + (144 + 192) * 4, b_bar = b_db3 + 16 * 4, b_bytes = b_bar + 32;
    // backward tensor-memory columns
    static constexpr uint32_t tA = 0, tB = 64, tW1 = tB + (K1 > 64 ? K1 : 64), tW2 = tW1 + K1, tW3 = tW2 + 64,
                              tb1 = tW3 + 16, tb2 = tb1 + 16, used = tb2 + 16;
};

// Radiance forward on tcgen05 (models/texture.py:23-58 with the dual colour of
// :100-149): per 128-sample tile, Z1 = X W1^T, ReLU, Z2 = H1 W2^T, ReLU,
// out = H2 W3^T, sigmoid (+ sigmoid(feature[1:4])).  The next tile's input is
// staged while the current tile's later layers run.  FP16: fp16 operands
// (the buffer prepared in fp16); one pass stages and multiplies the hi parts.
template <int KT1, bool FP16>
__global__ void __launch_bounds__(kTcThreads, 1) rad_fwd_tc_kernel(const __grid_constant__ RadParams P) {
    using Sh = RadShape<KT1>;
    constexpr int K1 = Sh::K1;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane, slice = warp >> 2;
    const RadLayout &L = P.L;
    auto copy16 = [&](uint32_t dst, int64_t src, uint32_t bytes) {
        for (uint32_t i = tid * 16; i < bytes; i += kTcThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(Sh::off_w1, L.off_tw1, 2 * Sh::w1);
    copy16(Sh::off_w2, L.off_tw2, 2 * Sh::w2);
    copy16(Sh::off_w3, L.off_tw3, 2 * Sh::w3);
    float *vec = reinterpret_cast<float *>(smem + Sh::f_vec);   // b1 [64], b2 [64], b3 [16]
    for (int i = tid; i < 144; i += kTcThreads)
        vec[i] = i < 64 ? reinterpret_cast<const float *>(P.net + L.off_b1)[i]
                 : i < 128 ? reinterpret_cast<const float *>(P.net + L.off_b2)[i - 64]
                           : reinterpret_cast<const float *>(P.net + L.off_b3)[i - 128];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + Sh::f_bar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    char *xh = smem + Sh::off_x, *xl = xh + Sh::x, *hh = smem + Sh::f_h, *hl = hh + Sh::h;
    if (warp == 0) {
        tc::tmem_alloc(slot, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(bar, 1);
    tc_publish();
    const uint32_t tmem = *slot;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t sW1 = tc::smem_addr(smem + Sh::off_w1), sW2 = tc::smem_addr(smem + Sh::off_w2),
                   sW3 = tc::smem_addr(smem + Sh::off_w3), sX = tc::smem_addr(xh), sH = tc::smem_addr(hh);
    const TcOp Xk = op_k(sX, Sh::x, K1), Hk = op_k(sH, Sh::h, 64);
    const TcOp W1k = op_k(sW1, Sh::w1, K1), W2k = op_k(sW2, Sh::w2, 64), W3k = op_k(sW3, Sh::w3, 64);
    constexpr uint32_t id64 = tc::idesc_f32(128, 64, FP16), id16 = tc::idesc_f32(128, 16, FP16);
    const bool with_lo = P.passes != 1;
    uint32_t phase = 0;
    bool alive = true;
    const int64_t n_tiles = (P.S + 127) / 128;
    if ((int64_t)blockIdx.x < n_tiles)
        rad_stage_x<KT1, FP16>(P, blockIdx.x * 128 + row, blockIdx.x * 128 + row < P.S, row, slice, xh, xl, with_lo);
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const int64_t s = t * 128 + row;
        const bool v = s < P.S;
        tc_publish();
        if (tid == 0) {
            tc_mma_p<KT1>(tmem, Xk, W1k, id64, false, P.passes);
            tc::commit(bar);
        }
        if (!(alive = tc_wait_all(bar, phase))) break;
        phase ^= 1;
        // the input staging is free: the next tile's
        const int64_t tn = t + gridDim.x;
        if (tn < n_tiles) rad_stage_x<KT1, FP16>(P, tn * 128 + row, tn * 128 + row < P.S, row, slice, xh, xl, with_lo);
#pragma unroll 1
        for (int layer = 0; layer < 2; ++layer) {
            float z[16];
            tc::ld16(tmem + lane_off + 64 * layer + 16 * slice, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) z[j] = fmaxf(z[j] + vec[64 * layer + 16 * slice + j], 0.f);
            stage16f<FP16>(hh, hl, row, 16 * slice, 64, z, with_lo);
            tc_publish();
            if (tid == 0) {
                if (layer == 0) tc_mma_p<4>(tmem + 64, Hk, W2k, id64, false, P.passes);
                else tc_mma_p<4>(tmem, Hk, W3k, id16, false, P.passes);
                tc::commit(bar);
            }
            if (!(alive = tc_wait_all(bar, phase))) break;
            phase ^= 1;
        }
        if (!alive) break;
        if (slice == 0) {
            float o[16];
            tc::ld16(tmem + lane_off, o);
            if (v) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float val = sigm(o[c] + vec[128 + c]);
                    if (P.dual) val += sigm(P.feature[s * P.feat_stride + 1 + c]);
                    P.rgb[s * 3 + c] = val;
                }
            }
        }
    }
    if (!alive && tid == 0) atomicAdd(&g_rad_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

// dL/dX block b (columns 16 b ..) of sample s: dL/dfeature (plus the dual
// colour's sigmoid term on columns 1..3) and, from the normal columns,
// dL/dgrad through normalize (models/texture.py:35)
__device__ __forceinline__ void rad_dx_out(const RadParams &P, int64_t s, int b, const float (&dx)[16],
                                           const float (&dual_g)[3]) {
    const int F = P.L.feat_dim;
    float dn[3] = {0.f, 0.f, 0.f};
    bool has_n = false;
    float o[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int c = 16 * b + j;
        o[j] = dx[j];
        if (P.dual && c >= 1 && c <= 3) o[j] += dual_g[c - 1];
        if (c >= F + 16 && c < F + 19) {
            dn[c - F - 16] = dx[j];
            has_n = true;
        }
    }
    float *drow = P.d_feature + s * P.feat_stride;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = 16 * b + 4 * q;
        if (P.vec4 && c + 3 < F) {
            *reinterpret_cast<float4 *>(drow + c) = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (c + t < F) drow[c + t] = o[4 * q + t];
        }
    }
    if (!has_n || !P.d_grad) return;
    const float *g = P.grad + s * 3;
    const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    const float den = fmaxf(gn, 1e-12f);
    float n[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = g[k] / den;
    if (gn >= 1e-12f) {
        const float nd = n[0] * dn[0] + n[1] * dn[1] + n[2] * dn[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) P.d_grad[s * 3 + k] = (dn[k] - n[k] * nd) / gn;
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) P.d_grad[s * 3 + k] = dn[k] / 1e-12f;
    }
}

// Radiance backward on tcgen05: the forward recomputed per 128-sample tile,
// then dY through the output sigmoid, dH2 = dY W3 (rank three, in registers),
// dH1 = dZ2 W2 with dW2 += dZ2^T H1, db2 and dW3^T += H2^T dY, dX = dZ1 W1
// with dW1 += dZ1^T X and db1; the weight gradients stay in tensor memory
// (M = 64 accumulators) for the CTA's whole loop; dX gives dL/dfeature and,
// through the normalisation, dL/dgrad.
template <int KT1>
__global__ void __launch_bounds__(kTcThreads, 1) rad_bwd_tc_kernel(const __grid_constant__ RadParams P) {
    using Sh = RadShape<KT1>;
    constexpr int K1 = Sh::K1;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane, slice = warp >> 2;
    const RadLayout &L = P.L;
    auto copy16 = [&](uint32_t dst, int64_t src, uint32_t bytes) {
        for (uint32_t i = tid * 16; i < bytes; i += kTcThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(Sh::off_w1, L.off_tw1, 2 * Sh::w1);
    copy16(Sh::off_w2, L.off_tw2, 2 * Sh::w2);
    copy16(Sh::off_w3, L.off_tw3, 2 * Sh::w3);
    float *vec = reinterpret_cast<float *>(smem + Sh::b_vec);   // b1 [64], b2 [64], b3 [16], W3 [3][64]
    for (int i = tid; i < 144 + 192; i += kTcThreads)
        vec[i] = i < 64 ? reinterpret_cast<const float *>(P.net + L.off_b1)[i]
                 : i < 128 ? reinterpret_cast<const float *>(P.net + L.off_b2)[i - 64]
                 : i < 144 ? reinterpret_cast<const float *>(P.net + L.off_b3)[i - 128]
                           : reinterpret_cast<const float *>(P.net + L.off_w3)[i - 144];
    const float *w3f = vec + 144;
    uint16_t *ones = reinterpret_cast<uint16_t *>(smem + Sh::b_ones);
    fill_ones_operand(ones, tid, kTcThreads);
    float *db3 = reinterpret_cast<float *>(smem + Sh::b_db3);
    for (int i = tid; i < 16; i += kTcThreads) db3[i] = 0.f;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + Sh::b_bar);   // [0] epilogue, [1] round
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 2);
    char *xh = smem + Sh::off_x, *xl = xh + Sh::x, *h1h = smem + Sh::b_h1, *h1l = h1h + Sh::h;
    char *h2h = smem + Sh::b_h2, *h2l = h2h + Sh::h, *zh = smem + Sh::b_z, *zl = zh + Sh::h;
    char *yh = smem + Sh::b_y, *yl = yh + Sh::y;
    if (warp == 0) {
        tc::tmem_alloc(slot, 512);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc_publish();
    const uint32_t tmem = *slot;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    tmem_zero(tmem + lane_off, Sh::tW1, Sh::used, slice);
    tc_publish();
    const uint32_t sW1 = tc::smem_addr(smem + Sh::off_w1), sW2 = tc::smem_addr(smem + Sh::off_w2),
                   sW3 = tc::smem_addr(smem + Sh::off_w3), sX = tc::smem_addr(xh), sH1 = tc::smem_addr(h1h),
                   sH2 = tc::smem_addr(h2h), sZ = tc::smem_addr(zh), sY = tc::smem_addr(yh),
                   sOnes = tc::smem_addr(ones);
    const TcOp W1k = op_k(sW1, Sh::w1, K1), W1t = op_t(sW1, Sh::w1, K1);
    const TcOp W2k = op_k(sW2, Sh::w2, 64), W2t = op_t(sW2, Sh::w2, 64), W3k = op_k(sW3, Sh::w3, 64);
    const TcOp Xk = op_k(sX, Sh::x, K1), Xt = op_t(sX, Sh::x, K1);
    const TcOp H1k = op_k(sH1, Sh::h, 64), H1t = op_t(sH1, Sh::h, 64), H2k = op_k(sH2, Sh::h, 64),
               H2t = op_t(sH2, Sh::h, 64);
    const TcOp Zk = op_k(sZ, Sh::h, 64), Zt = op_t(sZ, Sh::h, 64), Yt = op_t(sY, Sh::y, 16),
               Ones = op_t(sOnes, 0u, 16);
    constexpr uint32_t id64 = tc::idesc_bf16_f32(128, 64), id_out = tc::idesc_bf16_f32(128, 16);
    constexpr uint32_t id_dh = tc::idesc_bf16_f32(128, 64, 0, 1), id_dx = tc::idesc_bf16_f32(128, K1, 0, 1);
    constexpr uint32_t id_w1 = tc::idesc_bf16_f32(64, K1, 1, 1), id_w2 = tc::idesc_bf16_f32(64, 64, 1, 1),
                       id_16 = tc::idesc_bf16_f32(64, 16, 1, 1);
    uint32_t ph0 = 0, ph1 = 0;
    bool alive = true;
    const int64_t n_tiles = (P.S + 127) / 128;
    bool first = true;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const int64_t s = t * 128 + row;
        const bool v = s < P.S;
        if (!first) {
            if (!(alive = tc_wait_all(&bar[1], ph1))) break;
            ph1 ^= 1;
        }
        first = false;
        rad_stage_x<KT1>(P, s, v, row, slice, xh, xl);
        tc_publish();
        // forward, recomputed: Z1, Z2, out
        if (tid == 0) {
            tc_mma<KT1>(tmem + Sh::tA, Xk, W1k, id64, false);
            tc::commit(&bar[0]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        uint32_t m1 = 0, m2 = 0;   // ReLU masks of this slice
        {
            float z[16];
            tc::ld16(tmem + lane_off + Sh::tA + 16 * slice, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                z[j] += vec[16 * slice + j];
                m1 |= (z[j] > 0.f ? 1u : 0u) << j;
                z[j] = fmaxf(z[j], 0.f);
            }
            stage16(h1h, h1l, row, 16 * slice, 64, z);
        }
        tc_publish();
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tB, H1k, W2k, id64, false);
            tc::commit(&bar[0]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        {
            float z[16];
            tc::ld16(tmem + lane_off + Sh::tB + 16 * slice, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                z[j] += vec[64 + 16 * slice + j];
                m2 |= (z[j] > 0.f ? 1u : 0u) << j;
                z[j] = fmaxf(z[j], 0.f);
            }
            stage16(h2h, h2l, row, 16 * slice, 64, z);
        }
        tc_publish();
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tA, H2k, W3k, id_out, false);
            tc::commit(&bar[0]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        // dL/d(out) through the sigmoid, dH2 = dY W3, dZ2; the dual colour's
        // dL/dfeature[1..3] is kept by slice 0 for the dX epilogue
        float dual_g[3] = {0.f, 0.f, 0.f};
        {
            float o[16], dy[3];
            tc::ld16(tmem + lane_off + Sh::tA, o);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float sg = sigm(o[c] + vec[128 + c]);
                dy[c] = v ? P.g_rgb[s * 3 + c] * sg * (1.f - sg) : 0.f;
            }
            float dz[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int u = 16 * slice + j;
                const float dh = dy[0] * w3f[u] + dy[1] * w3f[64 + u] + dy[2] * w3f[128 + u];
                dz[j] = (m2 >> j) & 1u ? dh : 0.f;
            }
            stage16(zh, zl, row, 16 * slice, 64, dz);
            if (slice == 0) {
                float yv[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) yv[j] = j < 3 ? dy[j] : 0.f;
                stage16(yh, yl, row, 0, 16, yv);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float a = dy[c];
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
                    if (lane == 0 && a != 0.f) red_add(db3 + c, a);
                }
                if (P.dual && v) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float sf = sigm(P.feature[s * P.feat_stride + 1 + c]);
                        dual_g[c] = P.g_rgb[s * 3 + c] * sf * (1.f - sf);
                    }
                }
            }
        }
        tc_publish();
        // dH1 (epilogue), then dW2, db2, dW3
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tA, Zk, W2t, id_dh, false);
            tc::commit(&bar[0]);
            tc_mma<8>(tmem + Sh::tW2, Zt, H1t, id_w2, true);
            tc_mma<8>(tmem + Sh::tb2, Zt, Ones, id_16, true, true);
            tc_mma<8>(tmem + Sh::tW3, H2t, Yt, id_16, true);
            tc::commit(&bar[1]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        {
            float dz[16];
            tc::ld16(tmem + lane_off + Sh::tA + 16 * slice, dz);
#pragma unroll
            for (int j = 0; j < 16; ++j) dz[j] = (m1 >> j) & 1u ? dz[j] : 0.f;
            if (!(alive = tc_wait_all(&bar[1], ph1))) break;
            ph1 ^= 1;
            stage16(h1h, h1l, row, 16 * slice, 64, dz);   // H1 -> dZ1
        }
        tc_publish();
        // dX (epilogue), then dW1, db1
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tB, H1k, W1t, id_dx, false);
            tc::commit(&bar[0]);
            tc_mma<8>(tmem + Sh::tW1, H1t, Xt, id_w1, true);
            tc_mma<8>(tmem + Sh::tb1, H1t, Ones, id_16, true, true);
            tc::commit(&bar[1]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        for (int b = slice; b < KT1; b += 4) {
            float dx[16];
            __syncwarp();
            tc::ld16(tmem + lane_off + Sh::tB + 16 * b, dx);
            if (v) rad_dx_out(P, s, b, dx, dual_g);
        }
    }
    if (alive && !first) alive = tc_wait_all(&bar[1], ph1);
    if (alive) {
        // add the CTA's gradients: tensor-memory rows 16 (warp % 4) + lane
        const int unit = 16 * (warp & 3) + lane;
        float *dW2 = P.d_net + 64 * K1, *dW3 = dW2 + 64 * 64, *db1 = dW3 + 16 * 64, *db2 = db1 + 64,
              *dB3 = db2 + 64;
        for (uint32_t c0 = Sh::tW1 + 16 * slice; c0 < Sh::used; c0 += 64) {
            float w[16];
            __syncwarp();
            tc::ld16(tmem + lane_off + c0, w);
#pragma unroll
            for (int j = 0; j < 16 && lane < 16; ++j) {
                const uint32_t c = c0 + j;
                float *dst = nullptr;
                if (c < Sh::tW2) dst = P.d_net + unit * K1 + (c - Sh::tW1);
                else if (c < Sh::tW3) dst = dW2 + unit * 64 + (c - Sh::tW2);
                else if (c < Sh::tb1) dst = dW3 + (c - Sh::tW3) * 64 + unit;
                else if (c == Sh::tb1) dst = db1 + unit;
                else if (c == Sh::tb2) dst = db2 + unit;
                if (dst && w[j] != 0.f) atomicAdd(dst, w[j]);
            }
        }
        for (int o = tid; o < 16; o += kTcThreads)
            if (db3[o] != 0.f) atomicAdd(dB3 + o, db3[o]);
    }
    if (!alive && tid == 0) atomicAdd(&g_rad_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------ compositing

struct CompParams {
    const int64_t *off;
    int64_t n_rays;
    const float *sdf, *grad, *t0, *t1, *rays_d, *rgb, *variance, *bg;
    float cos_ratio, eps, gate;
    // forward outputs
    float *opacity, *depth, *comp_rgb, *comp_normal, *comp_full, *acc_n, *weights, *trans, *alpha;
    // backward
    const float *g_opacity, *g_depth, *g_rgb, *g_normal, *g_full;
    float *d_sdf, *d_grad, *d_rgb, *d_variance;
};

__device__ __forceinline__ float inv_s_of(const float *variance) {
    const float s = expf(*variance * 10.0f);
    return fminf(fmaxf(s, 1e-6f), 1e6f);
}

struct AlphaParts {
    float alpha, u, pc, nc, prv, nxt, cosv, iter;
};

// NeuSModel.get_alpha for one sample; fp64 for the sigmoid difference when
// inv_s > gate.
__device__ __forceinline__ AlphaParts neus_alpha(float sdf, float cosv, float dist, float s,
                                                 float ratio, float gate) {
    AlphaParts a;
    a.cosv = cosv;
    a.iter = -(fmaxf(-cosv * 0.5f + 0.5f, 0.f) * (1.0f - ratio) + fmaxf(-cosv, 0.f) * ratio);
    a.nxt = sdf + a.iter * dist * 0.5f;
    a.prv = sdf - a.iter * dist * 0.5f;
    if (s > gate) {
        const double pc = 1.0 / (1.0 + exp(-(double)a.prv * (double)s));
        const double nc = 1.0 / (1.0 + exp(-(double)a.nxt * (double)s));
        const double u = (pc - nc + 1e-5) / (pc + 1e-5);
        a.pc = (float)pc;
        a.nc = (float)nc;
        a.u = (float)u;
    } else {
        a.pc = 1.0f / (1.0f + expf(-a.prv * s));
        a.nc = 1.0f / (1.0f + expf(-a.nxt * s));
        a.u = (a.pc - a.nc + 1e-5f) / (a.pc + 1e-5f);
    }
    a.alpha = fminf(fmaxf(a.u, 0.f), 1.f);
    return a;
}

__device__ __forceinline__ void sample_normal(const float *g, float n[3], float *gn) {
    *gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    const float den = fmaxf(*gn, 1e-12f);
    for (int k = 0; k < 3; ++k) n[k] = g[k] / den;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) comp_fwd_kernel(const __grid_constant__ CompParams P) {
    const int lane = threadIdx.x & 31;
    const int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (ray >= P.n_rays) return;
    const float s = inv_s_of(P.variance);
    const float d0 = P.rays_d[ray * 3], d1 = P.rays_d[ray * 3 + 1], d2 = P.rays_d[ray * 3 + 2];
    const int64_t b = P.off[ray], e = P.off[ray + 1];
    float carry = 0.f;  // log T at the chunk start
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float log_eps = logf(P.eps);
    for (int64_t c0 = b; c0 < e; c0 += 32) {
        const int64_t j = c0 + lane;
        const bool v = j < e;
        float a = 0.f, tm = 0.f, n[3] = {0.f, 0.f, 0.f}, l = 0.f;
        if (v) {
            float gn;
            sample_normal(P.grad + j * 3, n, &gn);
            const float cosv = d0 * n[0] + d1 * n[1] + d2 * n[2];
            const float t0 = P.t0[j], t1 = P.t1[j];
            tm = (t0 + t1) * 0.5f;
            a = neus_alpha(P.sdf[j], cosv, t1 - t0, s, P.cos_ratio, P.gate).alpha;
            l = log1pf(-a);
        }
        // inclusive prefix sum of log(1 - a), then exclusive by a one-lane shift
        float incl = l;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        float excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = 0.f;
        const float logT = carry + excl;
        const float T = __expf(logT);
        const bool live = T >= P.eps;
        const float wgt = v && live ? a * T : 0.f;
        if (v) {
            P.weights[j] = wgt;
            if (P.trans) P.trans[j] = T;
            if (P.alpha) P.alpha[j] = a;
            const float *c = P.rgb + j * 3;
            acc[0] += wgt;
            acc[1] += wgt * tm;
            acc[2] += wgt * c[0];
            acc[3] += wgt * c[1];
            acc[4] += wgt * c[2];
            acc[5] += wgt * n[0];
            acc[6] += wgt * n[1];
            acc[7] += wgt * n[2];
        }
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0) {
        const float op = acc[0];
        P.opacity[ray] = op;
        P.depth[ray] = acc[1];
        float nn = sqrtf(acc[5] * acc[5] + acc[6] * acc[6] + acc[7] * acc[7]);
        nn = fmaxf(nn, 1e-12f);
        for (int k = 0; k < 3; ++k) {
            P.comp_rgb[ray * 3 + k] = acc[2 + k];
            P.comp_full[ray * 3 + k] = acc[2 + k] + P.bg[k] * (1.0f - op);
            P.comp_normal[ray * 3 + k] = op > 0.1f ? acc[5 + k] / nn : 0.f;
            if (P.acc_n) P.acc_n[ray * 3 + k] = acc[5 + k];
        }
    }
}

__global__ void __launch_bounds__(256) comp_bwd_kernel(const __grid_constant__ CompParams P) {
    const int lane = threadIdx.x & 31;
    const int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float ds_acc = 0.f;
    if (ray < P.n_rays) {
        const float s = inv_s_of(P.variance);
        const float d[3] = {P.rays_d[ray * 3], P.rays_d[ray * 3 + 1], P.rays_d[ray * 3 + 2]};
        const int64_t b = P.off[ray], e = P.off[ray + 1];
        // per-ray output gradients
        float g_op = P.g_opacity ? P.g_opacity[ray] : 0.f;
        const float g_dep = P.g_depth ? P.g_depth[ray] : 0.f;
        float g_c[3], g_an[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k) {
            const float gf = P.g_full ? P.g_full[ray * 3 + k] : 0.f;
            g_c[k] = (P.g_rgb ? P.g_rgb[ray * 3 + k] : 0.f) + gf;
            g_op -= gf * P.bg[k];
        }
        const float op = P.opacity[ray];
        if (P.g_normal && op > 0.1f) {
            const float *an = P.acc_n + ray * 3;
            const float nn = sqrtf(an[0] * an[0] + an[1] * an[1] + an[2] * an[2]);
            const float den = fmaxf(nn, 1e-12f);
            float cn[3], gcn[3];
            for (int k = 0; k < 3; ++k) {
                cn[k] = an[k] / den;
                gcn[k] = P.g_normal[ray * 3 + k];
            }
            if (nn >= 1e-12f) {
                const float dotv = cn[0] * gcn[0] + cn[1] * gcn[1] + cn[2] * gcn[2];
                for (int k = 0; k < 3; ++k) g_an[k] = (gcn[k] - cn[k] * dotv) / nn;
            } else {
                for (int k = 0; k < 3; ++k) g_an[k] = gcn[k] / 1e-12f;
            }
        }
        float R = 0.f;  // R at the last sample of the current chunk
        const int64_t n = e - b;
        for (int64_t c0 = b + ((n - 1) / 32) * 32; n > 0 && c0 >= b; c0 -= 32) {
            const int64_t j = c0 + lane;
            const bool v = j < e;
            float a = 0.f, T = 0.f, g = 0.f, wgt = 0.f, n3[3] = {0.f, 0.f, 0.f}, gn = 0.f;
            AlphaParts ap{};
            if (v) {
                sample_normal(P.grad + j * 3, n3, &gn);
                const float cosv = d[0] * n3[0] + d[1] * n3[1] + d[2] * n3[2];
                const float t0 = P.t0[j], t1 = P.t1[j];
                ap = neus_alpha(P.sdf[j], cosv, t1 - t0, s, P.cos_ratio, P.gate);
                a = ap.alpha;
                T = P.trans[j];
                wgt = P.weights[j];
                const float tm = (t0 + t1) * 0.5f;
                const float *c = P.rgb + j * 3;
                const float dw = g_op + g_dep * tm + g_c[0] * c[0] + g_c[1] * c[1] + g_c[2] * c[2] +
                                 g_an[0] * n3[0] + g_an[1] * n3[1] + g_an[2] * n3[2];
                g = (T >= P.eps) ? dw : 0.f;
                for (int k = 0; k < 3; ++k) P.d_rgb[j * 3 + k] = wgt * g_c[k];
            }
            // affine suffix scan: R_{l} = A_l * R_chunk_end + B_l with the map of
            // sample l+1 (a, b) = (1 - alpha, g * alpha); identity past the ray end
            const float am = v ? 1.f - a : 1.f, bm = v ? g * a : 0.f;
            float A = __shfl_down_sync(0xffffffffu, am, 1);
            float B = __shfl_down_sync(0xffffffffu, bm, 1);
            if (lane == 31) {
                A = 1.f;
                B = 0.f;
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float A2 = __shfl_down_sync(0xffffffffu, A, o);
                const float B2 = __shfl_down_sync(0xffffffffu, B, o);
                if (lane + o < 32) {
                    B = A * B2 + B;
                    A = A * A2;
                }
            }
            const float Rl = A * R + B;
            // carry into the previous chunk: R at its last sample = map of lane 0
            const float Rprev = am * Rl + bm;
            R = __shfl_sync(0xffffffffu, Rprev, 0);
            if (v) {
                const float da = T * (g - Rl);
                // alpha = clip(u, 0, 1)
                const float du = (ap.u >= 0.f && ap.u <= 1.f) ? da : 0.f;
                const float den = ap.pc + 1e-5f;
                const float dpc = du * ap.nc / (den * den);
                const float dnc = -du / den;
                const float dprv_arg = dpc * ap.pc * (1.f - ap.pc);   // d/d(prv*s)
                const float dnxt_arg = dnc * ap.nc * (1.f - ap.nc);
                const float dsdf = (dprv_arg + dnxt_arg) * s;
                const float t0 = P.t0[j], t1 = P.t1[j];
                const float dist = t1 - t0;
                // prv = sdf - iter*dist/2, nxt = sdf + iter*dist/2
                const float diter = (-dprv_arg + dnxt_arg) * s * dist * 0.5f;
                const float r = P.cos_ratio;
                const float dcos = diter * ((1.f - r) * 0.5f * ((-ap.cosv * 0.5f + 0.5f) > 0.f ? 1.f : 0.f) +
                                            r * ((-ap.cosv) > 0.f ? 1.f : 0.f));
                ds_acc += dprv_arg * ap.prv + dnxt_arg * ap.nxt;
                P.d_sdf[j] = dsdf;
                float dn[3];
                for (int k = 0; k < 3; ++k) dn[k] = dcos * d[k] + wgt * g_an[k];
                const float den2 = fmaxf(gn, 1e-12f);
                if (gn >= 1e-12f) {
                    const float nd = n3[0] * dn[0] + n3[1] * dn[1] + n3[2] * dn[2];
                    for (int k = 0; k < 3; ++k) P.d_grad[j * 3 + k] = (dn[k] - n3[k] * nd) / gn;
                } else {
                    for (int k = 0; k < 3; ++k) P.d_grad[j * 3 + k] = dn[k] / den2;
                }
            }
        }
    }
    // dL/dvariance: dL/ds * ds/dvariance with s = exp(10 v) inside the clip
    ds_acc = warp_sum(ds_acc);
    if (lane == 0 && ds_acc != 0.f) {
        const float sraw = expf(*P.variance * 10.0f);
        if (sraw >= 1e-6f && sraw <= 1e6f) atomicAdd(P.d_variance, ds_acc * sraw * 10.0f);
    }
}

// ------------------------------------------- density compositing (background)
// The learned background's compositing (models/neus.py:171-177 with nerfacc
// 0.3.3 render_weight_from_density and accumulate_along_rays), one warp per
// ray over chunks of 32 samples: tau_j = sigma_j (t1_j - t0_j), T_j =
// exp(-(tau_0 + .. + tau_{j-1})) from a warp prefix sum carried across the
// chunks, w_j = (1 - exp(-tau_j)) T_j; per ray opacity = sum w, depth =
// sum w (t0 + t1) / 2, rgb = sum w rgb + bg (1 - opacity).  The backward
// walks the chunks back to front with a warp suffix sum:
// dL/dsigma_j = dt_j (g_j T_j exp(-tau_j) - sum_{k>j} g_k w_k),
// g_j = dL/dw_j, dL/drgb_j = w_j dL/drgb.

struct DCompParams {
    const int64_t *off;
    int64_t n_rays;
    const float *sigma, *t0, *t1, *rgb, *bg;
    float *opacity, *depth, *comp_rgb, *weights, *trans;
    const float *g_opacity, *g_depth, *g_rgb;
    float *d_sigma, *d_rgb;
};

__global__ void __launch_bounds__(256) dcomp_fwd_kernel(const __grid_constant__ DCompParams P) {
    const int lane = threadIdx.x & 31;
    const int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (ray >= P.n_rays) return;
    const int64_t b = P.off[ray], e = P.off[ray + 1];
    float carry = 0.f;   // optical depth before the chunk
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int64_t c0 = b; c0 < e; c0 += 32) {
        const int64_t j = c0 + lane;
        const bool v = j < e;
        float tau = 0.f, tm = 0.f;
        if (v) {
            const float t0 = P.t0[j], t1 = P.t1[j];
            tau = __fmul_rn(P.sigma[j], __fsub_rn(t1, t0));
            tm = (t0 + t1) * 0.5f;
        }
        float incl = tau;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        float excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = 0.f;
        const float T = expf(-(carry + excl));
        if (v) {
            const float w = (1.0f - expf(-tau)) * T;
            P.weights[j] = w;
            P.trans[j] = T;
            const float *c = P.rgb + j * 3;
            acc[0] += w;
            acc[1] += w * tm;
            acc[2] += w * c[0];
            acc[3] += w * c[1];
            acc[4] += w * c[2];
        }
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0) {
        P.opacity[ray] = acc[0];
        P.depth[ray] = acc[1];
        for (int k = 0; k < 3; ++k) P.comp_rgb[ray * 3 + k] = acc[2 + k] + P.bg[k] * (1.0f - acc[0]);
    }
}

__global__ void __launch_bounds__(256) dcomp_bwd_kernel(const __grid_constant__ DCompParams P) {
    const int lane = threadIdx.x & 31;
    const int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (ray >= P.n_rays) return;
    const int64_t b = P.off[ray], e = P.off[ray + 1];
    float g_c[3], g_op = P.g_opacity ? P.g_opacity[ray] : 0.f;
    const float g_dep = P.g_depth ? P.g_depth[ray] : 0.f;
    for (int k = 0; k < 3; ++k) {
        g_c[k] = P.g_rgb ? P.g_rgb[ray * 3 + k] : 0.f;
        g_op -= g_c[k] * P.bg[k];   // rgb = .. + bg (1 - opacity)
    }
    float R = 0.f;   // sum of g_k w_k over the samples after the chunk
    const int64_t n = e - b;
    for (int64_t c0 = b + ((n - 1) / 32) * 32; n > 0 && c0 >= b; c0 -= 32) {
        const int64_t j = c0 + lane;
        const bool v = j < e;
        float gw = 0.f, w = 0.f, tau = 0.f, T = 0.f, dt = 0.f;
        if (v) {
            const float t0 = P.t0[j], t1 = P.t1[j];
            dt = __fsub_rn(t1, t0);
            tau = __fmul_rn(P.sigma[j], dt);
            const float tm = (t0 + t1) * 0.5f;
            const float *c = P.rgb + j * 3;
            w = P.weights[j];
            T = P.trans[j];
            gw = g_op + g_dep * tm + g_c[0] * c[0] + g_c[1] * c[1] + g_c[2] * c[2];
            for (int k = 0; k < 3; ++k) P.d_rgb[j * 3 + k] = w * g_c[k];
        }
        // inclusive suffix sum of g w within the chunk, then exclusive
        float suf = gw * w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_down_sync(0xffffffffu, suf, o);
            if (lane + o < 32) suf += y;
        }
        float after = __shfl_down_sync(0xffffffffu, suf, 1);
        if (lane == 31) after = 0.f;
        if (v) P.d_sigma[j] = dt * (gw * T * expf(-tau) - (after + R));
        R += __shfl_sync(0xffffffffu, suf, 0);
    }
}

}  // namespace

// ------------------------------------------------------------------ host API

extern "C" int angelo_density_composite_fwd(const int64_t *offsets, int64_t n_rays, const float *sigmas,
                                            const float *t_starts, const float *t_ends, const float *rgb,
                                            const float *bg, float *opacity, float *depth, float *comp_rgb,
                                            float *weights, float *trans, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "density_composite_fwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(offsets && sigmas && t_starts && t_ends && rgb && bg && opacity && depth && comp_rgb &&
                       weights && trans,
                   "density_composite_fwd: null pointer");
    DCompParams P{};
    P.off = offsets;
    P.n_rays = n_rays;
    P.sigma = sigmas;
    P.t0 = t_starts;
    P.t1 = t_ends;
    P.rgb = rgb;
    P.bg = bg;
    P.opacity = opacity;
    P.depth = depth;
    P.comp_rgb = comp_rgb;
    P.weights = weights;
    P.trans = trans;
    dcomp_fwd_kernel<<<blocks_for(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(P);
    return check_launch("density_composite_fwd");
}

extern "C" int angelo_density_composite_bwd(const int64_t *offsets, int64_t n_rays, const float *sigmas,
                                            const float *t_starts, const float *t_ends, const float *rgb,
                                            const float *bg, const float *weights, const float *trans,
                                            const float *g_opacity, const float *g_depth, const float *g_rgb,
                                            float *d_sigmas, float *d_rgb, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "density_composite_bwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(offsets && sigmas && t_starts && t_ends && rgb && bg && weights && trans && d_sigmas && d_rgb,
                   "density_composite_bwd: null pointer");
    DCompParams P{};
    P.off = offsets;
    P.n_rays = n_rays;
    P.sigma = sigmas;
    P.t0 = t_starts;
    P.t1 = t_ends;
    P.rgb = rgb;
    P.bg = bg;
    P.weights = const_cast<float *>(weights);   // read only in the backward
    P.trans = const_cast<float *>(trans);
    P.g_opacity = g_opacity;
    P.g_depth = g_depth;
    P.g_rgb = g_rgb;
    P.d_sigma = d_sigmas;
    P.d_rgb = d_rgb;
    dcomp_bwd_kernel<<<blocks_for(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(P);
    return check_launch("density_composite_bwd");
}

namespace angelo {
// CTAs of the radiance kernels that stopped waiting for the tensor cores
int64_t radiance_tc_timeouts(int reset) {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_rad_tc_timeouts, sizeof(v)) != cudaSuccess) return -1;
    if (reset) {
        const unsigned int z = 0;
        if (cudaMemcpyToSymbol(g_rad_tc_timeouts, &z, sizeof(z)) != cudaSuccess) return -1;
    }
    return (int64_t)v;
}
}  // namespace angelo

extern "C" int64_t angelo_radiance_net_bytes(int32_t feat_dim) {
    if (feat_dim < 1 || feat_dim + 19 > kXCols) return -1;
    return rad_layout(feat_dim).bytes;
}

extern "C" int64_t angelo_radiance_grad_size(int32_t feat_dim) {
    const int kt = (feat_dim + 19 + 15) / 16;
    return 64 * 16 * kt + 64 * 64 + 16 * 64 + 64 + 64 + 16;
}

extern "C" int angelo_radiance_prep_format(int32_t feat_dim, int32_t operand_format, const float *W1,
                                           const float *b1, const float *W2, const float *b2,
                                           const float *W3, const float *b3, void *net, void *stream) {
    ANGELO_REQUIRE(feat_dim >= 1 && feat_dim + 19 <= kXCols, "radiance_prep: feature width %d",
                   feat_dim);
    ANGELO_REQUIRE(W1 && b1 && W2 && b2 && W3 && b3 && net, "radiance_prep: null pointer");
    ANGELO_REQUIRE(operand_format == ANGELO_OPERAND_BF16 || operand_format == ANGELO_OPERAND_FP16,
                   "radiance_prep: operand_format %d", operand_format);
    const RadLayout L = rad_layout(feat_dim);
    rad_prep_kernel<<<blocks_for(rad_prep_threads(L), 256), 256, 0, as_stream(stream)>>>(
        W1, b1, W2, b2, W3, b3, L, operand_format == ANGELO_OPERAND_FP16, reinterpret_cast<char *>(net));
    return check_launch("radiance_prep");
}

extern "C" int angelo_radiance_prep(int32_t feat_dim, const float *W1, const float *b1,
                                    const float *W2, const float *b2, const float *W3,
                                    const float *b3, void *net, void *stream) {
    return angelo_radiance_prep_format(feat_dim, ANGELO_OPERAND_BF16, W1, b1, W2, b2, W3, b3, net, stream);
}

namespace {
template <int KT1, bool BWD, bool FP16 = false>
int launch_rad(const RadParams &P, cudaStream_t st) {
    using Sh = RadShape<KT1>;
    const size_t smem = BWD ? Sh::b_bytes : Sh::f_bytes;
    auto k = BWD ? rad_bwd_tc_kernel<KT1> : rad_fwd_tc_kernel<KT1, FP16>;
    static PersistentLaunch cfg;
    const int rc = persistent_setup(k, smem, kTcThreads, cfg, BWD ? "radiance_bwd" : "radiance_fwd");
    if (rc != ANGELO_OK) return rc;
    // tensor memory: the backward holds all 512 columns of an SM, the forward 128
    const int per_sm = std::min(cfg.per_sm, BWD ? 1 : 4);
    const int64_t tiles = (P.S + 127) / 128;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)cfg.sms * per_sm);
    k<<<grid, kTcThreads, smem, st>>>(P);
    return check_launch(BWD ? "radiance_bwd" : "radiance_fwd");
}

template <bool BWD>
int dispatch_rad(const RadParams &P, cudaStream_t st) {
    const bool f16 = !BWD && P.fp16;
    switch (P.L.k_tiles1) {
        case 2: return f16 ? launch_rad<2, BWD, true>(P, st) : launch_rad<2, BWD>(P, st);
        case 3: return f16 ? launch_rad<3, BWD, true>(P, st) : launch_rad<3, BWD>(P, st);
        case 6: return f16 ? launch_rad<6, BWD, true>(P, st) : launch_rad<6, BWD>(P, st);
        default:
            set_error("radiance: input width %d not instantiated (feature width 8, 16 or 68)", P.L.in_dim);
            return ANGELO_E_UNSUPPORTED;
    }
}
}  // namespace

extern "C" int angelo_radiance_fwd(int32_t feat_dim, const void *net, const float *feature,
                                   int64_t feat_stride, const float *grad, const int32_t *ray_idx,
                                   const float *rays_d, int64_t n, int32_t flags, float *rgb,
                                   void *stream) {
    ANGELO_REQUIRE((flags & ~7) == 0, "radiance_fwd: flags %d", flags);
    ANGELO_REQUIRE(feat_dim >= 1 && feat_dim + 19 <= kXCols, "radiance_fwd: feature width");
    ANGELO_REQUIRE(n >= 0, "radiance_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(net && feature && ray_idx && rays_d && rgb && feat_stride >= feat_dim,
                   "radiance_fwd: bad argument");
    RadParams P{};
    P.L = rad_layout(feat_dim);
    P.net = reinterpret_cast<const char *>(net);
    P.feature = feature;
    P.feat_stride = feat_stride;
    P.grad = grad;
    P.ray_idx = ray_idx;
    P.rays_d = rays_d;
    P.S = n;
    P.dual = flags & 1;
    P.passes = (flags & 2) ? 1 : 3;
    P.fp16 = (flags & 4) != 0;
    P.vec4 = (feat_stride % 4 == 0) && (reinterpret_cast<uintptr_t>(feature) % 16 == 0);
    P.rgb = rgb;
    return dispatch_rad<false>(P, as_stream(stream));
}

extern "C" int angelo_radiance_bwd(int32_t feat_dim, const void *net, const float *feature,
                                   int64_t feat_stride, const float *grad, const int32_t *ray_idx,
                                   const float *rays_d, int64_t n, int32_t dual, const float *g_rgb,
                                   float *d_feature, float *d_grad, float *d_net, void *stream) {
    ANGELO_REQUIRE(feat_dim >= 1 && feat_dim + 19 <= kXCols, "radiance_bwd: feature width");
    ANGELO_REQUIRE(n >= 0, "radiance_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(net && feature && ray_idx && rays_d && g_rgb && d_feature && d_net &&
                       feat_stride >= feat_dim && (grad != nullptr) == (d_grad != nullptr),
                   "radiance_bwd: bad argument");
    RadParams P{};
    P.L = rad_layout(feat_dim);
    P.net = reinterpret_cast<const char *>(net);
    P.feature = feature;
    P.feat_stride = feat_stride;
    P.grad = grad;
    P.ray_idx = ray_idx;
    P.rays_d = rays_d;
    P.S = n;
    P.dual = dual;
    P.g_rgb = g_rgb;
    P.d_feature = d_feature;
    P.d_grad = d_grad;
    P.d_net = d_net;
    P.vec4 = (feat_stride % 4 == 0) && (reinterpret_cast<uintptr_t>(feature) % 16 == 0) &&
             (reinterpret_cast<uintptr_t>(d_feature) % 16 == 0);
    return dispatch_rad<true>(P, as_stream(stream));
}

extern "C" int angelo_composite_fwd(const int64_t *offsets, int64_t n_rays, const float *sdf,
                                    const float *grad, const float *t_starts, const float *t_ends,
                                    const float *rays_d, const float *rgb, const float *variance,
                                    float cos_anneal_ratio, const float *bg, float early_stop_eps,
                                    float fp64_gate, float *opacity, float *depth, float *comp_rgb,
                                    float *comp_normal, float *comp_rgb_full, float *acc_normal,
                                    float *weights, float *trans, float *alpha, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "composite_fwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(offsets && sdf && grad && t_starts && t_ends && rays_d && rgb && variance && bg &&
                   opacity && depth && comp_rgb && comp_normal && comp_rgb_full && weights,
                   "composite_fwd: null argument");
    CompParams P{};
    P.off = offsets;
    P.n_rays = n_rays;
    P.sdf = sdf;
    P.grad = grad;
    P.t0 = t_starts;
    P.t1 = t_ends;
    P.rays_d = rays_d;
    P.rgb = rgb;
    P.variance = variance;
    P.bg = bg;
    P.cos_ratio = cos_anneal_ratio;
    P.eps = early_stop_eps;
    P.gate = fp64_gate;
    P.opacity = opacity;
    P.depth = depth;
    P.comp_rgb = comp_rgb;
    P.comp_normal = comp_normal;
    P.comp_full = comp_rgb_full;
    P.acc_n = acc_normal;
    P.weights = weights;
    P.trans = trans;
    P.alpha = alpha;
    comp_fwd_kernel<<<blocks_for(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(P);
    return check_launch("composite_fwd");
}

extern "C" int angelo_composite_bwd(const int64_t *offsets, int64_t n_rays, const float *sdf,
                                    const float *grad, const float *t_starts, const float *t_ends,
                                    const float *rays_d, const float *rgb, const float *variance,
                                    float cos_anneal_ratio, const float *bg, float early_stop_eps,
                                    float fp64_gate, const float *opacity,
                                    const float *acc_normal, const float *weights,
                                    const float *trans, const float *g_opacity,
                                    const float *g_depth, const float *g_comp_rgb,
                                    const float *g_comp_normal, const float *g_comp_rgb_full,
                                    float *d_sdf, float *d_grad, float *d_rgb, float *d_variance,
                                    void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "composite_bwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(offsets && sdf && grad && t_starts && t_ends && rays_d && rgb && variance && bg &&
                   opacity && acc_normal && weights && trans && d_sdf && d_grad && d_rgb &&
                   d_variance, "composite_bwd: null argument");
    CompParams P{};
    P.off = offsets;
    P.n_rays = n_rays;
    P.sdf = sdf;
    P.grad = grad;
    P.t0 = t_starts;
    P.t1 = t_ends;
    P.rays_d = rays_d;
    P.rgb = rgb;
    P.variance = variance;
    P.bg = bg;
    P.cos_ratio = cos_anneal_ratio;
    P.eps = early_stop_eps;
    P.gate = fp64_gate;
    P.opacity = const_cast<float *>(opacity);
    P.acc_n = const_cast<float *>(acc_normal);
    P.weights = const_cast<float *>(weights);
    P.trans = const_cast<float *>(trans);
    P.g_opacity = g_opacity;
    P.g_depth = g_depth;
    P.g_rgb = g_comp_rgb;
    P.g_normal = g_comp_normal;
    P.g_full = g_comp_rgb_full;
    P.d_sdf = d_sdf;
    P.d_grad = d_grad;
    P.d_rgb = d_rgb;
    P.d_variance = d_variance;
    comp_bwd_kernel<<<blocks_for(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(P);
    return check_launch("composite_bwd");
}
