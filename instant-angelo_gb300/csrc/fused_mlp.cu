// Fused VanillaMLP on the tcgen05 tensor cores (models/network_utils.py:96-140
// with ReLU between layers and no output activation): the learned
// background's density network (models/geometry.py:152-177, VanillaMLP of one
// hidden layer on [x*2-1, hash grid]) and any other ReLU MLP of one or two
// hidden layers of 64 units, in_dim <= 64 inputs and out_dim <= 16 outputs.
//
// A CTA of 16 warps owns 128 rows at a time (row r = tensor-memory lane r;
// four threads per row, one 16-column slice each).  The input rows X (fp32,
// any row stride) are staged in shared memory as bf16 hi/lo operands; every
// layer is three tcgen05 products (hi*hi + hi*lo + lo*hi, fp32 accumulation
// in tensor memory), bias and ReLU in the epilogue.  The forward stages the
// next tile's rows while the current tile's later layers run.  The backward
// recomputes the hidden activations from X (no stash), then
//   dH_last = dY W3            (rank out_dim, in registers)
//   dH1 = dZ2 W2,  dW2 += dZ2^T H1, db2  (two hidden layers)
//   dX = dZ1 W1,   dW1 += dZ1^T X,  db1,  dW3^T += H_last^T dY
// with the weight gradients resident in tensor memory (M = 64 accumulators)
// for the CTA's whole loop and added to the global gradient once.
#include <algorithm>

#include "common.cuh"
#include "mlp.cuh"
#include "tc.cuh"
#include "tc_mlp.cuh"

using namespace angelo;

namespace {

constexpr int kMlpMaxInTiles = 4;   // in_dim <= 64

struct MlpLayout {
    int in_dim, n_hidden, out_dim, k_tiles1;
    // tensor-core operands, bf16 hi then lo, K-major [n][k] (Y = X W^T): W1
    // 64 x 16 k_tiles1, W2 64 x 64 (two hidden layers), W3 16 x 64 (rows
    // out_dim .. 15 zero); fp32 b1, b2, b3 (16) and W3 (16 x 64)
    int64_t off_tw1, off_tw2, off_tw3, off_b1, off_b2, off_b3, off_w3, bytes;
};

bool mlp_layout(int in_dim, int n_hidden, int out_dim, MlpLayout *out) {
    if (in_dim < 1 || in_dim > 16 * kMlpMaxInTiles || (n_hidden != 1 && n_hidden != 2) || out_dim < 1 ||
        out_dim > 16)
        return false;
    MlpLayout L{};
    L.in_dim = in_dim;
    L.n_hidden = n_hidden;
    L.out_dim = out_dim;
    L.k_tiles1 = (in_dim + 15) / 16;
    int64_t o = 0;
    auto take = [&](int64_t b) { const int64_t r = o; o += (b + 15) / 16 * 16; return r; };
    L.off_tw1 = take(2 * 64 * 16 * L.k_tiles1 * 2);
    L.off_tw2 = take(n_hidden == 2 ? 2 * 64 * 64 * 2 : 0);
    L.off_tw3 = take(2 * 16 * 64 * 2);
    L.off_b1 = take(64 * 4);
    L.off_b2 = take(64 * 4);
    L.off_b3 = take(16 * 4);
    L.off_w3 = take(16 * 64 * 4);
    L.bytes = o;
    *out = L;
    return true;
}

// floats of the flat weight gradient: dW1 (64 x 16 k_tiles1), dW2 (64 x 64,
// two hidden layers), dW3 (16 x 64), db1 (64), db2 (64, two hidden layers), db3 (16)
int64_t mlp_grad_floats(const MlpLayout &L) {
    return 64 * 16 * L.k_tiles1 + (L.n_hidden == 2 ? 64 * 64 + 64 : 0) + 16 * 64 + 64 + 16;
}

__global__ void mlp_prep_kernel(const float *W1, const float *b1, const float *W2, const float *b2,
                                const float *W3, const float *b3, MlpLayout L, char *net) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int K1 = 16 * L.k_tiles1;
    const int n1 = 64 * K1, n2 = L.n_hidden == 2 ? 64 * 64 : 0, n3 = 16 * 64;
    int n, k, K;
    float w;
    int64_t off, half;
    if (i < n1) {
        K = K1, n = i / K1, k = i % K1, off = L.off_tw1, half = (int64_t)n1 * 2;
        w = k < L.in_dim ? W1[n * L.in_dim + k] : 0.f;
    } else if ((i -= n1) < n2) {
        K = 64, n = i / 64, k = i % 64, off = L.off_tw2, half = (int64_t)n2 * 2;
        w = W2[n * 64 + k];
    } else if ((i -= n2) < n3) {
        K = 64, n = i / 64, k = i % 64, off = L.off_tw3, half = (int64_t)n3 * 2;
        w = n < L.out_dim ? W3[n * 64 + k] : 0.f;
        reinterpret_cast<float *>(net + L.off_w3)[n * 64 + k] = w;
    } else {
        i -= n3;
        float *fb1 = reinterpret_cast<float *>(net + L.off_b1);
        float *fb2 = reinterpret_cast<float *>(net + L.off_b2);
        float *fb3 = reinterpret_cast<float *>(net + L.off_b3);
        if (i < 64) fb1[i] = b1[i];
        else if (i < 128) fb2[i - 64] = L.n_hidden == 2 ? b2[i - 64] : 0.f;
        else if (i < 144) fb3[i - 128] = i - 128 < L.out_dim ? b3[i - 128] : 0.f;
        return;
    }
    const Split sp = split2(w, 0.0f);
    const uint32_t o = tc::kmajor_offset(n, k, K);
    *reinterpret_cast<uint16_t *>(net + off + o) = (uint16_t)(sp.hi & 0xFFFFu);
    *reinterpret_cast<uint16_t *>(net + off + half + o) = (uint16_t)(sp.lo & 0xFFFFu);
}

int mlp_prep_threads(const MlpLayout &L) {
    return 64 * 16 * L.k_tiles1 + (L.n_hidden == 2 ? 64 * 64 : 0) + 16 * 64 + 144;
}

struct MlpParams {
    MlpLayout L;
    const char *net;
    const float *x;
    int64_t x_stride;
    const int32_t *x_rows;   // row r reads x row x_rows[r] (NULL: row r)
    int64_t S;
    float *out;
    int64_t out_stride;
    const float *g_out;
    int64_t g_stride;
    float *d_x;
    int64_t dx_stride;
    float *d_net;
};

__device__ unsigned int g_mlp_tc_timeouts;   // CTAs that stopped waiting for the tensor cores

template <int KT1, int NH>
struct MlpShape {
    static constexpr int K1 = 16 * KT1;
    // bytes of one (hi or lo) half
    static constexpr uint32_t w1 = 64 * K1 * 2, w2 = NH == 2 ? 64 * 64 * 2 : 0, w3 = 16 * 64 * 2;
    static constexpr uint32_t x = 128 * K1 * 2, h = 128 * 64 * 2, y = 128 * 16 * 2, ones = 128 * 16 * 2;
    static constexpr uint32_t off_w1 = 0, off_w2 = 2 * w1, off_w3 = off_w2 + 2 * w2, off_x = off_w3 + 2 * w3;
    // forward: one activation staging (H1, then H2)
    static constexpr uint32_t f_h = off_x + 2 * x, f_vec = f_h + 2 * h, f_bar = f_vec + 144 * 4,
                              f_bytes = f_bar + 16;
    // forward tensor memory: Z1 [0, 64), Z2 [64, 128); the output in [64, 80)
    // (one hidden layer) or [0, 16) (two)
    static constexpr uint32_t f_out = NH == 2 ? 0 : 64;
    // backward
    static constexpr uint32_t b_h1 = off_x + 2 * x,                  // H1, then dZ1 (two layers)
        b_h2 = b_h1 + 2 * h,                                         // H2 (two layers)
        b_z = b_h2 + (NH == 2 ? 2 * h : 0),                          // dZ of the last hidden layer
        b_y = b_z + 2 * h, b_ones = b_y + 2 * y,
        b_vec = b_ones + ones,                                       // b1, b2, b3 (16), W3 (16 x 64)
        b_db3 = b_vec + (144 + 16 * 64) * 4, b_bar = b_db3 + 16 * 4, b_bytes = b_bar + 32;
    // backward tensor-memory columns: per tile A, B; CTA-resident dW1, dW2,
    // dW3^T, db1, db2 (M = 64 accumulators)
    static constexpr uint32_t tA = 0, tB = 64, tW1 = tB + (K1 > 64 ? K1 : 64), tW2 = tW1 + K1,
                              tW3 = tW2 + (NH == 2 ? 64 : 0), tb1 = tW3 + 16, tb2 = tb1 + 16,
                              used = tb2 + (NH == 2 ? 16 : 0), b_tmem = used <= 256 ? 256 : 512;
};

// Input row s (in_dim columns, zero padded to 16 KT1) as the 16-column blocks
// slice, slice + 4, .. of a K-major staging
template <int KT1>
__device__ __forceinline__ void mlp_stage_x(const MlpParams &P, int64_t s, bool v, int row, int slice, char *xh,
                                            char *xl) {
    for (int b = slice; b < KT1; b += 4) {
        const int c0 = 16 * b;
        float x[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = 0.f;
        if (v) {
            const float *src = P.x + (P.x_rows ? (int64_t)P.x_rows[s] : s) * P.x_stride;
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (c0 + j < P.L.in_dim) x[j] = __ldg(src + c0 + j);
        }
        stage16(xh, xl, row, c0, 16 * KT1, x);
    }
}

template <int KT1, int NH>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_fwd_tc_kernel(const __grid_constant__ MlpParams P) {
    using Sh = MlpShape<KT1, NH>;
    constexpr int K1 = Sh::K1;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane, slice = warp >> 2;
    const MlpLayout &L = P.L;
    auto copy16 = [&](uint32_t dst, int64_t src, uint32_t bytes) {
        for (uint32_t i = tid * 16; i < bytes; i += kTcThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(Sh::off_w1, L.off_tw1, 2 * Sh::w1);
    if (NH == 2) copy16(Sh::off_w2, L.off_tw2, 2 * Sh::w2);
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
    constexpr uint32_t id64 = tc::idesc_bf16_f32(128, 64), id16 = tc::idesc_bf16_f32(128, 16);
    uint32_t phase = 0;
    bool alive = true;
    const int64_t n_tiles = (P.S + 127) / 128;
    if ((int64_t)blockIdx.x < n_tiles)
        mlp_stage_x<KT1>(P, blockIdx.x * 128 + row, blockIdx.x * 128 + row < P.S, row, slice, xh, xl);
    for (int64_t t = blockIdx.x; t < n_tiles && alive; t += gridDim.x) {
        const int64_t s = t * 128 + row;
        const bool v = s < P.S;
        tc_publish();
        if (tid == 0) {
            tc_mma<KT1>(tmem, Xk, W1k, id64, false);
            tc::commit(bar);
        }
        if (!(alive = tc_wait_all(bar, phase))) break;
        phase ^= 1;
        // the input staging is free: the next tile's rows, whose loads overlap
        // this tile's remaining layers
        const int64_t tn = t + gridDim.x;
        if (tn < n_tiles) mlp_stage_x<KT1>(P, tn * 128 + row, tn * 128 + row < P.S, row, slice, xh, xl);
#pragma unroll
        for (int layer = 0; layer < NH; ++layer) {
            float z[16];
            tc::ld16(tmem + lane_off + 64 * layer + 16 * slice, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) z[j] = fmaxf(z[j] + vec[64 * layer + 16 * slice + j], 0.f);
            stage16(hh, hl, row, 16 * slice, 64, z);
            tc_publish();
            if (tid == 0) {
                if (layer + 1 < NH) tc_mma<4>(tmem + 64, Hk, W2k, id64, false);
                else tc_mma<4>(tmem + Sh::f_out, Hk, W3k, id16, false);
                tc::commit(bar);
            }
            if (!(alive = tc_wait_all(bar, phase))) break;
            phase ^= 1;
        }
        if (!alive) break;
        if (slice == 0) {
            float o[16];
            tc::ld16(tmem + lane_off + Sh::f_out, o);
            if (v) {
                float *dst = P.out + s * P.out_stride;
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    if (c < L.out_dim) dst[c] = o[c] + vec[128 + c];
            }
        }
    }
    if (!alive && tid == 0) atomicAdd(&g_mlp_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

template <int KT1, int NH>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_bwd_tc_kernel(const __grid_constant__ MlpParams P) {
    using Sh = MlpShape<KT1, NH>;
    constexpr int K1 = Sh::K1;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane, slice = warp >> 2;
    const MlpLayout &L = P.L;
    auto copy16 = [&](uint32_t dst, int64_t src, uint32_t bytes) {
        for (uint32_t i = tid * 16; i < bytes; i += kTcThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(Sh::off_w1, L.off_tw1, 2 * Sh::w1);
    if (NH == 2) copy16(Sh::off_w2, L.off_tw2, 2 * Sh::w2);
    copy16(Sh::off_w3, L.off_tw3, 2 * Sh::w3);
    float *vec = reinterpret_cast<float *>(smem + Sh::b_vec);   // b1 [64], b2 [64], b3 [16], W3 [16][64]
    for (int i = tid; i < 144 + 16 * 64; i += kTcThreads)
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
        tc::tmem_alloc(slot, Sh::b_tmem);
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
                   sX = tc::smem_addr(xh), sH1 = tc::smem_addr(h1h), sH2 = tc::smem_addr(h2h),
                   sZ = tc::smem_addr(zh), sY = tc::smem_addr(yh), sOnes = tc::smem_addr(ones);
    const TcOp W1k = op_k(sW1, Sh::w1, K1), W1t = op_t(sW1, Sh::w1, K1);
    const TcOp W2k = op_k(sW2, Sh::w2, 64), W2t = op_t(sW2, Sh::w2, 64);
    const TcOp Xk = op_k(sX, Sh::x, K1), Xt = op_t(sX, Sh::x, K1);
    const TcOp H1k = op_k(sH1, Sh::h, 64), H1t = op_t(sH1, Sh::h, 64), H2t = op_t(sH2, Sh::h, 64);
    const TcOp Zk = op_k(sZ, Sh::h, 64), Zt = op_t(sZ, Sh::h, 64), Yt = op_t(sY, Sh::y, 16),
               Ones = op_t(sOnes, 0u, 16);
    // dZ1 lives in the H1 staging with two hidden layers, in the dZ staging with one
    const TcOp D1k = NH == 2 ? H1k : Zk, D1t = NH == 2 ? H1t : Zt, HLt = NH == 2 ? H2t : H1t;
    constexpr uint32_t id64 = tc::idesc_bf16_f32(128, 64);
    constexpr uint32_t id_dh = tc::idesc_bf16_f32(128, 64, 0, 1), id_dx = tc::idesc_bf16_f32(128, K1, 0, 1);
    constexpr uint32_t id_w1 = tc::idesc_bf16_f32(64, K1, 1, 1), id_w2 = tc::idesc_bf16_f32(64, 64, 1, 1),
                       id_16 = tc::idesc_bf16_f32(64, 16, 1, 1);
    const int od = L.out_dim;
    uint32_t ph0 = 0, ph1 = 0;
    bool alive = true;
    const int64_t n_tiles = (P.S + 127) / 128;
    bool first = true;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const int64_t s = t * 128 + row;
        const bool v = s < P.S;
        if (!first) {
            // the previous tile's weight-gradient products read every staging
            if (!(alive = tc_wait_all(&bar[1], ph1))) break;
            ph1 ^= 1;
        }
        first = false;
        mlp_stage_x<KT1>(P, s, v, row, slice, xh, xl);
        tc_publish();
        // forward, recomputed: Z1 (and Z2)
        if (tid == 0) {
            tc_mma<KT1>(tmem + Sh::tA, Xk, W1k, id64, false);
            tc::commit(&bar[0]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        uint32_t m1 = 0, ml = 0;   // ReLU masks of this slice (layer 1, last layer)
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
        ml = m1;
        if (NH == 2) {
            tc_publish();
            if (tid == 0) {
                tc_mma<4>(tmem + Sh::tB, H1k, W2k, id64, false);
                tc::commit(&bar[0]);
            }
            if (!(alive = tc_wait_all(&bar[0], ph0))) break;
            ph0 ^= 1;
            float z[16];
            tc::ld16(tmem + lane_off + Sh::tB + 16 * slice, z);
            ml = 0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                z[j] += vec[64 + 16 * slice + j];
                ml |= (z[j] > 0.f ? 1u : 0u) << j;
                z[j] = fmaxf(z[j], 0.f);
            }
            stage16(h2h, h2l, row, 16 * slice, 64, z);
        }
        // dY (the incoming gradient of the output row), dH of the last hidden
        // layer = dY W3 (rank out_dim), dZ = dH through the ReLU
        {
            float dy[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) dy[c] = 0.f;
            if (v) {
                const float *g = P.g_out + s * P.g_stride;
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    if (c < od) dy[c] = g[c];
            }
            float dz[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int u = 16 * slice + j;
                float dh = 0.f;
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    if (c < od) dh = fmaf(dy[c], w3f[c * 64 + u], dh);
                dz[j] = (ml >> j) & 1u ? dh : 0.f;
            }
            stage16(zh, zl, row, 16 * slice, 64, dz);
            if (slice == 0) {
                stage16(yh, yl, row, 0, 16, dy);
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    if (c >= od) continue;
                    float a = dy[c];
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                    if (lane == 0 && a != 0.f) red_add(db3 + c, a);
                }
            }
        }
        tc_publish();
        if (NH == 2) {
            // dH1 (epilogue), then dW2, db2, dW3
            if (tid == 0) {
                tc_mma<4>(tmem + Sh::tA, Zk, W2t, id_dh, false);
                tc::commit(&bar[0]);
                tc_mma<8>(tmem + Sh::tW2, Zt, H1t, id_w2, true);
                tc_mma<8>(tmem + Sh::tb2, Zt, Ones, id_16, true, true);
                tc_mma<8>(tmem + Sh::tW3, HLt, Yt, id_16, true);
                tc::commit(&bar[1]);
            }
            if (!(alive = tc_wait_all(&bar[0], ph0))) break;
            ph0 ^= 1;
            float dz[16];
            tc::ld16(tmem + lane_off + Sh::tA + 16 * slice, dz);
#pragma unroll
            for (int j = 0; j < 16; ++j) dz[j] = (m1 >> j) & 1u ? dz[j] : 0.f;
            // H1 is read by dW2: rewrite it as dZ1 after the round completed
            if (!(alive = tc_wait_all(&bar[1], ph1))) break;
            ph1 ^= 1;
            stage16(h1h, h1l, row, 16 * slice, 64, dz);
            tc_publish();
        }
        // dX (epilogue), then dW1, db1 (one hidden layer: also dW3)
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tB, D1k, W1t, id_dx, false);
            tc::commit(&bar[0]);
            tc_mma<8>(tmem + Sh::tW1, D1t, Xt, id_w1, true);
            tc_mma<8>(tmem + Sh::tb1, D1t, Ones, id_16, true, true);
            if (NH == 1) tc_mma<8>(tmem + Sh::tW3, HLt, Yt, id_16, true);
            tc::commit(&bar[1]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        if (P.d_x) {
            for (int b = slice; b < KT1; b += 4) {
                float dx[16];
                __syncwarp();
                tc::ld16(tmem + lane_off + Sh::tB + 16 * b, dx);
                if (v) {
                    float *dst = P.d_x + s * P.dx_stride;
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (16 * b + j < L.in_dim) dst[16 * b + j] = dx[j];
                }
            }
        }
    }
    if (alive && !first) alive = tc_wait_all(&bar[1], ph1);
    if (alive) {
        // add the CTA's gradients: tensor-memory rows 16 (warp % 4) + lane
        const int unit = 16 * (warp & 3) + lane;
        float *dW2 = P.d_net + 64 * K1, *dW3 = dW2 + (NH == 2 ? 64 * 64 : 0), *db1 = dW3 + 16 * 64,
              *db2 = db1 + 64, *dB3 = db1 + 64 + (NH == 2 ? 64 : 0);
        for (uint32_t c0 = Sh::tW1 + 16 * slice; c0 < Sh::used; c0 += 64) {
            float w[16];
            __syncwarp();
            tc::ld16(tmem + lane_off + c0, w);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const uint32_t c = c0 + j;
                float *dst = nullptr;
                if (lane >= 16) dst = nullptr;
                else if (c < Sh::tW2) dst = P.d_net + unit * K1 + (c - Sh::tW1);
                else if (c < Sh::tW3) dst = dW2 + unit * 64 + (c - Sh::tW2);
                else if (c < Sh::tb1) dst = (int)(c - Sh::tW3) < L.out_dim ? dW3 + (c - Sh::tW3) * 64 + unit : nullptr;
                else if (c == Sh::tb1) dst = db1 + unit;
                else if (NH == 2 && c == Sh::tb2) dst = db2 + unit;
                if (dst && w[j] != 0.f) atomicAdd(dst, w[j]);
            }
        }
        for (int o = tid; o < 16; o += kTcThreads)
            if (o < L.out_dim && db3[o] != 0.f) atomicAdd(dB3 + o, db3[o]);
    }
    if (!alive && tid == 0) atomicAdd(&g_mlp_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, Sh::b_tmem);
}

template <int KT1, int NH, bool BWD>
int launch_mlp(const MlpParams &P, cudaStream_t st) {
    using Sh = MlpShape<KT1, NH>;
    const size_t smem = BWD ? Sh::b_bytes : Sh::f_bytes;
    auto k = BWD ? mlp_bwd_tc_kernel<KT1, NH> : mlp_fwd_tc_kernel<KT1, NH>;
    static PersistentLaunch cfg;
    const int rc = persistent_setup(k, smem, kTcThreads, cfg, BWD ? "mlp_fused_bwd" : "mlp_fused_fwd");
    if (rc != ANGELO_OK) return rc;
    // tensor memory: a forward CTA holds 128 columns, a backward CTA b_tmem
    const int per_sm = std::min(cfg.per_sm, BWD ? (int)(512 / Sh::b_tmem) : 4);
    const int64_t tiles = (P.S + 127) / 128;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)cfg.sms * per_sm);
    k<<<grid, kTcThreads, smem, st>>>(P);
    return check_launch(BWD ? "mlp_fused_bwd" : "mlp_fused_fwd");
}

template <bool BWD>
int dispatch_mlp(const MlpParams &P, cudaStream_t st) {
    const int key = P.L.k_tiles1 * 4 + P.L.n_hidden;
    switch (key) {
        case 1 * 4 + 1: return launch_mlp<1, 1, BWD>(P, st);
        case 1 * 4 + 2: return launch_mlp<1, 2, BWD>(P, st);
        case 2 * 4 + 1: return launch_mlp<2, 1, BWD>(P, st);
        case 2 * 4 + 2: return launch_mlp<2, 2, BWD>(P, st);
        case 3 * 4 + 1: return launch_mlp<3, 1, BWD>(P, st);
        case 3 * 4 + 2: return launch_mlp<3, 2, BWD>(P, st);
        case 4 * 4 + 1: return launch_mlp<4, 1, BWD>(P, st);
        case 4 * 4 + 2: return launch_mlp<4, 2, BWD>(P, st);
        default:
            set_error("mlp_fused: %d input tiles, %d hidden layers not instantiated", P.L.k_tiles1,
                      P.L.n_hidden);
            return ANGELO_E_UNSUPPORTED;
    }
}

}  // namespace

namespace angelo {
// CTAs of the fused MLP kernels that stopped waiting for the tensor cores
int64_t mlp_tc_timeouts(int reset) {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_mlp_tc_timeouts, sizeof(v)) != cudaSuccess) return -1;
    if (reset) {
        const unsigned int z = 0;
        if (cudaMemcpyToSymbol(g_mlp_tc_timeouts, &z, sizeof(z)) != cudaSuccess) return -1;
    }
    return (int64_t)v;
}
}  // namespace angelo

extern "C" int64_t angelo_mlp_net_bytes(int32_t in_dim, int32_t n_hidden, int32_t out_dim) {
    MlpLayout L;
    return mlp_layout(in_dim, n_hidden, out_dim, &L) ? L.bytes : -1;
}

extern "C" int64_t angelo_mlp_grad_size(int32_t in_dim, int32_t n_hidden, int32_t out_dim) {
    MlpLayout L;
    return mlp_layout(in_dim, n_hidden, out_dim, &L) ? mlp_grad_floats(L) : -1;
}

extern "C" int angelo_mlp_prep(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const float *W1,
                               const float *b1, const float *W2, const float *b2, const float *W3,
                               const float *b3, void *net, void *stream) {
    MlpLayout L;
    ANGELO_REQUIRE(mlp_layout(in_dim, n_hidden, out_dim, &L),
                   "mlp_prep: in_dim %d (1..64), n_hidden %d (1 or 2), out_dim %d (1..16)", in_dim, n_hidden,
                   out_dim);
    ANGELO_REQUIRE(W1 && b1 && W3 && b3 && net && (n_hidden == 1 || (W2 && b2)), "mlp_prep: null pointer");
    mlp_prep_kernel<<<blocks_for(mlp_prep_threads(L), 256), 256, 0, as_stream(stream)>>>(
        W1, b1, W2, b2, W3, b3, L, reinterpret_cast<char *>(net));
    return check_launch("mlp_prep");
}

extern "C" int angelo_mlp_fused_fwd(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const void *net,
                                    const float *x, int64_t x_stride, int64_t n, float *out,
                                    int64_t out_stride, void *stream) {
    MlpLayout L;
    ANGELO_REQUIRE(mlp_layout(in_dim, n_hidden, out_dim, &L), "mlp_fused_fwd: unsupported shape");
    ANGELO_REQUIRE(n >= 0, "mlp_fused_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(net && x && out && x_stride >= in_dim && out_stride >= out_dim, "mlp_fused_fwd: bad argument");
    MlpParams P{};
    P.L = L;
    P.net = reinterpret_cast<const char *>(net);
    P.x = x;
    P.x_stride = x_stride;
    P.S = n;
    P.out = out;
    P.out_stride = out_stride;
    return dispatch_mlp<false>(P, as_stream(stream));
}

extern "C" int angelo_mlp_fused_bwd(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const void *net,
                                    const float *x, int64_t x_stride, const int32_t *x_rows, int64_t n,
                                    const float *g_out,
                                    int64_t g_stride, float *d_x, int64_t dx_stride, float *d_net,
                                    void *stream) {
    MlpLayout L;
    ANGELO_REQUIRE(mlp_layout(in_dim, n_hidden, out_dim, &L), "mlp_fused_bwd: unsupported shape");
    ANGELO_REQUIRE(n >= 0, "mlp_fused_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(net && x && g_out && d_net && x_stride >= in_dim && g_stride >= out_dim &&
                       (!d_x || dx_stride >= in_dim),
                   "mlp_fused_bwd: bad argument");
    MlpParams P{};
    P.L = L;
    P.net = reinterpret_cast<const char *>(net);
    P.x = x;
    P.x_stride = x_stride;
    P.x_rows = x_rows;
    P.S = n;
    P.g_out = g_out;
    P.g_stride = g_stride;
    P.d_x = d_x;
    P.dx_stride = dx_stride;
    P.d_net = d_net;
    return dispatch_mlp<true>(P, as_stream(stream));
}
