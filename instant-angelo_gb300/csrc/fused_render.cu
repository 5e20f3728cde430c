// Fused radiance network and fused compositing.
//
// Radiance (models/texture.py:23-58): per sample the input row
// [feature, SH4((d+1)/2), normalize(grad)] is staged in shared memory, the
// ReLU MLP runs on tensor cores (bf16x3, fp32 accumulation), and the output
// sigmoid (plus sigmoid(feature[1:4]) for the dual-colour network) is applied
// in the epilogue.  The backward recomputes the activations from the same
// inputs (no stash) and returns dL/dfeature, dL/dgrad and dL/dW.
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

using namespace angelo;

namespace {

constexpr int kRW = 8;               // warps per CTA
constexpr int kRT = kRW * 32;
constexpr int kXCols = 96;           // staged input width (6 k-tiles)

struct RadLayout {
    int k_tiles1;   // input k-tiles (ceil(in_dim / 16))
    int in_dim;
    int feat_dim;   // width of the feature input
    int64_t off_w1f, off_w2f, off_w3f, off_w1b, off_w2b, off_w3b, off_b1, off_b2, off_b3, bytes;
};

RadLayout rad_layout(int feat_dim) {
    RadLayout L{};
    L.feat_dim = feat_dim;
    L.in_dim = feat_dim + 16 + 3;
    L.k_tiles1 = (L.in_dim + 15) / 16;
    int64_t o = 0;
    auto take = [&](int64_t b) { const int64_t r = o; o += (b + 15) / 16 * 16; return r; };
    L.off_w1f = take(2 * frag_count(L.k_tiles1, 8) * 8);
    L.off_w2f = take(2 * frag_count(4, 8) * 8);
    L.off_w3f = take(2 * frag_count(4, 1) * 8);
    L.off_w1b = take(2 * frag_count(4, 2 * L.k_tiles1) * 8);
    L.off_w2b = take(2 * frag_count(4, 8) * 8);
    L.off_w3b = take(2 * frag_count(1, 8) * 8);
    L.off_b1 = take(64 * 4);
    L.off_b2 = take(64 * 4);
    L.off_b3 = take(8 * 4);
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
                                const float *W3, const float *b3, RadLayout L, char *net) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = tid & 31, r = lane >> 2, c = (lane & 3) * 2;
    int frag = tid >> 5;
    const int K1 = L.k_tiles1;
    const int counts[6] = {K1 * 8, 32, 4, 4 * 2 * K1, 32, 8};
    int which = 0;
    while (which < 6 && frag >= counts[which]) frag -= counts[which++];
    if (which >= 6) {
        const int j = frag * 32 + lane;
        float *fb1 = reinterpret_cast<float *>(net + L.off_b1);
        float *fb2 = reinterpret_cast<float *>(net + L.off_b2);
        float *fb3 = reinterpret_cast<float *>(net + L.off_b3);
        if (j < 64) fb1[j] = b1[j];
        else if (j < 128) fb2[j - 64] = b2[j - 64];
        else if (j < 136) fb3[j - 128] = j - 128 < 3 ? b3[j - 128] : 0.f;
        return;
    }
    const int layer = which % 3 + 1;
    const bool bwd = which >= 3;
    const int NT = !bwd ? (layer == 3 ? 1 : 8) : (layer == 1 ? 2 * K1 : 8);
    const int KT = !bwd ? (layer == 1 ? K1 : 4) : (layer == 3 ? 1 : 4);
    const int64_t off = !bwd ? (layer == 1 ? L.off_w1f : layer == 2 ? L.off_w2f : L.off_w3f)
                             : (layer == 1 ? L.off_w1b : layer == 2 ? L.off_w2b : L.off_w3b);
    const int kt = frag / NT, nt = frag % NT;
    float v[4];
    for (int i = 0; i < 4; ++i) {
        const int k = kt * 16 + c + (i & 1) + (i >> 1) * 8;
        const int n = nt * 8 + r;
        v[i] = !bwd ? rad_w(layer, n, k, W1, W2, W3, L.in_dim) : rad_w(layer, k, n, W1, W2, W3, L.in_dim);
    }
    const Split s0 = split2(v[0], v[1]), s1 = split2(v[2], v[3]);
    uint2 *dst = reinterpret_cast<uint2 *>(net + off);
    const int64_t n_frag = frag_count(KT, NT);
    const int64_t idx = (int64_t)(kt * NT + nt) * 32 + lane;
    dst[idx] = make_uint2(s0.hi, s1.hi);
    dst[n_frag + idx] = make_uint2(s0.lo, s1.lo);
}

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
    float *rgb;
    const float *g_rgb;
    float *d_feature;
    float *d_grad;
    float *d_net;
};

struct RadWarp {
    float x[16][kXCols];
    float dual_g[16][3];
    float dn[16][3];
};

__device__ __forceinline__ float sigm(float v) { return 1.0f / (1.0f + __expf(-v)); }

// stage the 16 input rows of a tile: [feature, SH, normal, 0...]
__device__ __forceinline__ void stage_rows(const RadParams &P, RadWarp &w, int64_t s0, int lane) {
    const int F = P.L.feat_dim;
    for (int i = lane; i < 16 * kXCols; i += 32) {
        const int row = i / kXCols, col = i % kXCols;
        const int64_t s = s0 + row;
        float v = 0.f;
        if (s < P.S && col < F) v = P.feature[s * P.feat_stride + col];
        w.x[row][col] = v;
    }
    __syncwarp();
    if (lane < 16) {
        const int64_t s = s0 + lane;
        float sh[16], nrm[3] = {0.f, 0.f, 0.f};
        if (s < P.S) {
            const float *d = P.rays_d + (int64_t)P.ray_idx[s] * 3;
            const float x = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[0], 1.f), 2.f), 2.f), 1.f);
            const float y = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[1], 1.f), 2.f), 2.f), 1.f);
            const float z = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn(d[2], 1.f), 2.f), 2.f), 1.f);
            sh4_eval(x, y, z, sh);
            const float *g = P.grad + s * 3;
            const float gn = fmaxf(sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12f);
            for (int k = 0; k < 3; ++k) nrm[k] = g[k] / gn;
        } else {
            for (int k = 0; k < 16; ++k) sh[k] = 0.f;
        }
        for (int k = 0; k < 16; ++k) w.x[lane][F + k] = sh[k];
        for (int k = 0; k < 3; ++k) w.x[lane][F + 16 + k] = nrm[k];
    }
    __syncwarp();
}

template <int KT1>
__device__ __forceinline__ void rows_to_a(const RadWarp &w, int lane, uint32_t (&ah)[KT1][4],
                                          uint32_t (&al)[KT1][4]) {
    const int r = lane >> 2, c = (lane & 3) * 2;
#pragma unroll
    for (int kt = 0; kt < KT1; ++kt)
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int col = kt * 16 + hf * 8 + c;
            const Split a = split2(w.x[r][col], w.x[r][col + 1]);
            const Split b = split2(w.x[r + 8][col], w.x[r + 8][col + 1]);
            ah[kt][hf * 2] = a.hi;
            al[kt][hf * 2] = a.lo;
            ah[kt][hf * 2 + 1] = b.hi;
            al[kt][hf * 2 + 1] = b.lo;
        }
}

struct RadNet {
    const uint2 *w1f, *w2f, *w3f, *w1b, *w2b, *w3b;
    const float *b1, *b2, *b3;
};

__device__ __forceinline__ RadNet rad_net(const char *base, const RadLayout &L) {
    RadNet n;
    n.w1f = reinterpret_cast<const uint2 *>(base + L.off_w1f);
    n.w2f = reinterpret_cast<const uint2 *>(base + L.off_w2f);
    n.w3f = reinterpret_cast<const uint2 *>(base + L.off_w3f);
    n.w1b = reinterpret_cast<const uint2 *>(base + L.off_w1b);
    n.w2b = reinterpret_cast<const uint2 *>(base + L.off_w2b);
    n.w3b = reinterpret_cast<const uint2 *>(base + L.off_w3b);
    n.b1 = reinterpret_cast<const float *>(base + L.off_b1);
    n.b2 = reinterpret_cast<const float *>(base + L.off_b2);
    n.b3 = reinterpret_cast<const float *>(base + L.off_b3);
    return n;
}

template <int KT1>
__global__ void __launch_bounds__(kRT, 1) rad_fwd_kernel(const __grid_constant__ RadParams P) {
    extern __shared__ __align__(16) char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int64_t i = tid * 16; i < P.L.bytes; i += kRT * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(P.net + i);
    RadWarp &w = reinterpret_cast<RadWarp *>(smem + P.L.bytes)[warp];
    __syncthreads();
    const RadNet N = rad_net(smem, P.L);
    const int r = lane >> 2, q = lane & 3;
    const int64_t tiles = (P.S + 15) / 16;
    for (int64_t t = (int64_t)blockIdx.x * kRW + warp; t < tiles; t += (int64_t)gridDim.x * kRW) {
        const int64_t s0 = t * 16;
        stage_rows(P, w, s0, lane);
        uint32_t xh[KT1][4], xl[KT1][4];
        rows_to_a<KT1>(w, lane, xh, xl);
        float Z[8][4];
        uint32_t hh[4][4], hl[4][4];
        hidden_layer<KT1>(xh, xl, N.w1f, N.b1, lane, Z);
        activate_relu(Z, hh, hl);
        hidden_layer<4>(hh, hl, N.w2f, N.b2, lane, Z);
        activate_relu(Z, hh, hl);
        float D[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const int64_t i = (int64_t)kt * 32 + lane;
            mma_x3(D, hh[kt], hl[kt], N.w3f[i], N.w3f[4 * 32 + i]);
        }
        const int c = q * 2;
        if (q < 2) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int64_t s = s0 + r + 8 * rr;
                if (s >= P.S) continue;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int col = c + k;
                    if (col >= 3) continue;
                    float v = sigm(D[2 * rr + k] + N.b3[col]);
                    if (P.dual) v += sigm(P.feature[s * P.feat_stride + 1 + col]);
                    P.rgb[s * 3 + col] = v;
                }
            }
        }
        __syncwarp();
    }
}

template <int KT1>
__global__ void __launch_bounds__(kRT, 1) rad_bwd_kernel(const __grid_constant__ RadParams P) {
    extern __shared__ __align__(16) char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int64_t i = tid * 16; i < P.L.bytes; i += kRT * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(P.net + i);
    const int K1cols = 16 * KT1;
    float *acc = reinterpret_cast<float *>(smem + P.L.bytes);
    const int n1 = 64 * K1cols, n2 = 64 * 64, n3 = 16 * 64;
    const int n_acc = n1 + n2 + n3 + 64 + 64 + 16;
    float *dW1 = acc, *dW2 = acc + n1, *dW3 = acc + n1 + n2;
    float *db1 = acc + n1 + n2 + n3, *db2 = db1 + 64, *db3 = db2 + 64;
    for (int i = tid; i < n_acc; i += kRT) acc[i] = 0.f;
    RadWarp &w = reinterpret_cast<RadWarp *>(acc + ((n_acc + 3) / 4) * 4)[warp];
    __syncthreads();
    const RadNet N = rad_net(smem, P.L);
    const int r = lane >> 2, q = lane & 3, c = q * 2;
    const int F = P.L.feat_dim;
    const int64_t tiles = (P.S + 15) / 16;
    for (int64_t t = (int64_t)blockIdx.x * kRW + warp; t < tiles; t += (int64_t)gridDim.x * kRW) {
        const int64_t s0 = t * 16;
        stage_rows(P, w, s0, lane);
        uint32_t xh[KT1][4], xl[KT1][4];
        rows_to_a<KT1>(w, lane, xh, xl);
        float Z1[8][4], Z2[8][4];
        uint32_t h1h[4][4], h1l[4][4], h2h[4][4], h2l[4][4];
        hidden_layer<KT1>(xh, xl, N.w1f, N.b1, lane, Z1);
        activate_relu(Z1, h1h, h1l);
        hidden_layer<4>(h1h, h1l, N.w2f, N.b2, lane, Z2);
        activate_relu(Z2, h2h, h2l);
        float D[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const int64_t i = (int64_t)kt * 32 + lane;
            mma_x3(D, h2h[kt], h2l[kt], N.w3f[i], N.w3f[4 * 32 + i]);
        }
        // dL/d(out) through the sigmoid; dual colour: dL/dfeature[1..3]
        float dY[1][4] = {{0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int64_t s = s0 + r + 8 * rr;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int col = c + k;
                if (col >= 3 || s >= P.S) continue;
                const float g = P.g_rgb[s * 3 + col];
                const float sg = sigm(D[2 * rr + k] + N.b3[col]);
                dY[0][2 * rr + k] = g * sg * (1.f - sg);
                if (P.dual) {
                    const float sf = sigm(P.feature[s * P.feat_stride + 1 + col]);
                    w.dual_g[r + 8 * rr][col] = g * sf * (1.f - sf);
                }
            }
        }
        uint32_t yh[1][4], yl[1][4];
        {
            const Split a = split2(dY[0][0], dY[0][1]), b = split2(dY[0][2], dY[0][3]);
            yh[0][0] = a.hi;
            yl[0][0] = a.lo;
            yh[0][1] = b.hi;
            yl[0][1] = b.lo;
            yh[0][2] = yh[0][3] = yl[0][2] = yl[0][3] = 0u;
        }
        float dH[8][4];
        mm_nobias<1, 8>(yh, yl, N.w3b, 8, lane, dH);
        accumulate_dw<1, 4>(yh, yl, h2h, h2l, dW3, 64, lane);
        accumulate_db<1>(dY, db3, lane);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) dH[nt][i] = Z2[nt][i] > 0.f ? dH[nt][i] : 0.f;
        uint32_t dzh[4][4], dzl[4][4];
        c_to_a(dH, dzh, dzl);
        accumulate_dw<4, 4>(dzh, dzl, h1h, h1l, dW2, 64, lane);
        accumulate_db<8>(dH, db2, lane);
        mm_nobias<4, 8>(dzh, dzl, N.w2b, 8, lane, dH);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) dH[nt][i] = Z1[nt][i] > 0.f ? dH[nt][i] : 0.f;
        c_to_a(dH, dzh, dzl);
        accumulate_dw<4, KT1>(dzh, dzl, xh, xl, dW1, K1cols, lane);
        accumulate_db<8>(dH, db1, lane);
        float dX[2 * KT1][4];
        mm_nobias<4, 2 * KT1>(dzh, dzl, N.w1b, 2 * KT1, lane, dX);
        __syncwarp();
        // dL/dfeature and dL/dnormal
#pragma unroll
        for (int nt = 0; nt < 2 * KT1; ++nt) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int row = r + 8 * rr;
                const int64_t s = s0 + row;
                if (s >= P.S) continue;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int col = nt * 8 + c + k;
                    const float v = dX[nt][2 * rr + k];
                    if (col < F) {
                        float o = v;
                        if (P.dual && col >= 1 && col <= 3) o += w.dual_g[row][col - 1];
                        P.d_feature[s * P.feat_stride + col] = o;
                    } else if (col >= F + 16 && col < F + 19) {
                        w.dn[row][col - F - 16] = v;
                    }
                }
            }
        }
        __syncwarp();
        if (lane < 16 && s0 + lane < P.S) {
            const int64_t s = s0 + lane;
            const float *g = P.grad + s * 3;
            const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            const float den = fmaxf(gn, 1e-12f);
            float n[3], dn[3];
            for (int k = 0; k < 3; ++k) {
                n[k] = g[k] / den;
                dn[k] = w.dn[lane][k];
            }
            if (gn >= 1e-12f) {
                const float nd = n[0] * dn[0] + n[1] * dn[1] + n[2] * dn[2];
                for (int k = 0; k < 3; ++k) P.d_grad[s * 3 + k] = (dn[k] - n[k] * nd) / gn;
            } else {
                for (int k = 0; k < 3; ++k) P.d_grad[s * 3 + k] = dn[k] / 1e-12f;
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int i = tid; i < n_acc; i += kRT) {
        const float v = acc[i];
        if (v != 0.f) atomicAdd(P.d_net + i, v);
    }
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

}  // namespace

// ------------------------------------------------------------------ host API

extern "C" int64_t angelo_radiance_net_bytes(int32_t feat_dim) {
    if (feat_dim < 1 || feat_dim + 19 > kXCols) return -1;
    return rad_layout(feat_dim).bytes;
}

extern "C" int64_t angelo_radiance_grad_size(int32_t feat_dim) {
    const int kt = (feat_dim + 19 + 15) / 16;
    return 64 * 16 * kt + 64 * 64 + 16 * 64 + 64 + 64 + 16;
}

extern "C" int angelo_radiance_prep(int32_t feat_dim, const float *W1, const float *b1,
                                    const float *W2, const float *b2, const float *W3,
                                    const float *b3, void *net, void *stream) {
    ANGELO_REQUIRE(feat_dim >= 1 && feat_dim + 19 <= kXCols, "radiance_prep: feature width %d",
                   feat_dim);
    ANGELO_REQUIRE(W1 && b1 && W2 && b2 && W3 && b3 && net, "radiance_prep: null pointer");
    const RadLayout L = rad_layout(feat_dim);
    const int frags = L.k_tiles1 * 8 + 32 + 4 + 4 * 2 * L.k_tiles1 + 32 + 8 + 5;
    rad_prep_kernel<<<blocks_for((int64_t)frags * 32, 256), 256, 0, as_stream(stream)>>>(
        W1, b1, W2, b2, W3, b3, L, reinterpret_cast<char *>(net));
    return check_launch("radiance_prep");
}

namespace {
template <int KT1, bool BWD>
int launch_rad(const RadParams &P, cudaStream_t st) {
    const int n_acc = 64 * 16 * KT1 + 64 * 64 + 16 * 64 + 64 + 64 + 16;
    const size_t smem = P.L.bytes + (BWD ? ((n_acc + 3) / 4) * 16 : 0) + kRW * sizeof(RadWarp);
    auto k = BWD ? rad_bwd_kernel<KT1> : rad_fwd_kernel<KT1>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("radiance(smem attribute)");
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kRT, smem);
    if (per_sm < 1) {
        set_error("radiance: %zu bytes of shared memory do not fit an SM", smem);
        return ANGELO_E_UNSUPPORTED;
    }
    const int64_t want = ((P.S + 15) / 16 + kRW - 1) / kRW;
    const int grid = (int)std::min<int64_t>(want, (int64_t)sms * per_sm);
    k<<<grid, kRT, smem, st>>>(P);
    return check_launch(BWD ? "radiance_bwd" : "radiance_fwd");
}

template <bool BWD>
int dispatch_rad(const RadParams &P, cudaStream_t st) {
    switch (P.L.k_tiles1) {
        case 3: return launch_rad<3, BWD>(P, st);
        case 6: return launch_rad<6, BWD>(P, st);
        default:
            set_error("radiance: input width %d not instantiated (feature width 16 or 68)", P.L.in_dim);
            return ANGELO_E_UNSUPPORTED;
    }
}
}  // namespace

extern "C" int angelo_radiance_fwd(int32_t feat_dim, const void *net, const float *feature,
                                   int64_t feat_stride, const float *grad, const int32_t *ray_idx,
                                   const float *rays_d, int64_t n, int32_t dual, float *rgb,
                                   void *stream) {
    ANGELO_REQUIRE(feat_dim >= 1 && feat_dim + 19 <= kXCols, "radiance_fwd: feature width");
    ANGELO_REQUIRE(n >= 0, "radiance_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(net && feature && grad && ray_idx && rays_d && rgb && feat_stride >= feat_dim,
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
    P.dual = dual;
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
    ANGELO_REQUIRE(net && feature && grad && ray_idx && rays_d && g_rgb && d_feature && d_grad &&
                   d_net && feat_stride >= feat_dim, "radiance_bwd: bad argument");
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
