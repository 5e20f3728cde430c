// Fused VolumeSDF (models/geometry.py:195-287 with grad_type finite_difference):
// per sample, 13 evaluations of hash grid + geometry MLP (the point, the 6-tap
// finite-difference stencil, the 6-tap curvature stencil around the
// tangent-shifted point), all in one kernel, with the MLP on tensor cores
// (bf16x3 split, fp32 accumulation) and the stencil arithmetic in fp32.
//
// Work split: a warp owns 16 samples at a time; evaluation e of those 16
// samples is one m16 tile.  Lane (r = lane/4, q = lane%4) encodes rows r and
// r+8 at hash levels q + 4j, which are exactly the A-fragment entries it
// feeds to mma.sync (the encoding input is reordered [hash levels..., xyz,
// zero pad]; the first-layer weights are permuted to match on the host).
//
// Training: the forward kernel stashes the 13 encodings (fp32) and the 13 SDF
// values of each sample; the backward kernel recomputes the MLP activations
// from them, back-propagates through the stencil arithmetic (curvature ->
// shifted stencil -> tangent -> normal -> FD gradient -> FD stencil -> point),
// scatters dL/dtable with vector atomics, and accumulates dL/dW in shared
// memory (one global flush per CTA).
#include <math.h>

#include "common.cuh"
#include "mlp.cuh"

using namespace angelo;

// angelo_sdf_net_layout (include/angelo_gb.h): k_tiles1 = first-layer k-tiles
// (1 + levels/8), n_tiles3 = output n-tiles (width padded to 8), k_tiles3b =
// output width padded to 16 in k-tiles; byte offsets of the forward and
// backward B fragments (hi then lo of each), biases and output row 0.

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

struct NetSmem {
    const uint2 *w1f, *w2f, *w3f;  // hi at [0, n), lo at [n, 2n)
    const float *b1, *b2, *b3;
};

// ------------------------------------------------------------------- prep
// Effective fp32 weights (after weight normalisation) -> bf16 hi/lo B
// fragments.  W1 columns are permuted from the reference order [xyz(3),
// hash(2L)] to the kernel order [hash(2L), xyz(3), 0...].

__device__ __forceinline__ float w1_kernel_col(const float *W1, int in_dim, int n_hash, int n, int k) {
    int src;
    if (k < n_hash) src = 3 + k;
    else if (k < n_hash + 3) src = k - n_hash;
    else return 0.0f;
    return src < in_dim ? W1[n * in_dim + src] : 0.0f;
}

// value of the layer matrix as used by Y = X W^T, kernel ordering, zero padded
__device__ __forceinline__ float layer_w(int layer, int n, int k, const float *W1, const float *W2,
                                         const float *W3, int in_dim, int n_hash, int out_dim) {
    if (layer == 1) return n < 64 ? w1_kernel_col(W1, in_dim, n_hash, n, k) : 0.0f;
    if (layer == 2) return (n < 64 && k < 64) ? W2[n * 64 + k] : 0.0f;
    return (n < out_dim && k < 64) ? W3[n * 64 + k] : 0.0f;
}

__global__ void sdf_prep_kernel(const float *__restrict__ W1, const float *__restrict__ b1,
                                const float *__restrict__ W2, const float *__restrict__ b2,
                                const float *__restrict__ W3, const float *__restrict__ b3,
                                int in_dim, int n_hash, angelo_sdf_net_layout lay,
                                char *__restrict__ net) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = tid & 31;
    const int r = lane >> 2, c = (lane & 3) * 2;
    int frag = tid >> 5;
    // forward fragments: B[k][n] = W[n][k]
    struct Spec {
        int layer, kt, nt;
        int64_t off;
        bool bwd;
    };
    const int K1 = lay.k_tiles1, NT3 = lay.n_tiles3, KT3 = lay.k_tiles3b;
    const int nh = lay.n_hidden;
    // enumerate all fragments: fwd L1 (K1 x 8), fwd L2 (4 x 8), fwd L3 (4 x NT3),
    // bwd L1 (4 x 2*K1), bwd L2 (4 x 8), bwd L3 (KT3 x 8)
    const int counts[6] = {K1 * 8, nh == 2 ? 32 : 0, 4 * NT3, 4 * 2 * K1, nh == 2 ? 32 : 0, KT3 * 8};
    int which = 0;
    while (which < 6 && frag >= counts[which]) frag -= counts[which++];
    if (which >= 6) {
        // biases and the fp32 row 0 of the output layer
        int j = frag * 32 + lane;
        float *fb1 = reinterpret_cast<float *>(net + lay.off_b1);
        float *fb2 = reinterpret_cast<float *>(net + lay.off_b2);
        float *fb3 = reinterpret_cast<float *>(net + lay.off_b3);
        float *fr0 = reinterpret_cast<float *>(net + lay.off_w3row0);
        if (j < 64) fb1[j] = b1[j];
        else if (j < 128) { if (nh == 2) fb2[j - 64] = b2[j - 64]; }
        else if (j < 128 + 8 * NT3) { const int o = j - 128; fb3[o] = o < lay.out_dim ? b3[o] : 0.f; }
        else if (j < 192 + 8 * NT3) { const int o = j - 128 - 8 * NT3; fr0[o] = W3[o]; }
        return;
    }
    const int layer = which % 3 + 1;
    const bool bwd = which >= 3;
    int NT;
    int64_t off;
    if (!bwd) {
        NT = layer == 3 ? NT3 : 8;
        off = layer == 1 ? lay.off_w1f : (layer == 2 ? lay.off_w2f : lay.off_w3f);
    } else {
        NT = layer == 1 ? 2 * K1 : 8;
        off = layer == 1 ? lay.off_w1b : (layer == 2 ? lay.off_w2b : lay.off_w3b);
    }
    const int kt = frag / NT, nt = frag % NT;
    const int KT = !bwd ? (layer == 1 ? K1 : 4) : (layer == 3 ? KT3 : 4);
    float v[4];
    for (int i = 0; i < 4; ++i) {
        const int k = kt * 16 + c + (i & 1) + (i >> 1) * 8;  // reg0: k=c,c+1; reg1: k=c+8,c+9
        const int n = nt * 8 + r;
        // forward: B[k][n] = W[n][k]; backward (dX = dY W): B[k=out][n=in] = W[k][n]
        v[i] = !bwd ? layer_w(layer, n, k, W1, W2, W3, in_dim, n_hash, lay.out_dim)
                    : layer_w(layer, k, n, W1, W2, W3, in_dim, n_hash, lay.out_dim);
    }
    const Split s0 = split2(v[0], v[1]);
    const Split s1 = split2(v[2], v[3]);
    uint2 *dst = reinterpret_cast<uint2 *>(net + off);
    const int64_t n_frag = frag_count(KT, NT);
    const int64_t idx = (int64_t)(kt * NT + nt) * 32 + lane;
    dst[idx] = make_uint2(s0.hi, s1.hi);
    dst[n_frag + idx] = make_uint2(s0.lo, s1.lo);
}

// ----------------------------------------------------------- kernel params

struct SdfParams {
    angelo_hashgrid_layout_t lay;
    int active;
    const float *pos;        // (S,3) world
    const float *rdir;       // (S,3) curvature random directions (may be null)
    int64_t S;
    const void *table;
    int tdtype;
    const char *net;
    angelo_sdf_net_layout nl;
    float radius, eps;
    int with_grad, with_laplace, with_feature;
    // outputs
    float *sdf, *grad, *feature, *laplace;
    int64_t feat_stride;
    // stash (training)
    float *stash_x;   // (S, 13, 36)
    float *stash_s;   // (S, 13)
    // backward inputs
    const float *g_sdf, *g_grad, *g_feature, *g_laplace;
    int64_t gfeat_stride;
    // backward outputs
    float *d_table;   // float32 table gradient (atomic)
    float *d_net;     // (64*K1 + 64*64 + N3*64 + 64 + 64 + N3) fp32, kernel order (atomic)
};

constexpr int kStashCols = 36;

// per-warp scratch: 16 samples
struct WarpScratch {
    float pos[16][3];
    float rd[16][3];
    float s13[16][13];
    float shifted[16][3];
    float ds[16][13];       // backward: dL/d(sdf) of each of the 13 evaluations
    float dshift[16][3];    // backward: dL/d(shifted point)
    float n[16][3];
};

// Position of evaluation e for a sample: e = 0 the point, 1..6 the FD
// stencil (+x,-x,+y,-y,+z,-z) clamped to the box, 7..12 the same stencil
// around the shifted point.  Returns contracted coordinates; mask bit d is
// set when the clamp passed coordinate d through (its gradient is 1).
__device__ __forceinline__ void eval_point(const SdfParams &P, const WarpScratch &ws, int row, int e,
                                           float xc[3], int *mask) {
    const float r = P.radius;
    const float two_r = __fsub_rn(r, -r);
    int m = 0;
    for (int d = 0; d < 3; ++d) {
        float v;
        if (e == 0) {
            v = ws.pos[row][d];
        } else {
            const int k = (e - 1) % 6;
            const float base = e <= 6 ? ws.pos[row][d] : ws.shifted[row][d];
            const float off = (k >> 1) == d ? ((k & 1) ? -P.eps : P.eps) : 0.0f;
            v = __fadd_rn(base, off);
            const bool inside = v >= -r && v <= r;
            v = fminf(fmaxf(v, -r), r);
            m |= inside << d;
        }
        xc[d] = __fdiv_rn(__fsub_rn(v, -r), two_r);
    }
    *mask = e == 0 ? 7 : m;
}

// ------------------------------------------------------------ forward eval
// Encodes rows r, r+8 of evaluation e into A fragments (hi/lo) and runs the
// MLP; returns the output tile(s) in C layout.  KH = hash k-tiles (L/8).

template <int KH>
struct AFrag {
    uint32_t hi[KH + 1][4];
    uint32_t lo[KH + 1][4];
};

template <int KH>
__device__ __forceinline__ void encode_rows(const SdfParams &P, const float xc0[3],
                                            const float xc1[3], int q, AFrag<KH> &A,
                                            float *stash0, float *stash1) {
    // hash levels q + 4j, j < 2*KH; k-tile j/2, upper half when j is odd
#pragma unroll
    for (int j = 0; j < 2 * KH; ++j) {
        const int l = q + 4 * j;
        float f0[2] = {0.f, 0.f}, f1[2] = {0.f, 0.f};
        if (l < P.active) {
            const uint64_t base = P.lay.offsets[l];
            const float s = P.lay.scales[l];
            const LevelPos p0 = level_pos(xc0[0], xc0[1], xc0[2], s);
            const LevelPos p1 = level_pos(xc1[0], xc1[1], xc1[2], s);
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w0 = corner_weight(p0, cc), w1 = corner_weight(p1, cc);
                const float2 v0 = load_entry(P.table, P.tdtype, base + corner_index(P.lay, l, p0, cc));
                const float2 v1 = load_entry(P.table, P.tdtype, base + corner_index(P.lay, l, p1, cc));
                f0[0] = __fmaf_rn(w0, v0.x, f0[0]);
                f0[1] = __fmaf_rn(w0, v0.y, f0[1]);
                f1[0] = __fmaf_rn(w1, v1.x, f1[0]);
                f1[1] = __fmaf_rn(w1, v1.y, f1[1]);
            }
        }
        const Split s0 = split2(f0[0], f0[1]);
        const Split s1 = split2(f1[0], f1[1]);
        const int kt = j >> 1, h = (j & 1) * 2;
        A.hi[kt][h] = s0.hi;
        A.lo[kt][h] = s0.lo;
        A.hi[kt][h + 1] = s1.hi;
        A.lo[kt][h + 1] = s1.lo;
        if (stash0) *reinterpret_cast<float2 *>(stash0 + 2 * l) = make_float2(f0[0], f0[1]);
        if (stash1) *reinterpret_cast<float2 *>(stash1 + 2 * l) = make_float2(f1[0], f1[1]);
    }
    // xyz k-tile: cols 2L + {0,1,2} = x*2-1; q = 0 holds (x, y), q = 1 holds (z, 0)
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
    if (q == 0) {
        a0 = __fsub_rn(__fmul_rn(xc0[0], 2.f), 1.f);
        a1 = __fsub_rn(__fmul_rn(xc0[1], 2.f), 1.f);
        b0 = __fsub_rn(__fmul_rn(xc1[0], 2.f), 1.f);
        b1 = __fsub_rn(__fmul_rn(xc1[1], 2.f), 1.f);
    } else if (q == 1) {
        a0 = __fsub_rn(__fmul_rn(xc0[2], 2.f), 1.f);
        b0 = __fsub_rn(__fmul_rn(xc1[2], 2.f), 1.f);
    }
    const Split s0 = split2(a0, a1), s1 = split2(b0, b1);
    A.hi[KH][0] = s0.hi;
    A.lo[KH][0] = s0.lo;
    A.hi[KH][1] = s1.hi;
    A.lo[KH][1] = s1.lo;
    A.hi[KH][2] = A.hi[KH][3] = A.lo[KH][2] = A.lo[KH][3] = 0u;
    if (q < 2) {
        if (stash0) *reinterpret_cast<float2 *>(stash0 + 16 * KH + 2 * q) = make_float2(a0, a1);
        if (stash1) *reinterpret_cast<float2 *>(stash1 + 16 * KH + 2 * q) = make_float2(b0, b1);
    }
}

// A fragments from stashed fp32 encodings (same positions as encode_rows)
template <int KH>
__device__ __forceinline__ void load_rows(const float *st0, const float *st1, int q, AFrag<KH> &A) {
#pragma unroll
    for (int j = 0; j < 2 * KH; ++j) {
        const int l = q + 4 * j;
        const float2 v0 = st0 ? *reinterpret_cast<const float2 *>(st0 + 2 * l) : make_float2(0.f, 0.f);
        const float2 v1 = st1 ? *reinterpret_cast<const float2 *>(st1 + 2 * l) : make_float2(0.f, 0.f);
        const Split s0 = split2(v0.x, v0.y), s1 = split2(v1.x, v1.y);
        const int kt = j >> 1, h = (j & 1) * 2;
        A.hi[kt][h] = s0.hi;
        A.lo[kt][h] = s0.lo;
        A.hi[kt][h + 1] = s1.hi;
        A.lo[kt][h + 1] = s1.lo;
    }
    float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
    if (q < 2) {
        if (st0) v0 = *reinterpret_cast<const float2 *>(st0 + 16 * KH + 2 * q);
        if (st1) v1 = *reinterpret_cast<const float2 *>(st1 + 16 * KH + 2 * q);
    }
    const Split s0 = split2(v0.x, v0.y), s1 = split2(v1.x, v1.y);
    A.hi[KH][0] = s0.hi;
    A.lo[KH][0] = s0.lo;
    A.hi[KH][1] = s1.hi;
    A.lo[KH][1] = s1.lo;
    A.hi[KH][2] = A.hi[KH][3] = A.lo[KH][2] = A.lo[KH][3] = 0u;
}

// Hidden layer: D (8 n-tiles) = A (KT k-tiles) x W + b, fp32 C layout.
// C layout (8 n-tiles) -> softplus -> split A fragments (4 k-tiles)
// Output layer restricted to the first NTO n-tiles
template <int NTO>
__device__ __forceinline__ void out_layer(const uint32_t (&hh)[4][4], const uint32_t (&hl)[4][4],
                                          const uint2 *wf, int NT3, const float *bias, int lane,
                                          float (&D)[NTO][4]) {
    const int c = (lane & 3) * 2;
    const int64_t n_frag = frag_count(4, NT3);
#pragma unroll
    for (int nt = 0; nt < NTO; ++nt) {
        D[nt][0] = D[nt][1] = D[nt][2] = D[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const int64_t i = (int64_t)(kt * NT3 + nt) * 32 + lane;
            mma_x3(D[nt], hh[kt], hl[kt], wf[i], wf[n_frag + i]);
        }
        const float b0 = bias[nt * 8 + c], b1 = bias[nt * 8 + c + 1];
        D[nt][0] += b0;
        D[nt][1] += b1;
        D[nt][2] += b0;
        D[nt][3] += b1;
    }
}

template <int KH, int NH>
struct Fwd {
    // hidden activations of the last hidden layer (A fragments) after the MLP
    uint32_t hh[4][4], hl[4][4];

    __device__ __forceinline__ void run(const AFrag<KH> &A, const NetSmem &net, int lane) {
        float Z[8][4];
        hidden_layer<KH + 1>(A.hi, A.lo, net.w1f, net.b1, lane, Z);
        activate(Z, hh, hl);
        if (NH == 2) {
            hidden_layer<4>(hh, hl, net.w2f, net.b2, lane, Z);
            activate(Z, hh, hl);
        }
    }
};

// ------------------------------------------------------------ forward kernel

template <int KH, int NH, int NT3>
__global__ void __launch_bounds__(kThreads, 1) sdf_fwd_kernel(const __grid_constant__ SdfParams P) {
    extern __shared__ __align__(16) char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const angelo_sdf_net_layout &nl = P.nl;
    // network fragments -> shared memory (forward set + biases)
    const int64_t fwd_bytes = nl.off_w1b;                   // forward fragments come first
    const int64_t bias_bytes = nl.bytes - nl.off_b1;
    for (int64_t i = tid * 16; i < fwd_bytes; i += kThreads * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(P.net + i);
    for (int64_t i = tid * 4; i < bias_bytes; i += kThreads * 4)
        *reinterpret_cast<float *>(smem + fwd_bytes + i) =
            *reinterpret_cast<const float *>(P.net + nl.off_b1 + i);
    WarpScratch *wsa = reinterpret_cast<WarpScratch *>(smem + fwd_bytes + ((bias_bytes + 15) / 16) * 16);
    WarpScratch &ws = wsa[warp];
    __syncthreads();
    NetSmem net;
    net.w1f = reinterpret_cast<const uint2 *>(smem + nl.off_w1f);
    net.w2f = reinterpret_cast<const uint2 *>(smem + nl.off_w2f);
    net.w3f = reinterpret_cast<const uint2 *>(smem + nl.off_w3f);
    net.b1 = reinterpret_cast<const float *>(smem + fwd_bytes);
    net.b2 = reinterpret_cast<const float *>(smem + fwd_bytes + (nl.off_b2 - nl.off_b1));
    net.b3 = reinterpret_cast<const float *>(smem + fwd_bytes + (nl.off_b3 - nl.off_b1));

    const int r = lane >> 2, q = lane & 3;
    const int64_t n_tiles = (P.S + 15) / 16;
    const int n_evals = P.with_laplace ? 13 : (P.with_grad ? 7 : 1);
    for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < n_tiles; t += (int64_t)gridDim.x * kWarps) {
        const int64_t s0 = t * 16;
        if (lane < 16) {
            const int64_t s = s0 + lane;
            for (int d = 0; d < 3; ++d) {
                ws.pos[lane][d] = s < P.S ? P.pos[s * 3 + d] : 0.f;
                ws.rd[lane][d] = (s < P.S && P.rdir) ? P.rdir[s * 3 + d] : 1.f;
            }
        }
        __syncwarp();
        const bool v0 = s0 + r < P.S, v1 = s0 + r + 8 < P.S;
        for (int e = 0; e < n_evals; ++e) {
            if (e == 7) {
                // tangent-shifted points (models/geometry.py:236-246)
                if (lane < 16) {
                    const float eps = P.eps;
                    float g[3];
                    for (int d = 0; d < 3; ++d)
                        g[d] = __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][1 + 2 * d], ws.s13[lane][2 + 2 * d]), eps);
                    const float gn = fmaxf(sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12f);
                    float nrm[3], rd[3];
                    const float rn = fmaxf(sqrtf(ws.rd[lane][0] * ws.rd[lane][0] + ws.rd[lane][1] * ws.rd[lane][1] +
                                                 ws.rd[lane][2] * ws.rd[lane][2]), 1e-12f);
                    for (int d = 0; d < 3; ++d) {
                        nrm[d] = g[d] / gn;
                        rd[d] = ws.rd[lane][d] / rn;
                        ws.n[lane][d] = nrm[d];
                    }
                    const float tg[3] = {nrm[1] * rd[2] - nrm[2] * rd[1], nrm[2] * rd[0] - nrm[0] * rd[2],
                                         nrm[0] * rd[1] - nrm[1] * rd[0]};
                    const float r_ = P.radius;
                    for (int d = 0; d < 3; ++d) {
                        const float xc = __fdiv_rn(__fsub_rn(ws.pos[lane][d], -r_), __fsub_rn(r_, -r_));
                        ws.shifted[lane][d] = __fadd_rn(xc, __fmul_rn(tg[d], eps));
                    }
                }
                __syncwarp();
            }
            float xc0[3], xc1[3];
            int m0, m1;
            eval_point(P, ws, r, e, xc0, &m0);
            eval_point(P, ws, r + 8, e, xc1, &m1);
            AFrag<KH> A;
            float *st0 = (P.stash_x && v0) ? P.stash_x + ((s0 + r) * 13 + e) * kStashCols : nullptr;
            float *st1 = (P.stash_x && v1) ? P.stash_x + ((s0 + r + 8) * 13 + e) * kStashCols : nullptr;
            encode_rows<KH>(P, xc0, xc1, q, A, st0, st1);
            Fwd<KH, NH> f;
            f.run(A, net, lane);
            if (e == 0 && P.with_feature) {
                float D[NT3][4];
                out_layer<NT3>(f.hh, f.hl, net.w3f, NT3, net.b3, lane, D);
                const int od = nl.out_dim;
#pragma unroll
                for (int nt = 0; nt < NT3; ++nt) {
                    const int col = nt * 8 + q * 2;
                    if (v0) {
                        float *o = P.feature + (s0 + r) * P.feat_stride;
                        if (col < od) o[col] = D[nt][0];
                        if (col + 1 < od) o[col + 1] = D[nt][1];
                    }
                    if (v1) {
                        float *o = P.feature + (s0 + r + 8) * P.feat_stride;
                        if (col < od) o[col] = D[nt][2];
                        if (col + 1 < od) o[col + 1] = D[nt][3];
                    }
                }
                if (q == 0) {
                    ws.s13[r][0] = D[0][0];
                    ws.s13[r + 8][0] = D[0][2];
                    for (int d = 0; d < 3; ++d) {
                        if (v0) P.feature[(s0 + r) * P.feat_stride + od + d] = __fsub_rn(__fmul_rn(xc0[d], 2.f), 1.f);
                        if (v1) P.feature[(s0 + r + 8) * P.feat_stride + od + d] = __fsub_rn(__fmul_rn(xc1[d], 2.f), 1.f);
                    }
                }
            } else {
                float D[1][4];
                out_layer<1>(f.hh, f.hl, net.w3f, NT3, net.b3, lane, D);
                if (q == 0) {
                    ws.s13[r][e] = D[0][0];
                    ws.s13[r + 8][e] = D[0][2];
                }
            }
            __syncwarp();
        }
        // per-sample outputs
        if (lane < 16 && s0 + lane < P.S) {
            const int64_t s = s0 + lane;
            const float eps = P.eps;
            P.sdf[s] = ws.s13[lane][0];
            if (P.with_grad) {
                for (int d = 0; d < 3; ++d)
                    P.grad[s * 3 + d] =
                        __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][1 + 2 * d], ws.s13[lane][2 + 2 * d]), eps);
            }
            if (P.with_laplace) {
                float g[3];
                for (int d = 0; d < 3; ++d)
                    g[d] = __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][7 + 2 * d], ws.s13[lane][8 + 2 * d]), eps);
                const float gn = fmaxf(sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12f);
                float dot = 0.f;
                for (int d = 0; d < 3; ++d) dot += ws.n[lane][d] * (g[d] / gn);
                dot = fminf(fmaxf(dot, -1.0f + 1e-6f), 1.0f - 1e-6f);
                P.laplace[s] = acosf(dot) / 3.14159265358979f;
            }
            if (P.stash_s)
                for (int e = 0; e < 13; ++e) P.stash_s[s * 13 + e] = e < n_evals ? ws.s13[lane][e] : 0.f;
        }
        __syncwarp();
    }
}

// ----------------------------------------------------------- backward eval

struct BwdSmem {
    const uint2 *w1f, *w2f, *w3f, *w1b, *w2b, *w3b;
    const float *b1, *b2, *b3, *w3row0;
    float *dW1, *dW2, *dW3, *db1, *db2, *db3;  // fp32 accumulators, kernel order
    int K1cols, out_pad;                         // 16*k_tiles1, 16*k_tiles3b
};

// C layout -> split A fragments, no activation
// dW[n][k] += sum_m dZ[m][n] X[m][k] for a 16-row tile.  dZ given as split A
// fragments over n (KTN k-tiles), X as split A fragments over k (KTK k-tiles);
// both are transposed 8x8-blockwise with movmatrix.
// db[n] += sum over the 16 rows of a C-layout tile set (8 n-tiles)
// D (NTO n-tiles) = A (4 k-tiles) x Bfrags (KT=4, NT=NT) without bias
// Backward of one evaluation (rows r, r+8 of the tile).  MODE 0: main point
// (full output gradient from dL/dsdf and dL/dfeature), 1: FD stencil point
// (SDF gradient only), 2: shifted stencil point (SDF gradient only, plus the
// positional gradient into ws.dshift).
template <int KH, int NH, int NT3, int MODE>
__device__ __forceinline__ void eval_bwd(const SdfParams &P, const BwdSmem &S, WarpScratch &ws,
                                         int64_t s0, int e, int lane) {
    const int r = lane >> 2, q = lane & 3, c = q * 2;
    const bool v0 = s0 + r < P.S, v1 = s0 + r + 8 < P.S;
    const float *st0 = v0 ? P.stash_x + ((s0 + r) * 13 + e) * kStashCols : nullptr;
    const float *st1 = v1 ? P.stash_x + ((s0 + r + 8) * 13 + e) * kStashCols : nullptr;
    AFrag<KH> X;
    load_rows<KH>(st0, st1, q, X);
    // recompute the activations
    float Z1[8][4];
    hidden_layer<KH + 1>(X.hi, X.lo, S.w1f, S.b1, lane, Z1);
    uint32_t h1h[4][4], h1l[4][4];
    activate(Z1, h1h, h1l);
    float Z2[8][4];
    uint32_t h2h[4][4], h2l[4][4];
    if (NH == 2) {
        hidden_layer<4>(h1h, h1l, S.w2f, S.b2, lane, Z2);
        activate(Z2, h2h, h2l);
    }
    const uint32_t(&hlh)[4][4] = NH == 2 ? h2h : h1h;
    const uint32_t(&hll)[4][4] = NH == 2 ? h2l : h1l;
    float(&Zl)[8][4] = NH == 2 ? Z2 : Z1;
    // dL/dH_last
    float dH[8][4];
    if (MODE == 0) {
        constexpr int KT3 = (NT3 + 1) / 2;
        uint32_t yh[KT3][4], yl[KT3][4];
        const int od = P.nl.out_dim;
        auto gval = [&](int row, int col, bool valid) -> float {
            if (!valid || col >= od) return 0.f;
            float v = P.g_feature ? P.g_feature[(s0 + row) * P.gfeat_stride + col] : 0.f;
            if (col == 0) v += ws.ds[row][0];
            return v;
        };
#pragma unroll
        for (int kt = 0; kt < KT3; ++kt) {
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                const int col = kt * 16 + hf * 8 + c;
                const Split a = split2(gval(r, col, v0), gval(r, col + 1, v0));
                const Split b = split2(gval(r + 8, col, v1), gval(r + 8, col + 1, v1));
                yh[kt][hf * 2] = a.hi;
                yl[kt][hf * 2] = a.lo;
                yh[kt][hf * 2 + 1] = b.hi;
                yl[kt][hf * 2 + 1] = b.lo;
            }
        }
        mm_nobias<KT3, 8>(yh, yl, S.w3b, 8, lane, dH);
        accumulate_dw<KT3, 4>(yh, yl, hlh, hll, S.dW3, 64, lane);
        // db3 from the fp32 values
        float Y[2 * KT3][4];
#pragma unroll
        for (int nt = 0; nt < 2 * KT3; ++nt) {
            const int col = nt * 8 + c;
            Y[nt][0] = gval(r, col, v0);
            Y[nt][1] = gval(r, col + 1, v0);
            Y[nt][2] = gval(r + 8, col, v1);
            Y[nt][3] = gval(r + 8, col + 1, v1);
        }
        accumulate_db<2 * KT3>(Y, S.db3, lane);
    } else {
        const float dy0 = v0 ? ws.ds[r][e] : 0.f, dy1 = v1 ? ws.ds[r + 8][e] : 0.f;
        float part[8][2];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = nt * 8 + c;
            const float w0 = S.w3row0[col], w1 = S.w3row0[col + 1];
            dH[nt][0] = dy0 * w0;
            dH[nt][1] = dy0 * w1;
            dH[nt][2] = dy1 * w0;
            dH[nt][3] = dy1 * w1;
            part[nt][0] = dy0 * softplus100(Zl[nt][0]) + dy1 * softplus100(Zl[nt][2]);
            part[nt][1] = dy0 * softplus100(Zl[nt][1]) + dy1 * softplus100(Zl[nt][3]);
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                part[nt][0] += __shfl_xor_sync(0xffffffffu, part[nt][0], o);
                part[nt][1] += __shfl_xor_sync(0xffffffffu, part[nt][1], o);
            }
        }
        float sdy = dy0 + dy1;
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) sdy += __shfl_xor_sync(0xffffffffu, sdy, o);
        if (lane < 4) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                red_add(S.dW3 + nt * 8 + lane * 2, part[nt][0]);
                red_add(S.dW3 + nt * 8 + lane * 2 + 1, part[nt][1]);
            }
        }
        if (lane == 0) red_add(S.db3, sdy);
    }
    // through the last hidden activation
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) dH[nt][i] *= softplus100_grad(Zl[nt][i]);
    uint32_t dzh[4][4], dzl[4][4];
    c_to_a(dH, dzh, dzl);
    if (NH == 2) {
        accumulate_dw<4, 4>(dzh, dzl, h1h, h1l, S.dW2, 64, lane);
        accumulate_db<8>(dH, S.db2, lane);
        mm_nobias<4, 8>(dzh, dzl, S.w2b, 8, lane, dH);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) dH[nt][i] *= softplus100_grad(Z1[nt][i]);
        c_to_a(dH, dzh, dzl);
    }
    accumulate_dw<4, KH + 1>(dzh, dzl, X.hi, X.lo, S.dW1, S.K1cols, lane);
    accumulate_db<8>(dH, S.db1, lane);
    // dL/dX: hash columns (n-tiles 0 .. 2KH-1) and, for MODE 2, the xyz tile
    constexpr int NTX = 2 * KH + (MODE == 2 ? 1 : 0);
    float dX[NTX][4];
    mm_nobias<4, NTX>(dzh, dzl, S.w1b, 2 * (KH + 1), lane, dX);
    float xc0[3], xc1[3];
    int m0, m1;
    eval_point(P, ws, r, e, xc0, &m0);
    eval_point(P, ws, r + 8, e, xc1, &m1);
    float dxc0[3] = {0.f, 0.f, 0.f}, dxc1[3] = {0.f, 0.f, 0.f};
    float2 *dt = reinterpret_cast<float2 *>(P.d_table);
#pragma unroll
    for (int j = 0; j < 2 * KH; ++j) {
        const int l = q + 4 * j;
        const bool lvl_on = l < P.active;
        const uint64_t base = P.lay.offsets[l];
        const float sc = P.lay.scales[l];
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const bool valid = (rr ? v1 : v0) && lvl_on;
            const float g0 = dX[j][2 * rr], g1 = dX[j][2 * rr + 1];
            const bool live = valid && (g0 != 0.f || g1 != 0.f);
            const float *xc = rr ? xc1 : xc0;
            const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
            float dl[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w = corner_weight(p, cc);
                const uint64_t ent = live ? base + corner_index(P.lay, l, p, cc) : 0;
                // levels 0..7 (j < 2) are coarse: the 16 rows of the tile are
                // consecutive samples and mostly share corners, so aggregate
                // over the 8 lanes of a level group (lane stride 4) first
                if (dt) {
                    if (j < 2) aggregated_add2<4>(dt, ent, w * g0, w * g1, live);
                    else if (live) atomicAdd(dt + ent, make_float2(w * g0, w * g1));
                }
                if (MODE == 2 && live) {
                    const float2 v = load_entry(P.table, P.tdtype, ent);
                    const float gv = g0 * v.x + g1 * v.y;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        float wd = 1.f;
#pragma unroll
                        for (int k = 0; k < 3; ++k)
                            if (k != d) wd *= (cc >> k) & 1 ? p.f[k] : 1.f - p.f[k];
                        dl[d] += ((cc >> d) & 1 ? wd : -wd) * gv;
                    }
                }
            }
            if (MODE == 2) {
                float *dxc = rr ? dxc1 : dxc0;
#pragma unroll
                for (int d = 0; d < 3; ++d) dxc[d] += sc * dl[d];
            }
        }
    }
    if (MODE == 2) {
        // xyz columns: q = 0 holds (x, y), q = 1 holds z, of d(x*2-1)
        if (q == 0) {
            dxc0[0] += 2.f * dX[2 * KH][0];
            dxc0[1] += 2.f * dX[2 * KH][1];
            dxc1[0] += 2.f * dX[2 * KH][2];
            dxc1[1] += 2.f * dX[2 * KH][3];
        } else if (q == 1) {
            dxc0[2] += 2.f * dX[2 * KH][0];
            dxc1[2] += 2.f * dX[2 * KH][2];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
#pragma unroll
            for (int o = 1; o < 4; o <<= 1) {
                dxc0[d] += __shfl_xor_sync(0xffffffffu, dxc0[d], o);
                dxc1[d] += __shfl_xor_sync(0xffffffffu, dxc1[d], o);
            }
        }
        if (q == 0) {
            const float inv = 1.0f / __fsub_rn(P.radius, -P.radius);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if ((m0 >> d) & 1) ws.dshift[r][d] += dxc0[d] * inv;
                if ((m1 >> d) & 1) ws.dshift[r + 8][d] += dxc1[d] * inv;
            }
        }
    }
}

template <int KH, int NH, int NT3>
__global__ void __launch_bounds__(kThreads, 1) sdf_bwd_kernel(const __grid_constant__ SdfParams P) {
    extern __shared__ __align__(16) char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const angelo_sdf_net_layout &nl = P.nl;
    const int64_t net_bytes = nl.bytes;
    for (int64_t i = tid * 16; i < net_bytes; i += kThreads * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(P.net + i);
    BwdSmem S;
    S.w1f = reinterpret_cast<const uint2 *>(smem + nl.off_w1f);
    S.w2f = reinterpret_cast<const uint2 *>(smem + nl.off_w2f);
    S.w3f = reinterpret_cast<const uint2 *>(smem + nl.off_w3f);
    S.w1b = reinterpret_cast<const uint2 *>(smem + nl.off_w1b);
    S.w2b = reinterpret_cast<const uint2 *>(smem + nl.off_w2b);
    S.w3b = reinterpret_cast<const uint2 *>(smem + nl.off_w3b);
    S.b1 = reinterpret_cast<const float *>(smem + nl.off_b1);
    S.b2 = reinterpret_cast<const float *>(smem + nl.off_b2);
    S.b3 = reinterpret_cast<const float *>(smem + nl.off_b3);
    S.w3row0 = reinterpret_cast<const float *>(smem + nl.off_w3row0);
    S.K1cols = 16 * nl.k_tiles1;
    S.out_pad = 16 * nl.k_tiles3b;
    float *acc = reinterpret_cast<float *>(smem + net_bytes);
    const int n1 = 64 * S.K1cols, n2 = 64 * 64, n3 = S.out_pad * 64;
    const int n_acc = n1 + n2 + n3 + 64 + 64 + S.out_pad;
    S.dW1 = acc;
    S.dW2 = acc + n1;
    S.dW3 = acc + n1 + n2;
    S.db1 = acc + n1 + n2 + n3;
    S.db2 = S.db1 + 64;
    S.db3 = S.db2 + 64;
    for (int i = tid; i < n_acc; i += kThreads) acc[i] = 0.f;
    WarpScratch *wsa = reinterpret_cast<WarpScratch *>(acc + ((n_acc + 3) / 4) * 4);
    WarpScratch &ws = wsa[warp];
    __syncthreads();

    const int64_t n_tiles = (P.S + 15) / 16;
    const float eps = P.eps;
    for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < n_tiles; t += (int64_t)gridDim.x * kWarps) {
        const int64_t s0 = t * 16;
        if (lane < 16) {
            const int64_t s = s0 + lane;
            const bool v = s < P.S;
            for (int d = 0; d < 3; ++d) {
                ws.pos[lane][d] = v ? P.pos[s * 3 + d] : 0.f;
                ws.rd[lane][d] = (v && P.rdir) ? P.rdir[s * 3 + d] : 1.f;
                ws.dshift[lane][d] = 0.f;
            }
            for (int e = 0; e < 13; ++e) {
                ws.s13[lane][e] = v ? P.stash_s[s * 13 + e] : 0.f;
                ws.ds[lane][e] = 0.f;
            }
            // forward quantities of the stencil arithmetic
            float g[3], n[3];
            for (int d = 0; d < 3; ++d)
                g[d] = __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][1 + 2 * d], ws.s13[lane][2 + 2 * d]), eps);
            const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            for (int d = 0; d < 3; ++d) n[d] = g[d] / fmaxf(gn, 1e-12f);
            if (P.with_laplace && v) {
                float rd[3];
                const float rn = fmaxf(sqrtf(ws.rd[lane][0] * ws.rd[lane][0] + ws.rd[lane][1] * ws.rd[lane][1] +
                                             ws.rd[lane][2] * ws.rd[lane][2]), 1e-12f);
                for (int d = 0; d < 3; ++d) rd[d] = ws.rd[lane][d] / rn;
                const float tg[3] = {n[1] * rd[2] - n[2] * rd[1], n[2] * rd[0] - n[0] * rd[2],
                                     n[0] * rd[1] - n[1] * rd[0]};
                const float r_ = P.radius;
                for (int d = 0; d < 3; ++d) {
                    const float xc = __fdiv_rn(__fsub_rn(ws.pos[lane][d], -r_), __fsub_rn(r_, -r_));
                    ws.shifted[lane][d] = __fadd_rn(xc, __fmul_rn(tg[d], eps));
                }
                float gs[3], ns[3];
                for (int d = 0; d < 3; ++d)
                    gs[d] = __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][7 + 2 * d], ws.s13[lane][8 + 2 * d]), eps);
                const float gsn = sqrtf(gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2]);
                for (int d = 0; d < 3; ++d) ns[d] = gs[d] / fmaxf(gsn, 1e-12f);
                const float dot = n[0] * ns[0] + n[1] * ns[1] + n[2] * ns[2];
                const float lo = -1.0f + 1e-6f, hi = 1.0f - 1e-6f;
                const float dotc = fminf(fmaxf(dot, lo), hi);
                const float dang = P.g_laplace ? P.g_laplace[s] / 3.14159265358979f : 0.f;
                const float ddot = (dot >= lo && dot <= hi) ? -dang / sqrtf(1.0f - dotc * dotc) : 0.f;
                float dns[3], dgs[3];
                for (int d = 0; d < 3; ++d) {
                    ws.n[lane][d] = ddot * ns[d];  // dL/dn from the curvature, completed later
                    dns[d] = ddot * n[d];
                }
                normalize_bwd(gs, gsn, ns, dns, dgs);
                for (int d = 0; d < 3; ++d) {
                    const float h = __fdiv_rn(0.5f * dgs[d], eps);
                    ws.ds[lane][7 + 2 * d] = h;
                    ws.ds[lane][8 + 2 * d] = -h;
                }
            } else {
                for (int d = 0; d < 3; ++d) ws.n[lane][d] = 0.f;
            }
            ws.ds[lane][0] = (v && P.g_sdf) ? P.g_sdf[s] : 0.f;
        }
        __syncwarp();
        if (P.with_laplace)
            for (int e = 7; e < 13; ++e) eval_bwd<KH, NH, NT3, 2>(P, S, ws, s0, e, lane);
        __syncwarp();
        if (lane < 16 && P.with_grad) {
            const int64_t s = s0 + lane;
            const bool v = s < P.S;
            float g[3], n[3], dn[3], dg[3];
            for (int d = 0; d < 3; ++d)
                g[d] = __fdiv_rn(0.5f * __fsub_rn(ws.s13[lane][1 + 2 * d], ws.s13[lane][2 + 2 * d]), eps);
            const float gn = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            for (int d = 0; d < 3; ++d) {
                n[d] = g[d] / fmaxf(gn, 1e-12f);
                dn[d] = ws.n[lane][d];
            }
            if (P.with_laplace && v) {
                float rd[3], dtg[3];
                const float rn = fmaxf(sqrtf(ws.rd[lane][0] * ws.rd[lane][0] + ws.rd[lane][1] * ws.rd[lane][1] +
                                             ws.rd[lane][2] * ws.rd[lane][2]), 1e-12f);
                for (int d = 0; d < 3; ++d) {
                    rd[d] = ws.rd[lane][d] / rn;
                    dtg[d] = ws.dshift[lane][d] * eps;
                }
                // t = n x rd  ->  dL/dn += rd x dL/dt
                dn[0] += rd[1] * dtg[2] - rd[2] * dtg[1];
                dn[1] += rd[2] * dtg[0] - rd[0] * dtg[2];
                dn[2] += rd[0] * dtg[1] - rd[1] * dtg[0];
            }
            normalize_bwd(g, gn, n, dn, dg);
            for (int d = 0; d < 3; ++d) {
                const float gin = (v && P.g_grad) ? P.g_grad[s * 3 + d] : 0.f;
                const float h = __fdiv_rn(0.5f * (dg[d] + gin), eps);
                ws.ds[lane][1 + 2 * d] = v ? h : 0.f;
                ws.ds[lane][2 + 2 * d] = v ? -h : 0.f;
            }
        }
        __syncwarp();
        if (P.with_grad)
            for (int e = 1; e < 7; ++e) eval_bwd<KH, NH, NT3, 1>(P, S, ws, s0, e, lane);
        eval_bwd<KH, NH, NT3, 0>(P, S, ws, s0, 0, lane);
        __syncwarp();
    }
    __syncthreads();
    for (int i = tid; i < n_acc; i += kThreads) {
        const float v = acc[i];
        if (v != 0.f) atomicAdd(P.d_net + i, v);
    }
}

}  // namespace

// ------------------------------------------------------------------ host API

extern "C" int angelo_sdf_net_layout_query(int32_t n_levels, int32_t n_hidden, int32_t out_dim,
                                           angelo_sdf_net_layout *out) {
    ANGELO_REQUIRE(out != nullptr, "sdf_net_layout: null output");
    ANGELO_REQUIRE(n_levels == 8 || n_levels == 16, "sdf_net_layout: %d levels (8 or 16 supported)",
                   n_levels);
    ANGELO_REQUIRE(n_hidden == 1 || n_hidden == 2, "sdf_net_layout: %d hidden layers", n_hidden);
    ANGELO_REQUIRE(out_dim >= 1 && out_dim <= 72, "sdf_net_layout: feature_dim %d > 72", out_dim);
    angelo_sdf_net_layout L{};
    L.k_tiles1 = 1 + 2 * n_levels / 16;
    L.n_hidden = n_hidden;
    L.n_tiles3 = (out_dim + 7) / 8;
    L.k_tiles3b = (out_dim + 15) / 16;
    L.out_dim = out_dim;
    int64_t o = 0;
    auto take = [&](int64_t bytes) { const int64_t r = o; o += (bytes + 15) / 16 * 16; return r; };
    L.off_w1f = take(2 * frag_count(L.k_tiles1, 8) * 8);
    L.off_w2f = take(n_hidden == 2 ? 2 * frag_count(4, 8) * 8 : 0);
    L.off_w3f = take(2 * frag_count(4, L.n_tiles3) * 8);
    L.off_w1b = take(2 * frag_count(4, 2 * L.k_tiles1) * 8);
    L.off_w2b = take(n_hidden == 2 ? 2 * frag_count(4, 8) * 8 : 0);
    L.off_w3b = take(2 * frag_count(L.k_tiles3b, 8) * 8);
    L.off_b1 = take(64 * 4);
    L.off_b2 = take(64 * 4);
    L.off_b3 = take(8 * L.n_tiles3 * 4);
    L.off_w3row0 = take(64 * 4);
    L.bytes = o;
    *out = L;
    return ANGELO_OK;
}

extern "C" int angelo_sdf_prep(const angelo_sdf_net_layout *lay, int32_t n_levels, int32_t in_dim,
                               const float *W1, const float *b1, const float *W2, const float *b2,
                               const float *W3, const float *b3, void *net, void *stream) {
    ANGELO_REQUIRE(lay && W1 && b1 && W3 && b3 && net, "sdf_prep: null pointer");
    ANGELO_REQUIRE(lay->n_hidden == 1 || (W2 && b2), "sdf_prep: missing hidden layer 2");
    ANGELO_REQUIRE(in_dim == 3 + 2 * n_levels, "sdf_prep: in_dim %d != 3 + 2*levels", in_dim);
    const int K1 = lay->k_tiles1, nh = lay->n_hidden;
    const int frags = K1 * 8 + (nh == 2 ? 32 : 0) + 4 * lay->n_tiles3 + 4 * 2 * K1 +
                      (nh == 2 ? 32 : 0) + lay->k_tiles3b * 8;
    const int extra = (192 + 8 * lay->n_tiles3 + 31) / 32;
    const int threads = (frags + extra) * 32;
    sdf_prep_kernel<<<blocks_for(threads, 256), 256, 0, as_stream(stream)>>>(
        W1, b1, W2, b2, W3, b3, in_dim, 2 * n_levels, *lay, reinterpret_cast<char *>(net));
    return check_launch("sdf_prep");
}

namespace {
template <int KH, int NH, int NT3>
int launch_fwd(const SdfParams &P, cudaStream_t s) {
    const int64_t fwd_bytes = P.nl.off_w1b;
    const int64_t bias_bytes = ((P.nl.bytes - P.nl.off_b1 + 15) / 16) * 16;
    const size_t smem = fwd_bytes + bias_bytes + kWarps * sizeof(WarpScratch);
    auto k = sdf_fwd_kernel<KH, NH, NT3>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("sdf_fwd(smem attribute)");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem);
    const int64_t tiles = (P.S + 15) / 16;
    const int64_t want = (tiles + kWarps - 1) / kWarps;
    const int grid = (int)std::min<int64_t>(want, (int64_t)sms * std::max(per_sm, 1));
    k<<<grid, kThreads, smem, s>>>(P);
    return check_launch("sdf_fwd");
}

template <int KH, int NH>
int dispatch_nt3(const SdfParams &P, cudaStream_t s) {
    switch (P.nl.n_tiles3) {
        case 2: return launch_fwd<KH, NH, 2>(P, s);
        case 9: return launch_fwd<KH, NH, 9>(P, s);
        default:
            set_error("sdf_fwd: output width %d not instantiated (13 or 65 supported)", P.nl.out_dim);
            return ANGELO_E_UNSUPPORTED;
    }
}
}  // namespace

extern "C" int angelo_sdf_stencil_fwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                      const void *table, int32_t table_dtype,
                                      const angelo_sdf_net_layout *nl, const void *net,
                                      const float *pos, const float *rand_dirs, int64_t n,
                                      float radius, float eps, int32_t with_grad,
                                      int32_t with_laplace, int32_t with_feature, float *sdf,
                                      float *grad, float *feature, int64_t feat_stride,
                                      float *laplace, float *stash_x, float *stash_s, void *stream) {
    ANGELO_REQUIRE(lay && nl && net && table, "sdf_stencil_fwd: null argument");
    ANGELO_REQUIRE(n >= 0, "sdf_stencil_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(lay->n_levels == 8 * (nl->k_tiles1 - 1), "sdf_stencil_fwd: levels vs net");
    ANGELO_REQUIRE(active_levels >= 0 && active_levels <= lay->n_levels, "sdf_stencil_fwd: active");
    ANGELO_REQUIRE(pos && sdf, "sdf_stencil_fwd: null pos/sdf");
    ANGELO_REQUIRE(!with_laplace || with_grad, "sdf_stencil_fwd: laplace needs the gradient");
    ANGELO_REQUIRE(!with_grad || grad, "sdf_stencil_fwd: null grad");
    ANGELO_REQUIRE(!with_laplace || (laplace && rand_dirs), "sdf_stencil_fwd: null laplace/rand");
    ANGELO_REQUIRE(!with_feature || (feature && feat_stride >= nl->out_dim + 3),
                   "sdf_stencil_fwd: bad feature output");
    ANGELO_REQUIRE((stash_x == nullptr) == (stash_s == nullptr), "sdf_stencil_fwd: stash pair");
    ANGELO_REQUIRE(eps > 0.f && radius > 0.f, "sdf_stencil_fwd: eps/radius");
    SdfParams P{};
    P.lay = *lay;
    P.active = active_levels;
    P.pos = pos;
    P.rdir = rand_dirs;
    P.S = n;
    P.table = table;
    P.tdtype = table_dtype;
    P.net = reinterpret_cast<const char *>(net);
    P.nl = *nl;
    P.radius = radius;
    P.eps = eps;
    P.with_grad = with_grad;
    P.with_laplace = with_laplace;
    P.with_feature = with_feature;
    P.sdf = sdf;
    P.grad = grad;
    P.feature = feature;
    P.feat_stride = feat_stride;
    P.laplace = laplace;
    P.stash_x = stash_x;
    P.stash_s = stash_s;
    cudaStream_t s = as_stream(stream);
    if (nl->k_tiles1 == 3) {
        return nl->n_hidden == 2 ? dispatch_nt3<2, 2>(P, s) : dispatch_nt3<2, 1>(P, s);
    }
    return nl->n_hidden == 2 ? dispatch_nt3<1, 2>(P, s) : dispatch_nt3<1, 1>(P, s);
}

namespace {
template <int KH, int NH, int NT3>
int launch_bwd(const SdfParams &P, cudaStream_t s) {
    const int k1cols = 16 * P.nl.k_tiles1, outp = 16 * P.nl.k_tiles3b;
    const int n_acc = 64 * k1cols + 64 * 64 + outp * 64 + 64 + 64 + outp;
    const size_t smem = P.nl.bytes + ((n_acc + 3) / 4) * 16 + kWarps * sizeof(WarpScratch);
    auto k = sdf_bwd_kernel<KH, NH, NT3>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("sdf_bwd(smem attribute)");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem);
    if (per_sm < 1) {
        set_error("sdf_bwd: %zu bytes of shared memory do not fit an SM", smem);
        return ANGELO_E_UNSUPPORTED;
    }
    const int64_t tiles = (P.S + 15) / 16;
    const int64_t want = (tiles + kWarps - 1) / kWarps;
    const int grid = (int)std::min<int64_t>(want, (int64_t)sms * per_sm);
    k<<<grid, kThreads, smem, s>>>(P);
    return check_launch("sdf_bwd");
}

template <int KH, int NH>
int dispatch_bwd(const SdfParams &P, cudaStream_t s) {
    switch (P.nl.n_tiles3) {
        case 2: return launch_bwd<KH, NH, 2>(P, s);
        case 9: return launch_bwd<KH, NH, 9>(P, s);
        default:
            set_error("sdf_bwd: output width %d not instantiated (13 or 65 supported)", P.nl.out_dim);
            return ANGELO_E_UNSUPPORTED;
    }
}
}  // namespace

extern "C" int64_t angelo_sdf_grad_size(const angelo_sdf_net_layout *nl) {
    const int k1cols = 16 * nl->k_tiles1, outp = 16 * nl->k_tiles3b;
    return 64 * k1cols + 64 * 64 + outp * 64 + 64 + 64 + outp;
}

extern "C" int angelo_sdf_stencil_bwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                      const void *table, int32_t table_dtype,
                                      const angelo_sdf_net_layout *nl, const void *net,
                                      const float *pos, const float *rand_dirs, int64_t n,
                                      float radius, float eps, int32_t with_grad,
                                      int32_t with_laplace, const float *stash_x,
                                      const float *stash_s, const float *g_sdf,
                                      const float *g_grad, const float *g_feature,
                                      int64_t gfeat_stride, const float *g_laplace,
                                      float *d_table, float *d_net, void *stream) {
    ANGELO_REQUIRE(lay && nl && net && table && pos && stash_x && stash_s && d_net,
                   "sdf_stencil_bwd: null argument");
    ANGELO_REQUIRE(n >= 0, "sdf_stencil_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(lay->n_levels == 8 * (nl->k_tiles1 - 1), "sdf_stencil_bwd: levels vs net");
    ANGELO_REQUIRE(!with_laplace || (with_grad && rand_dirs), "sdf_stencil_bwd: laplace inputs");
    ANGELO_REQUIRE(g_feature == nullptr || gfeat_stride >= nl->out_dim, "sdf_stencil_bwd: stride");
    SdfParams P{};
    P.lay = *lay;
    P.active = active_levels;
    P.pos = pos;
    P.rdir = rand_dirs;
    P.S = n;
    P.table = table;
    P.tdtype = table_dtype;
    P.net = reinterpret_cast<const char *>(net);
    P.nl = *nl;
    P.radius = radius;
    P.eps = eps;
    P.with_grad = with_grad;
    P.with_laplace = with_laplace;
    P.stash_x = const_cast<float *>(stash_x);
    P.stash_s = const_cast<float *>(stash_s);
    P.g_sdf = g_sdf;
    P.g_grad = g_grad;
    P.g_feature = g_feature;
    P.gfeat_stride = gfeat_stride;
    P.g_laplace = g_laplace;
    P.d_table = d_table;
    P.d_net = d_net;
    cudaStream_t s = as_stream(stream);
    if (nl->k_tiles1 == 3) return nl->n_hidden == 2 ? dispatch_bwd<2, 2>(P, s) : dispatch_bwd<2, 1>(P, s);
    return nl->n_hidden == 2 ? dispatch_bwd<1, 2>(P, s) : dispatch_bwd<1, 1>(P, s);
}
