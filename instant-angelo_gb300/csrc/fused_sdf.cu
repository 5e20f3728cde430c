// Fused VolumeSDF (models/geometry.py:195-287 with grad_type finite_difference):
// per sample 13 evaluations of hash grid + geometry MLP -- the point, the
// 6-tap finite-difference stencil around it and the 6-tap curvature stencil
// around the tangent-shifted point -- in four kinds of kernels:
//
//   stencil_encode   thread per (sample, level).  The taps of one level share
//                    the 8 corner gathers of the stencil centre: a tap moved by
//                    eps along axis d keeps the corners of the centre's cell,
//                    or, when it crosses a cell face, the 4 corners of the face
//                    it shares and 4 new ones.  Each tap's features are
//                    computed exactly as encoding that tap alone (same cell,
//                    fraction, weights and summation order).  Output: the
//                    encodings X[e][l][s] (float2, level-major).
//   sdf_mlp_fwd      warp per 16 samples: the geometry MLP of every evaluation
//                    on tensor cores (bf16x3 split, fp32 accumulation) from X,
//                    then the stencil arithmetic (sdf, FD gradient, tangent
//                    shift, curvature) in fp32.
//   sdf_mlp_bwd      warp per 16 samples: recomputes the activations from X,
//                    back-propagates the stencil arithmetic and the MLP and
//                    writes dL/dX.  dL/dW is a GEMM whose reduction dimension
//                    is the sample: each CTA stages 128 rows of (dZ, layer
//                    input) in shared memory, every warp owns a slice of the
//                    dW tiles and keeps it in registers for the whole kernel;
//                    one atomic flush per CTA at the end.
//   stencil_scatter  thread per (sample, level): dL/dtable of the taps with the
//                    same corner sharing (one atomic per distinct corner, warp-
//                    aggregated at coarse levels), and for the curvature taps
//                    the hash grid's positional derivative into dL/d(shifted).
//
// Order: forward   encode(FD) -> mlp_fwd(FD) -> encode(curv) -> mlp_fwd(curv)
//        backward  mlp_bwd(curv) -> scatter(curv) -> mlp_bwd(FD) -> scatter(FD)
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include "mlp.cuh"
#include "tc.cuh"

using namespace angelo;

// angelo_sdf_net_layout (include/angelo_gb.h): k_tiles1 = first-layer k-tiles
// (1 + levels/8), n_tiles3 = output n-tiles (width padded to 8), k_tiles3b =
// output width padded to 16 in k-tiles; byte offsets of the forward and
// backward B fragments (hi then lo of each), biases and output row 0.

namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kEncThreads = 128;
constexpr int kState = 16;      // per sample: sdf of the 13 evaluations, shifted point (3)
constexpr int kBState = 8;      // per sample, backward: dL/dshifted (3), dL/dnormal from curvature (3)
constexpr int kStageRows = kWarps * 16;
constexpr int kStageLd = 72;    // bf16 row stride of staged 64-wide operands (conflict-free ldmatrix)
constexpr uint32_t kAggregateRes = 300;  // levels up to this resolution aggregate their atomics

enum Group { kPoint = 0, kFD = 1, kCurv = 2 };

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

// tcgen05 operands of the three layers (Y = X W^T, kernel column order):
// element (n, k) at kmajor_offset(n, k, K) of the region's hi half, its lo
// part at the same offset of the lo half.
__global__ void sdf_prep_tc_kernel(const float *__restrict__ W1, const float *__restrict__ W2,
                                   const float *__restrict__ W3, int in_dim, int n_hash,
                                   angelo_sdf_net_layout lay, char *__restrict__ net) {
    const int K1 = 16 * lay.k_tiles1, N3 = 16 * lay.k_tiles3b;
    const int n1 = 64 * K1, n2 = lay.n_hidden == 2 ? 64 * 64 : 0, n3 = N3 * 64;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int layer, n, k, K;
    int64_t off, half;
    if (i < n1) {
        layer = 1, K = K1, n = i / K, k = i % K, off = lay.off_tcw1, half = (int64_t)n1 * 2;
    } else if ((i -= n1) < n2) {
        layer = 2, K = 64, n = i / 64, k = i % 64, off = lay.off_tcw2, half = (int64_t)n2 * 2;
    } else if ((i -= n2) < n3) {
        layer = 3, K = 64, n = i / 64, k = i % 64, off = lay.off_tcw3, half = (int64_t)n3 * 2;
    } else {
        return;
    }
    const float v = layer_w(layer, n, k, W1, W2, W3, in_dim, n_hash, lay.out_dim);
    const Split sp = split2(v, 0.0f);
    const uint32_t o = tc::kmajor_offset(n, k, K);
    *reinterpret_cast<uint16_t *>(net + off + o) = (uint16_t)(sp.hi & 0xFFFFu);
    *reinterpret_cast<uint16_t *>(net + off + half + o) = (uint16_t)(sp.lo & 0xFFFFu);
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
    // forward workspace
    float2 *X;        // encodings, X[(e * n_levels + l) * S + s]
    float *state;     // (S, kState): sdf of the 13 evaluations, shifted point
    // backward inputs
    const float *g_sdf, *g_grad, *g_feature, *g_laplace;
    int64_t gfeat_stride;
    // backward workspace and outputs
    float2 *dX;       // dL/dX, layout of X
    float *bstate;    // (S, kBState)
    float *d_table;   // float32 table gradient (atomic)
    float *d_net;     // flat weight gradient, kernel order (atomic)
};

__device__ __forceinline__ int64_t xidx(const SdfParams &P, int e, int l, int64_t s) {
    return ((int64_t)e * P.lay.n_levels + l) * P.S + s;
}

__device__ __forceinline__ float x2m1(float x) { return __fsub_rn(__fmul_rn(x, 2.f), 1.f); }

// Contracted coordinates of evaluation e of a sample around `base` (the point
// for e <= 6, the shifted point for e >= 7): e = 0 the point itself, else the
// stencil tap (e - 1) % 6 = +x,-x,+y,-y,+z,-z moved by eps and clamped to the
// box (models/geometry.py:224-246).  Mask bit d is set when coordinate d
// passed the clamp (its derivative is 1).
__device__ __forceinline__ void tap_point(float r, float eps, const float base[3], int e, float xc[3],
                                          int *mask) {
    const float two_r = __fsub_rn(r, -r);
    int m = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float v;
        if (e == 0) {
            v = base[d];
        } else {
            const int k = (e - 1) % 6;
            const float off = (k >> 1) == d ? ((k & 1) ? -eps : eps) : 0.0f;
            v = __fadd_rn(base[d], off);
            const bool inside = v >= -r && v <= r;
            v = fminf(fmaxf(v, -r), r);
            m |= inside << d;
        }
        xc[d] = __fdiv_rn(__fsub_rn(v, -r), two_r);
    }
    *mask = e == 0 ? 7 : m;
}

// Whether the +eps and -eps taps of axis d around base coordinate b are the
// same point after the clamp to [-r, r] (b beyond the box by more than eps).
// Their evaluations are then identical, the two contributions +h and -h of
// the FD backward cancel exactly, and the backward gives them weight 0: the
// reference's formulation reaches them through normalize() of a zero FD
// gradient, whose derivative is scaled by 1e12, and fp32 accumulation of
// those cancelling terms would otherwise leave rounding noise of that size.
__device__ __forceinline__ bool coincident_taps(float b, float r, float eps) {
    return fminf(fmaxf(__fadd_rn(b, eps), -r), r) == fminf(fmaxf(__fadd_rn(b, -eps), -r), r);
}

// The stencil centre whose corners the taps share: the base clamped to the
// box, so that the coordinates a tap does not move are bit-identical to it.
__device__ __forceinline__ void clamped_centre(float r, const float base[3], float xc[3]) {
    const float two_r = __fsub_rn(r, -r);
#pragma unroll
    for (int d = 0; d < 3; ++d) xc[d] = __fdiv_rn(__fsub_rn(fminf(fmaxf(base[d], -r), r), -r), two_r);
}

// Cell offset of a tap along its axis d relative to the centre: the tap shares
// the centre's corners when its other two cell coordinates equal the centre's
// and delta is -1, 0 or +1.
__device__ __forceinline__ bool tap_aligned(const LevelPos &p, const LevelPos &pc, int d, int *delta) {
    const int dl = (int)(p.g[d] - pc.g[d]);
    *delta = dl;
    return p.g[(d + 1) % 3] == pc.g[(d + 1) % 3] && p.g[(d + 2) % 3] == pc.g[(d + 2) % 3] && dl >= -1 &&
           dl <= 1;
}

// Does corner cc of a tap (axis d, offset delta) coincide with a centre corner?
__device__ __forceinline__ bool corner_shared(bool aligned, int delta, int cc, int d) {
    const int b = (cc >> d) & 1;
    return aligned && (delta == 0 || ((delta == 1) == (b == 0)));
}

// Value of the centre corner that corner cc of the tap coincides with (given
// corner_shared): delta 0 the same corner; +1 the tap's lower face is the
// centre's upper face; -1 the tap's upper face is the centre's lower face.
// cc and d are compile-time after unrolling, so this is a register select.
__device__ __forceinline__ float2 centre_value(const float2 (&vc)[8], int delta, int cc, int d) {
    const float2 other = ((cc >> d) & 1) == 0 ? vc[cc | (1 << d)] : vc[cc & ~(1 << d)];
    return delta == 0 ? vc[cc] : other;
}

// ---------------------------------------------------------------- encode

template <int GROUP>
__global__ void __launch_bounds__(kEncThreads) stencil_encode_kernel(const __grid_constant__ SdfParams P) {
    const int l = blockIdx.y;
    const int64_t s = (int64_t)blockIdx.x * kEncThreads + threadIdx.x;
    if (s >= P.S) return;
    const float r = P.radius, eps = P.eps;
    const float *src = GROUP == kCurv ? P.state + s * kState + 13 : P.pos + s * 3;
    const float base[3] = {src[0], src[1], src[2]};
    const float sc = P.lay.scales[l];
    const uint64_t off = P.lay.offsets[l];
    float xcc[3];
    clamped_centre(r, base, xcc);
    const LevelPos pc = level_pos(xcc[0], xcc[1], xcc[2], sc);
    float2 vc[8];
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) vc[cc] = load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, pc, cc));
    if (GROUP != kCurv) {
        float xc[3];
        int m;
        tap_point(r, eps, base, 0, xc, &m);
        const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
        const bool same = p.g[0] == pc.g[0] && p.g[1] == pc.g[1] && p.g[2] == pc.g[2];
        float2 f = make_float2(0.f, 0.f);
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
            const float w = corner_weight(p, cc);
            const float2 v = same ? vc[cc] : load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, p, cc));
            f.x = __fmaf_rn(w, v.x, f.x);
            f.y = __fmaf_rn(w, v.y, f.y);
        }
        P.X[xidx(P, 0, l, s)] = f;
    }
    if (GROUP != kPoint) {
        constexpr int e0 = GROUP == kFD ? 1 : 7;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int d = k >> 1;
            float xc[3];
            int m, delta;
            tap_point(r, eps, base, e0 + k, xc, &m);
            const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
            const bool aligned = tap_aligned(p, pc, d, &delta);
            float2 f = make_float2(0.f, 0.f);
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w = corner_weight(p, cc);
                const float2 v = corner_shared(aligned, delta, cc, d)
                                     ? centre_value(vc, delta, cc, d)
                                     : load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, p, cc));
                f.x = __fmaf_rn(w, v.x, f.x);
                f.y = __fmaf_rn(w, v.y, f.y);
            }
            P.X[xidx(P, e0 + k, l, s)] = f;
        }
    }
}

// ------------------------------------------------------------ MLP operands
// A fragments of the first layer for rows g, g+8 of a 16-sample tile: hash
// levels q + 4j (k-tile j/2, upper half when j is odd) from X, the xyz k-tile
// (columns 2L + {0,1,2} = x*2-1; q = 0 holds (x, y), q = 1 holds (z, 0)).

template <int KH>
struct AFrag {
    uint32_t hi[KH + 1][4];
    uint32_t lo[KH + 1][4];
};

template <int KH>
__device__ __forceinline__ void load_x(const SdfParams &P, int e, int64_t s0, bool v0, bool v1, int lane,
                                       const float xc0[3], const float xc1[3], AFrag<KH> &A) {
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int j = 0; j < 2 * KH; ++j) {
        const int l = q + 4 * j;
        float2 f0 = make_float2(0.f, 0.f), f1 = make_float2(0.f, 0.f);
        if (l < P.active) {
            if (v0) f0 = __ldg(P.X + xidx(P, e, l, s0 + g));
            if (v1) f1 = __ldg(P.X + xidx(P, e, l, s0 + g + 8));
        }
        const Split a = split2(f0.x, f0.y), b = split2(f1.x, f1.y);
        const int kt = j >> 1, h = (j & 1) * 2;
        A.hi[kt][h] = a.hi;
        A.lo[kt][h] = a.lo;
        A.hi[kt][h + 1] = b.hi;
        A.lo[kt][h + 1] = b.lo;
    }
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
    if (q == 0) {
        a0 = x2m1(xc0[0]);
        a1 = x2m1(xc0[1]);
        b0 = x2m1(xc1[0]);
        b1 = x2m1(xc1[1]);
    } else if (q == 1) {
        a0 = x2m1(xc0[2]);
        b0 = x2m1(xc1[2]);
    }
    const Split sa = split2(a0, a1), sb = split2(b0, b1);
    A.hi[KH][0] = sa.hi;
    A.lo[KH][0] = sa.lo;
    A.hi[KH][1] = sb.hi;
    A.lo[KH][1] = sb.lo;
    A.hi[KH][2] = A.hi[KH][3] = A.lo[KH][2] = A.lo[KH][3] = 0u;
}

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

// unit FD normal from the six stencil SDFs s[0..5] = (+x,-x,+y,-y,+z,-z)
__device__ __forceinline__ float fd_grad(const float *s6, float eps, float g[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = __fdiv_rn(0.5f * __fsub_rn(s6[2 * d], s6[2 * d + 1]), eps);
    return sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
}

// --------------------------------------------------------------- MLP forward
// tcgen05: a CTA of 16 warps owns 128 consecutive samples through every
// evaluation of the group.  Row r (sample s0 + r, tensor-memory lane r) is
// shared by four threads: warp w serves lanes 32 (w % 4) .. + 31 and the
// 16-column slice w / 4 of every 64-wide layer.  Per evaluation and layer the
// layer input is staged as a bf16 hi/lo K-major operand (128 rows), one
// thread issues the three products of each 16-wide K step (lo*hi, hi*lo,
// hi*hi) into fp32 tensor memory and commits them to an mbarrier, and every
// thread reads its slice back (bias, softplus, the next layer's operand).
// Two CTAs per SM overlap one's tensor work with the other's epilogue.

__device__ unsigned int g_tc_timeouts;   // CTAs that stopped waiting for the tensor cores

constexpr uint32_t kTcWaitPolls = 1u << 24;
constexpr int kTcThreads = 512;

template <int KH, int NH, int NT3>
struct TcFwdShape {
    static constexpr int K1 = 16 * (KH + 1);
    static constexpr int N3 = 16 * ((NT3 + 1) / 2);
    // bytes of one (hi or lo) half of each operand
    static constexpr uint32_t w1 = 64 * K1 * 2, w2 = NH == 2 ? 64 * 64 * 2 : 0, w3 = N3 * 64 * 2;
    static constexpr uint32_t a1 = 128 * K1 * 2, a2 = 128 * 64 * 2;
    static constexpr uint32_t off_w1 = 0, off_w2 = off_w1 + 2 * w1, off_w3 = off_w2 + 2 * w2,
                              off_a1 = off_w3 + 2 * w3, off_a2 = off_a1 + 2 * a1, off_bias = off_a2 + 2 * a2,
                              off_s13 = off_bias + (128 + N3) * 4, off_bar = off_s13 + 13 * 128 * 4,
                              bytes = off_bar + 16;
    static constexpr uint32_t tmem_cols = 256;   // Z1 [0, 64), Z2 [64, 128), output [128, 128 + N3)
};

// D (128 x N) = A (128 x 16 KSTEPS) * B (N x 16 KSTEPS)^T in bf16x3, one thread
template <int KSTEPS>
__device__ __forceinline__ void tc_layer(uint32_t d_tmem, uint32_t a_hi, uint32_t a_lo, uint32_t a_sbo,
                                         uint32_t b_hi, uint32_t b_lo, uint32_t b_sbo, uint32_t idesc) {
#pragma unroll
    for (int ks = 0; ks < KSTEPS; ++ks) {
        const uint32_t o = ks * 256;
        const uint64_t ah = tc::smem_desc(a_hi + o, 128, a_sbo), al = tc::smem_desc(a_lo + o, 128, a_sbo);
        const uint64_t bh = tc::smem_desc(b_hi + o, 128, b_sbo), bl = tc::smem_desc(b_lo + o, 128, b_sbo);
        tc::mma_bf16(d_tmem, al, bh, idesc, ks > 0 ? 1u : 0u);
        tc::mma_bf16(d_tmem, ah, bl, idesc, 1u);
        tc::mma_bf16(d_tmem, ah, bh, idesc, 1u);
    }
}

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

// 16 consecutive columns c0 .. c0 + 15 (c0 % 16 == 0) of row r of a K-major
// operand with K columns, split into bf16 hi and lo
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

template <int KH, int NH, int NT3, int GROUP>
__global__ void __launch_bounds__(kTcThreads, 2) sdf_mlp_fwd_kernel(const __grid_constant__ SdfParams P) {
    using Sh = TcFwdShape<KH, NH, NT3>;
    constexpr int K1 = Sh::K1, N3 = Sh::N3;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane, slice = warp >> 2;   // row of the tile, 16-column slice
    const angelo_sdf_net_layout &nl = P.nl;
    auto copy16 = [&](uint32_t dst, int64_t src, uint32_t bytes) {
        for (uint32_t i = tid * 16; i < bytes; i += kTcThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(Sh::off_w1, nl.off_tcw1, 2 * Sh::w1);
    if (NH == 2) copy16(Sh::off_w2, nl.off_tcw2, 2 * Sh::w2);
    copy16(Sh::off_w3, nl.off_tcw3, 2 * Sh::w3);
    float *bias = reinterpret_cast<float *>(smem + Sh::off_bias);   // b1 [64], b2 [64], b3 [N3]
    for (int i = tid; i < 128 + N3; i += kTcThreads) {
        float v = 0.f;
        if (i < 64) v = reinterpret_cast<const float *>(P.net + nl.off_b1)[i];
        else if (i < 128) v = NH == 2 ? reinterpret_cast<const float *>(P.net + nl.off_b2)[i - 64] : 0.f;
        else if (i - 128 < 8 * NT3) v = reinterpret_cast<const float *>(P.net + nl.off_b3)[i - 128];
        bias[i] = v;
    }
    float *s13 = reinterpret_cast<float *>(smem + Sh::off_s13);      // [13][128]
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + Sh::off_bar);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    char *a1h = smem + Sh::off_a1, *a1l = a1h + Sh::a1, *a2h = smem + Sh::off_a2, *a2l = a2h + Sh::a2;
    if (warp == 0) {
        tc::tmem_alloc(slot, Sh::tmem_cols);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(bar, 1);
    tc_publish();
    const uint32_t tmem = *slot;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t sA1h = tc::smem_addr(a1h), sA1l = tc::smem_addr(a1l);
    const uint32_t sA2h = tc::smem_addr(a2h), sA2l = tc::smem_addr(a2l);
    const uint32_t sW1h = tc::smem_addr(smem + Sh::off_w1), sW1l = sW1h + Sh::w1;
    const uint32_t sW2h = tc::smem_addr(smem + Sh::off_w2), sW2l = sW2h + Sh::w2;
    const uint32_t sW3h = tc::smem_addr(smem + Sh::off_w3), sW3l = sW3h + Sh::w3;
    constexpr uint32_t id_hidden = tc::idesc_bf16_f32(128, 64);
    constexpr uint32_t id_out_main = tc::idesc_bf16_f32(128, N3), id_out_tap = tc::idesc_bf16_f32(128, 16);

    constexpr int e0 = GROUP == kCurv ? 7 : 0;
    constexpr int ne = GROUP == kPoint ? 1 : (GROUP == kFD ? 7 : 6);
    const float r_ = P.radius, eps = P.eps;
    const int od = nl.out_dim;
    uint32_t phase = 0;
    bool alive = true;
    // work items k = (tile blockIdx.x + (k / ne) gridDim.x, evaluation e0 + k % ne)
    const int64_t n_tiles = (P.S + 127) / 128;
    const int64_t my_tiles = (int64_t)blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t n_items = my_tiles * ne;
    auto item_sample = [&](int64_t k) { return (blockIdx.x + (k / ne) * (int64_t)gridDim.x) * 128 + row; };
    auto item_base = [&](int64_t sk, float b[3]) {
        const bool vk = sk < P.S;
        const float *src = GROUP == kCurv ? P.state + sk * kState + 13 : P.pos + sk * 3;
        for (int d = 0; d < 3; ++d) b[d] = vk ? src[d] : 0.f;
    };
    // layer-1 operand of item k: slice q < KH holds hash levels 8q .. 8q + 7,
    // slice KH the xyz columns
    auto stage_x = [&](int64_t k) {
        const int64_t sk = item_sample(k);
        const int ek = e0 + (int)(k % ne);
        const bool vk = sk < P.S;
        if (slice < KH) {
            float x[16];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int l = 8 * slice + j;
                const float2 f = (vk && l < P.active) ? __ldg(P.X + xidx(P, ek, l, sk)) : make_float2(0.f, 0.f);
                x[2 * j] = f.x;
                x[2 * j + 1] = f.y;
            }
            stage16(a1h, a1l, row, 16 * slice, K1, x);
        } else if (slice == KH) {
            float b[3], xc[3], x[16];
            int m;
            item_base(sk, b);
            tap_point(r_, eps, b, ek, xc, &m);
#pragma unroll
            for (int j = 0; j < 16; ++j) x[j] = 0.f;
            x[0] = x2m1(xc[0]);
            x[1] = x2m1(xc[1]);
            x[2] = x2m1(xc[2]);
            stage16(a1h, a1l, row, 16 * KH, K1, x);
        }
    };
    if (n_items > 0) stage_x(0);
    for (int64_t k = 0; k < n_items && alive; ++k) {
        const int64_t s = item_sample(k);
        const bool v = s < P.S;
        const int i = (int)(k % ne), e = e0 + i;
        float base[3], xc[3];
        int m;
        item_base(s, base);
        tap_point(r_, eps, base, e, xc, &m);
        {
            tc_publish();
            if (tid == 0) {
                tc_layer<K1 / 16>(tmem, sA1h, sA1l, 16 * K1, sW1h, sW1l, 16 * K1, id_hidden);
                tc::commit(bar);
            }
            if (!(alive = tc_wait_all(bar, phase))) break;
            phase ^= 1;
            // the layer-1 operand is free: stage the next item's, whose loads
            // overlap this item's remaining layers
            if (k + 1 < n_items) stage_x(k + 1);
            // hidden layers: bias, softplus, next operand
#pragma unroll
            for (int layer = 0; layer < NH; ++layer) {
                const uint32_t zcol = 64 * layer;
                {
                    float z[16];
                    tc::ld16(tmem + lane_off + zcol + 16 * slice, z);
#pragma unroll
                    for (int j = 0; j < 16; ++j) z[j] = softplus100(z[j] + bias[64 * layer + 16 * slice + j]);
                    stage16(a2h, a2l, row, 16 * slice, 64, z);
                }
                tc_publish();
                if (tid == 0) {
                    if (layer + 1 < NH)
                        tc_layer<4>(tmem + 64, sA2h, sA2l, 1024, sW2h, sW2l, 1024, id_hidden);
                    else if (GROUP != kCurv && e == 0 && P.with_feature)
                        tc_layer<4>(tmem + 128, sA2h, sA2l, 1024, sW3h, sW3l, 1024, id_out_main);
                    else
                        tc_layer<4>(tmem + 128, sA2h, sA2l, 1024, sW3h, sW3l, 1024, id_out_tap);
                    tc::commit(bar);
                }
                if (!(alive = tc_wait_all(bar, phase))) break;
                phase ^= 1;
            }
            if (!alive) break;
            if (GROUP != kCurv && e == 0 && P.with_feature) {
                for (int q = slice; q < N3 / 16; q += 4) {
                    float y[16];
                    tc::ld16(tmem + lane_off + 128 + 16 * q, y);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int col = 16 * q + j;
                        const float val = y[j] + bias[128 + col];
                        if (col == 0) s13[row] = val;
                        if (v && col < od) P.feature[s * P.feat_stride + col] = val;
                    }
                }
                if (v && slice == 0) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) P.feature[s * P.feat_stride + od + d] = x2m1(xc[d]);
                }
            } else if (slice == 0) {
                float y[16];
                tc::ld16(tmem + lane_off + 128, y);
                s13[e * 128 + row] = y[0] + bias[128];
            }
        }
        if (!alive) break;
        // after the tile's last evaluation: the sample's stencil arithmetic
        // (s13 of row r is written and read by the same slice-0 thread)
        if (i == ne - 1 && v && slice == 0) {
            float *st = P.state + s * kState;
            float sv[13];
            for (int e = e0; e < e0 + ne; ++e) sv[e] = s13[e * 128 + row];
            if (GROUP != kCurv) {
                P.sdf[s] = sv[0];
                st[0] = sv[0];
            }
            if (GROUP == kFD) {
                float gr[3];
                const float gn = fmaxf(fd_grad(&sv[1], eps, gr), 1e-12f);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    P.grad[s * 3 + d] = gr[d];
                    st[1 + 2 * d] = sv[1 + 2 * d];
                    st[2 + 2 * d] = sv[2 + 2 * d];
                }
                if (P.with_laplace) {
                    // tangent-shifted point (models/geometry.py:236-246): the
                    // unit normal crossed with the unit random direction, added
                    // in contracted coordinates
                    const float *rd = P.rdir + s * 3;
                    const float rn = fmaxf(sqrtf(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]), 1e-12f);
                    float nrm[3], rdn[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        nrm[d] = gr[d] / gn;
                        rdn[d] = rd[d] / rn;
                    }
                    const float tg[3] = {nrm[1] * rdn[2] - nrm[2] * rdn[1], nrm[2] * rdn[0] - nrm[0] * rdn[2],
                                         nrm[0] * rdn[1] - nrm[1] * rdn[0]};
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const float xc = __fdiv_rn(__fsub_rn(base[d], -r_), __fsub_rn(r_, -r_));
                        st[13 + d] = __fadd_rn(xc, __fmul_rn(tg[d], eps));
                    }
                }
            }
            if (GROUP == kCurv) {
                float gr[3], gs[3], fd[6];
                for (int kk = 0; kk < 6; ++kk) fd[kk] = st[1 + kk];
                const float gn = fmaxf(fd_grad(fd, eps, gr), 1e-12f);
                const float gsn = fmaxf(fd_grad(&sv[7], eps, gs), 1e-12f);
                float dot = 0.f;
#pragma unroll
                for (int d = 0; d < 3; ++d) dot += (gr[d] / gn) * (gs[d] / gsn);
                dot = fminf(fmaxf(dot, -1.0f + 1e-6f), 1.0f - 1e-6f);
                P.laplace[s] = acosf(dot) / 3.14159265358979f;
                for (int e = 7; e < 13; ++e) st[e] = sv[e];
            }
        }
    }
    if (!alive && tid == 0) atomicAdd(&g_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, Sh::tmem_cols);
}

// -------------------------------------------------------------- MLP backward

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(smem_u32(p)));
}

// Store split A fragments (KT k-tiles, rows g and g+8 of this warp's 16) into
// row-major bf16 staging arrays hi/lo with row stride ld.
template <int KT>
__device__ __forceinline__ void stage_a(const uint32_t (&h)[KT][4], const uint32_t (&l)[KT][4], uint16_t *hi,
                                        uint16_t *lo, int ld, int row0, int lane) {
    const int g = lane >> 2, c = (lane & 3) * 2;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = row0 + g + ((i & 1) << 3);
            const int col = kt * 16 + ((i >> 1) << 3) + c;
            *reinterpret_cast<uint32_t *>(hi + row * ld + col) = h[kt][i];
            *reinterpret_cast<uint32_t *>(lo + row * ld + col) = l[kt][i];
        }
    }
}

// acc[i] += dZ^T B over the kStageRows staged rows, for output tile (mt, nt0 + i):
// A = dZ^T (m = unit, k = row) read transposed from the row-major dZ staging,
// B (k = row, n = input column) read transposed from the row-major input staging.
template <int NTW>
__device__ __forceinline__ void staged_dw(float (&acc)[NTW][4], const uint16_t *zh, const uint16_t *zl,
                                          const uint16_t *bh, const uint16_t *bl, int ldb, int mt, int nt0,
                                          int lane) {
    const int i8 = lane >> 3, j8 = lane & 7;
#pragma unroll 2
    for (int k0 = 0; k0 < kStageRows; k0 += 16) {
        const int arow = k0 + j8 + ((i8 >> 1) << 3), acol = mt * 16 + ((i8 & 1) << 3);
        uint32_t ah[4], al[4];
        ldsm_x4_t(ah, zh + arow * kStageLd + acol);
        ldsm_x4_t(al, zl + arow * kStageLd + acol);
        const int brow = k0 + j8 + ((i8 & 1) << 3);
#pragma unroll
        for (int i = 0; i < NTW; ++i) {
            uint32_t b_h[2], b_l[2];
            ldsm_x2_t(b_h, bh + brow * ldb + (nt0 + i) * 8);
            ldsm_x2_t(b_l, bl + brow * ldb + (nt0 + i) * 8);
            mma_x3(acc[i], ah, al, make_uint2(b_h[0], b_h[1]), make_uint2(b_l[0], b_l[1]));
        }
    }
}

struct BwdWarp {
    float base[16][3];
    float ds[16][13];   // dL/d(sdf) of each evaluation
};

struct BwdSmem {
    const uint2 *w1f, *w2f, *w1b, *w2b, *w3b;
    const float *b1, *b2, *w3row0;
    float *dW3, *db1, *db2, *db3;  // shared fp32 accumulators, kernel order
    uint16_t *zh, *zl, *bh, *bl;   // staging
};

template <int KH, int NH, int NT3>
struct BwdShape {
    static constexpr int KT3 = (NT3 + 1) / 2;
    static constexpr int XS = 16 * (KH + 1) + 8;      // staged input row stride (bf16)
    static constexpr int OUTP = 16 * KT3;
    static constexpr int64_t w1f = 2 * (KH + 1) * 8 * 32 * 8;
    static constexpr int64_t w2f = NH == 2 ? 2 * 4 * 8 * 32 * 8 : 0;
    static constexpr int64_t w1b = 2 * 4 * (2 * (KH + 1)) * 32 * 8;
    static constexpr int64_t w2b = NH == 2 ? 2 * 4 * 8 * 32 * 8 : 0;
    static constexpr int64_t w3b = 2 * KT3 * 8 * 32 * 8;
    static constexpr int64_t vec = (3 * 64) * 4;
    static constexpr int64_t acc = (OUTP * 64 + 64 + 64 + OUTP) * 4;
    static constexpr int64_t stage1 = (int64_t)kStageRows * (kStageLd + XS) * 2 * 2;
    static constexpr int64_t stage2 = NH == 2 ? (int64_t)kStageRows * (kStageLd + kStageLd) * 2 * 2 : 0;
    static constexpr int64_t stage = stage1 > stage2 ? stage1 : stage2;
    static constexpr int64_t off_w2f = w1f, off_w1b = off_w2f + w2f, off_w2b = off_w1b + w1b,
                             off_w3b = off_w2b + w2b, off_vec = off_w3b + w3b, off_acc = off_vec + vec,
                             off_stage = (off_acc + acc + 15) / 16 * 16, off_warp = off_stage + stage;
    static constexpr int64_t bytes = off_warp + kWarps * sizeof(BwdWarp);
};

template <int KH, int NH, int NT3, int GROUP>
__global__ void __launch_bounds__(kThreads, 1) sdf_mlp_bwd_kernel(const __grid_constant__ SdfParams P) {
    using Sh = BwdShape<KH, NH, NT3>;
    constexpr int KT3 = Sh::KT3;
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const angelo_sdf_net_layout &nl = P.nl;
    auto copy16 = [&](int64_t dst, int64_t src, int64_t bytes) {
        for (int64_t i = tid * 16; i < bytes; i += kThreads * 16)
            *reinterpret_cast<uint4 *>(smem + dst + i) = *reinterpret_cast<const uint4 *>(P.net + src + i);
    };
    copy16(0, nl.off_w1f, Sh::w1f);
    if (NH == 2) copy16(Sh::off_w2f, nl.off_w2f, Sh::w2f);
    copy16(Sh::off_w1b, nl.off_w1b, Sh::w1b);
    if (NH == 2) copy16(Sh::off_w2b, nl.off_w2b, Sh::w2b);
    if (GROUP != kCurv) copy16(Sh::off_w3b, nl.off_w3b, Sh::w3b);
    float *vec = reinterpret_cast<float *>(smem + Sh::off_vec);
    for (int i = tid; i < 64; i += kThreads) {
        vec[i] = reinterpret_cast<const float *>(P.net + nl.off_b1)[i];
        vec[64 + i] = NH == 2 ? reinterpret_cast<const float *>(P.net + nl.off_b2)[i] : 0.f;
        vec[128 + i] = reinterpret_cast<const float *>(P.net + nl.off_w3row0)[i];
    }
    float *acc = reinterpret_cast<float *>(smem + Sh::off_acc);
    const int n_acc = Sh::OUTP * 64 + 64 + 64 + Sh::OUTP;
    for (int i = tid; i < n_acc; i += kThreads) acc[i] = 0.f;
    BwdSmem S;
    S.w1f = reinterpret_cast<const uint2 *>(smem);
    S.w2f = reinterpret_cast<const uint2 *>(smem + Sh::off_w2f);
    S.w1b = reinterpret_cast<const uint2 *>(smem + Sh::off_w1b);
    S.w2b = reinterpret_cast<const uint2 *>(smem + Sh::off_w2b);
    S.w3b = reinterpret_cast<const uint2 *>(smem + Sh::off_w3b);
    S.b1 = vec;
    S.b2 = vec + 64;
    S.w3row0 = vec + 128;
    S.dW3 = acc;
    S.db1 = acc + Sh::OUTP * 64;
    S.db2 = S.db1 + 64;
    S.db3 = S.db2 + 64;
    // staging: phase 2 (two hidden layers) dZ2 | H1, phase 1 dZ1 | X
    uint16_t *zh = reinterpret_cast<uint16_t *>(smem + Sh::off_stage);
    uint16_t *zl = zh + kStageRows * kStageLd;
    uint16_t *b1h = zl + kStageRows * kStageLd, *b1l = b1h + kStageRows * Sh::XS;
    uint16_t *b2h = b1h, *b2l = b2h + kStageRows * kStageLd;
    BwdWarp &ws = reinterpret_cast<BwdWarp *>(smem + Sh::off_warp)[warp];
    __syncthreads();

    // dW tiles owned by this warp: unit block mt = warp / 2, n-tiles nt1 ..
    // nt1 + KH of the first layer and nt2 .. nt2 + 3 of the second
    const int mt = warp >> 1, nt1 = (warp & 1) * (KH + 1), nt2 = (warp & 1) * 4;
    float acc1[KH + 1][4], acc2[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (i < KH + 1) acc1[i][j] = 0.f;
            acc2[i][j] = 0.f;
        }
    }

    constexpr int e0 = GROUP == kCurv ? 7 : 0;
    constexpr int ne = GROUP == kPoint ? 1 : (GROUP == kFD ? 7 : 6);
    const int g = lane >> 2, q = lane & 3, c = q * 2;
    const float r_ = P.radius, eps = P.eps;
    const float inv2r = 1.0f / __fsub_rn(r_, -r_);
    const int64_t n_tiles = (P.S + 15) / 16;
    // CTA-uniform loop (the staged dW GEMM synchronises the CTA); tiles past
    // the end have no valid rows and contribute zeros
    for (int64_t tb = (int64_t)blockIdx.x * kWarps; tb < n_tiles; tb += (int64_t)gridDim.x * kWarps) {
        const int64_t s0 = (tb + warp) * 16;
        if (lane < 16) {
            const int64_t s = s0 + lane;
            const bool v = s < P.S;
            const float *st = P.state + s * kState;
            const float *src = GROUP == kCurv ? st + 13 : P.pos + s * 3;
#pragma unroll
            for (int d = 0; d < 3; ++d) ws.base[lane][d] = v ? src[d] : 0.f;
            for (int e = 0; e < 13; ++e) ws.ds[lane][e] = 0.f;
            if (v && GROUP == kCurv) {
                // curvature (models/geometry.py:247-251) back to the six
                // shifted-stencil SDFs; dL/dnormal from it kept for the FD pass
                float gr[3], gs[3], n[3], ns[3], dns[3], dgs[3];
                const float gn = fd_grad(st + 1, eps, gr);
                const float gsn = fd_grad(st + 7, eps, gs);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    n[d] = gr[d] / fmaxf(gn, 1e-12f);
                    ns[d] = gs[d] / fmaxf(gsn, 1e-12f);
                }
                const float dot = n[0] * ns[0] + n[1] * ns[1] + n[2] * ns[2];
                const float lo = -1.0f + 1e-6f, hi = 1.0f - 1e-6f;
                const float dotc = fminf(fmaxf(dot, lo), hi);
                const float dang = P.g_laplace ? P.g_laplace[s] / 3.14159265358979f : 0.f;
                const float ddot = (dot >= lo && dot <= hi) ? -dang / sqrtf(1.0f - dotc * dotc) : 0.f;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    P.bstate[s * kBState + 3 + d] = ddot * ns[d];
                    dns[d] = ddot * n[d];
                }
                normalize_bwd(gs, gsn, ns, dns, dgs);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float h = coincident_taps(st[13 + d], r_, eps) ? 0.f : __fdiv_rn(0.5f * dgs[d], eps);
                    ws.ds[lane][7 + 2 * d] = h;
                    ws.ds[lane][8 + 2 * d] = -h;
                }
            }
            if (v && GROUP != kCurv) {
                ws.ds[lane][0] = P.g_sdf ? P.g_sdf[s] : 0.f;
                if (GROUP == kFD) {
                    // FD gradient (and, with curvature, the normal that set the
                    // tangent shift) back to the six stencil SDFs
                    float gr[3], n[3], dn[3] = {0.f, 0.f, 0.f}, dg[3];
                    const float gn = fd_grad(st + 1, eps, gr);
#pragma unroll
                    for (int d = 0; d < 3; ++d) n[d] = gr[d] / fmaxf(gn, 1e-12f);
                    if (P.with_laplace) {
                        const float *rd = P.rdir + s * 3;
                        const float *bs = P.bstate + s * kBState;
                        const float rn = fmaxf(sqrtf(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]), 1e-12f);
                        float rdn[3], dtg[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            rdn[d] = rd[d] / rn;
                            dtg[d] = bs[d] * eps;
                            dn[d] = bs[3 + d];
                        }
                        // t = n x rd  ->  dL/dn += rd x dL/dt
                        dn[0] += rdn[1] * dtg[2] - rdn[2] * dtg[1];
                        dn[1] += rdn[2] * dtg[0] - rdn[0] * dtg[2];
                        dn[2] += rdn[0] * dtg[1] - rdn[1] * dtg[0];
                    }
                    normalize_bwd(gr, gn, n, dn, dg);
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const float gin = P.g_grad ? P.g_grad[s * 3 + d] : 0.f;
                        const float h = coincident_taps(P.pos[s * 3 + d], r_, eps)
                                            ? 0.f
                                            : __fdiv_rn(0.5f * (dg[d] + gin), eps);
                        ws.ds[lane][1 + 2 * d] = h;
                        ws.ds[lane][2 + 2 * d] = -h;
                    }
                }
            }
        }
        __syncwarp();
        const bool v0 = s0 + g < P.S, v1 = s0 + g + 8 < P.S;
        float dsh0[3] = {0.f, 0.f, 0.f}, dsh1[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
        for (int i = 0; i < ne; ++i) {
            const int e = e0 + i;
            float xc0[3], xc1[3];
            int m0, m1;
            tap_point(r_, eps, ws.base[g], e, xc0, &m0);
            tap_point(r_, eps, ws.base[g + 8], e, xc1, &m1);
            AFrag<KH> X;
            load_x<KH>(P, e, s0, v0, v1, lane, xc0, xc1, X);
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
            const float(&Zl)[8][4] = NH == 2 ? Z2 : Z1;
            // dL/dH of the last hidden layer
            float dH[8][4];
            if (GROUP != kCurv && e == 0) {
                // the point: the whole output row (dL/dfeature; column 0 also dL/dsdf)
                const int od = nl.out_dim;
                auto gval = [&](int row, int col, bool valid) -> float {
                    if (!valid || col >= od) return 0.f;
                    float v = P.g_feature ? P.g_feature[(s0 + row) * P.gfeat_stride + col] : 0.f;
                    if (col == 0) v += ws.ds[row][0];
                    return v;
                };
                uint32_t yh[KT3][4], yl[KT3][4];
#pragma unroll
                for (int kt = 0; kt < KT3; ++kt) {
#pragma unroll
                    for (int hf = 0; hf < 2; ++hf) {
                        const int col = kt * 16 + hf * 8 + c;
                        const Split a = split2(gval(g, col, v0), gval(g, col + 1, v0));
                        const Split b = split2(gval(g + 8, col, v1), gval(g + 8, col + 1, v1));
                        yh[kt][hf * 2] = a.hi;
                        yl[kt][hf * 2] = a.lo;
                        yh[kt][hf * 2 + 1] = b.hi;
                        yl[kt][hf * 2 + 1] = b.lo;
                    }
                }
                mm_nobias<KT3, 8>(yh, yl, S.w3b, 8, lane, dH);
                accumulate_dw<KT3, 4>(yh, yl, hlh, hll, S.dW3, 64, lane);
                float Y[2 * KT3][4];
#pragma unroll
                for (int nt = 0; nt < 2 * KT3; ++nt) {
                    const int col = nt * 8 + c;
                    Y[nt][0] = gval(g, col, v0);
                    Y[nt][1] = gval(g, col + 1, v0);
                    Y[nt][2] = gval(g + 8, col, v1);
                    Y[nt][3] = gval(g + 8, col + 1, v1);
                }
                accumulate_db<2 * KT3>(Y, S.db3, lane);
            } else {
                // a stencil tap: only the SDF column carries a gradient
                const float dy0 = v0 ? ws.ds[g][e] : 0.f, dy1 = v1 ? ws.ds[g + 8][e] : 0.f;
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
                if (lane < 4) {
#pragma unroll
                    for (int nt = 0; nt < 8; ++nt) {
                        red_add(S.dW3 + nt * 8 + lane * 2, part[nt][0]);
                        red_add(S.dW3 + nt * 8 + lane * 2 + 1, part[nt][1]);
                    }
                }
                // the taps' SDF-bias gradient, sum_e ds_e, is exactly zero (each
                // axis contributes +h and -h): it is not accumulated, so that
                // large cancelling terms do not round into the bias
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int k = 0; k < 4; ++k) dH[nt][k] *= softplus100_grad(Zl[nt][k]);
            uint32_t dzh[4][4], dzl[4][4];
            c_to_a(dH, dzh, dzl);
            if (NH == 2) {
                accumulate_db<8>(dH, S.db2, lane);
                stage_a<4>(dzh, dzl, zh, zl, kStageLd, warp * 16, lane);
                stage_a<4>(h1h, h1l, b2h, b2l, kStageLd, warp * 16, lane);
                __syncthreads();
                staged_dw<4>(acc2, zh, zl, b2h, b2l, kStageLd, mt, nt2, lane);
                __syncthreads();
                mm_nobias<4, 8>(dzh, dzl, S.w2b, 8, lane, dH);
#pragma unroll
                for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                    for (int k = 0; k < 4; ++k) dH[nt][k] *= softplus100_grad(Z1[nt][k]);
                c_to_a(dH, dzh, dzl);
            }
            accumulate_db<8>(dH, S.db1, lane);
            stage_a<4>(dzh, dzl, zh, zl, kStageLd, warp * 16, lane);
            stage_a<KH + 1>(X.hi, X.lo, b1h, b1l, Sh::XS, warp * 16, lane);
            __syncthreads();
            staged_dw<KH + 1>(acc1, zh, zl, b1h, b1l, Sh::XS, mt, nt1, lane);
            __syncthreads();
            // dL/dX: hash columns (n-tiles 0 .. 2KH-1; lane q holds level 4 nt + q)
            // and, for the curvature taps, the xyz n-tile
            constexpr int NTX = 2 * KH + (GROUP == kCurv ? 1 : 0);
            float dX[NTX][4];
            mm_nobias<4, NTX>(dzh, dzl, S.w1b, 2 * (KH + 1), lane, dX);
#pragma unroll
            for (int nt = 0; nt < 2 * KH; ++nt) {
                const int l = nt * 4 + q;
                if (l < P.active) {
                    if (v0) P.dX[xidx(P, e, l, s0 + g)] = make_float2(dX[nt][0], dX[nt][1]);
                    if (v1) P.dX[xidx(P, e, l, s0 + g + 8)] = make_float2(dX[nt][2], dX[nt][3]);
                }
            }
            if (GROUP == kCurv) {
                // xyz columns x*2-1: q = 0 holds (x, y), q = 1 holds z
                float d0[3] = {0.f, 0.f, 0.f}, d1[3] = {0.f, 0.f, 0.f};
                if (q == 0) {
                    d0[0] = 2.f * dX[NTX - 1][0];
                    d0[1] = 2.f * dX[NTX - 1][1];
                    d1[0] = 2.f * dX[NTX - 1][2];
                    d1[1] = 2.f * dX[NTX - 1][3];
                } else if (q == 1) {
                    d0[2] = 2.f * dX[NTX - 1][0];
                    d1[2] = 2.f * dX[NTX - 1][2];
                }
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if ((m0 >> d) & 1) dsh0[d] += d0[d] * inv2r;
                    if ((m1 >> d) & 1) dsh1[d] += d1[d] * inv2r;
                }
            }
        }
        if (GROUP == kCurv) {
            // dL/dshifted from the xyz columns; the scatter pass adds the hash
            // grid's positional derivative atomically
#pragma unroll
            for (int d = 0; d < 3; ++d) {
#pragma unroll
                for (int o = 1; o < 4; o <<= 1) {
                    dsh0[d] += __shfl_xor_sync(0xffffffffu, dsh0[d], o);
                    dsh1[d] += __shfl_xor_sync(0xffffffffu, dsh1[d], o);
                }
            }
            if (q == 0) {
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (v0) P.bstate[(s0 + g) * kBState + d] = dsh0[d];
                    if (v1) P.bstate[(s0 + g + 8) * kBState + d] = dsh1[d];
                }
            }
        }
        __syncwarp();
    }
    // one flush per CTA: register-held dW1 / dW2 tiles, shared dW3 and biases
    __syncthreads();
    const int K1c = 16 * (KH + 1);
#pragma unroll
    for (int i = 0; i < KH + 1; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int row = mt * 16 + g + ((j >> 1) << 3), col = (nt1 + i) * 8 + c + (j & 1);
            if (acc1[i][j] != 0.f) atomicAdd(P.d_net + row * K1c + col, acc1[i][j]);
        }
    }
    if (NH == 2) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int row = mt * 16 + g + ((j >> 1) << 3), col = (nt2 + i) * 8 + c + (j & 1);
                if (acc2[i][j] != 0.f) atomicAdd(P.d_net + 64 * K1c + row * 64 + col, acc2[i][j]);
            }
        }
    }
    for (int i = tid; i < n_acc; i += kThreads) {
        const float v = acc[i];
        if (v != 0.f) atomicAdd(P.d_net + 64 * K1c + 64 * 64 + i, v);
    }
}

// ------------------------------------------------------------------ scatter

__device__ __forceinline__ void centre_add(float2 (&acc)[8], int delta, int cc, int d, float2 v) {
    const int o = ((cc >> d) & 1) == 0 ? (cc | (1 << d)) : (cc & ~(1 << d));
    const bool z = delta == 0;
    acc[cc].x += z ? v.x : 0.f;
    acc[cc].y += z ? v.y : 0.f;
    acc[o].x += z ? 0.f : v.x;
    acc[o].y += z ? 0.f : v.y;
}

template <int GROUP>
__global__ void __launch_bounds__(kEncThreads) stencil_scatter_kernel(const __grid_constant__ SdfParams P) {
    const int l = blockIdx.y;
    const int64_t s = (int64_t)blockIdx.x * kEncThreads + threadIdx.x;
    const bool valid = s < P.S;
    const int64_t sv = valid ? s : P.S - 1;   // lanes past the end stay for the warp-collective adds
    const float r = P.radius, eps = P.eps;
    const float *src = GROUP == kCurv ? P.state + sv * kState + 13 : P.pos + sv * 3;
    const float base[3] = {src[0], src[1], src[2]};
    const float sc = P.lay.scales[l];
    const uint64_t off = P.lay.offsets[l];
    float2 *dt = reinterpret_cast<float2 *>(P.d_table);
    float xcc[3];
    clamped_centre(r, base, xcc);
    const LevelPos pc = level_pos(xcc[0], xcc[1], xcc[2], sc);
    float2 acc[8], vc[8];
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
        acc[cc] = make_float2(0.f, 0.f);
        vc[cc] = make_float2(0.f, 0.f);
        if (GROUP == kCurv && valid) vc[cc] = load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, pc, cc));
    }
    float dsh[3] = {0.f, 0.f, 0.f};
    if (GROUP != kCurv) {
        const float2 gx = valid ? P.dX[xidx(P, 0, l, s)] : make_float2(0.f, 0.f);
        const bool live = valid && (gx.x != 0.f || gx.y != 0.f);
        float xc[3];
        int m;
        tap_point(r, eps, base, 0, xc, &m);
        const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
        const bool same = p.g[0] == pc.g[0] && p.g[1] == pc.g[1] && p.g[2] == pc.g[2];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
            const float w = corner_weight(p, cc);
            const float2 v = make_float2(w * gx.x, w * gx.y);
            if (same) {
                acc[cc].x += v.x;
                acc[cc].y += v.y;
            } else if (live && dt) {
                atomicAdd(dt + off + corner_index(P.lay, l, p, cc), v);
            }
        }
    }
    if (GROUP != kPoint) {
        constexpr int e0 = GROUP == kFD ? 1 : 7;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int d = k >> 1;
            const float2 gx = valid ? P.dX[xidx(P, e0 + k, l, s)] : make_float2(0.f, 0.f);
            const bool live = valid && (gx.x != 0.f || gx.y != 0.f);
            float xc[3];
            int m, delta;
            tap_point(r, eps, base, e0 + k, xc, &m);
            const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
            const bool aligned = tap_aligned(p, pc, d, &delta);
            float dl[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w = corner_weight(p, cc);
                const float2 v = make_float2(w * gx.x, w * gx.y);
                const bool shared = corner_shared(aligned, delta, cc, d);
                if (shared) centre_add(acc, delta, cc, d, v);
                else if (live && dt) atomicAdd(dt + off + corner_index(P.lay, l, p, cc), v);
                if (GROUP == kCurv && live) {
                    // positional derivative of the interpolation (d w / d frac)
                    const float2 tv = shared ? centre_value(vc, delta, cc, d)
                                             : load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, p, cc));
                    const float gv = gx.x * tv.x + gx.y * tv.y;
#pragma unroll
                    for (int dd = 0; dd < 3; ++dd) {
                        float wd = 1.f;
#pragma unroll
                        for (int kk = 0; kk < 3; ++kk)
                            if (kk != dd) wd *= (cc >> kk) & 1 ? p.f[kk] : 1.f - p.f[kk];
                        dl[dd] += ((cc >> dd) & 1 ? wd : -wd) * gv;
                    }
                }
            }
            if (GROUP == kCurv) {
#pragma unroll
                for (int dd = 0; dd < 3; ++dd)
                    if ((m >> dd) & 1) dsh[dd] += sc * dl[dd];
            }
        }
    }
    if (dt) {
        const bool coarse = P.lay.resolutions[l] <= kAggregateRes;
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
            const uint64_t ent = off + corner_index(P.lay, l, pc, cc);
            const bool nz = valid && (acc[cc].x != 0.f || acc[cc].y != 0.f);
            if (coarse) aggregated_add2<1>(dt, ent, acc[cc].x, acc[cc].y, nz);
            else if (nz) atomicAdd(dt + ent, acc[cc]);
        }
    }
    if (GROUP == kCurv && valid) {
        const float inv2r = 1.0f / __fsub_rn(r, -r);
#pragma unroll
        for (int dd = 0; dd < 3; ++dd)
            if (dsh[dd] != 0.f) atomicAdd(P.bstate + s * kBState + dd, dsh[dd] * inv2r);
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
    // instantiated shapes: 8 levels / 1 hidden layer / 9..16 outputs and
    // 16 levels / 2 hidden layers / 65..72 outputs
    const int nt3 = (out_dim + 7) / 8;
    ANGELO_REQUIRE((n_levels == 8 && n_hidden == 1 && nt3 == 2) || (n_levels == 16 && n_hidden == 2 && nt3 == 9),
                   "sdf_net_layout: (%d levels, %d hidden, %d outputs) has no fused kernel "
                   "(8/1/9..16 or 16/2/65..72)",
                   n_levels, n_hidden, out_dim);
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
    L.off_tcw1 = take(2 * 64 * (16 * L.k_tiles1) * 2);
    L.off_tcw2 = take(n_hidden == 2 ? 2 * 64 * 64 * 2 : 0);
    L.off_tcw3 = take(2 * (16 * L.k_tiles3b) * 64 * 2);
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
    const int tc_elems = 64 * 16 * K1 + (nh == 2 ? 64 * 64 : 0) + 16 * lay->k_tiles3b * 64;
    sdf_prep_tc_kernel<<<blocks_for(tc_elems, 256), 256, 0, as_stream(stream)>>>(
        W1, W2, W3, in_dim, 2 * n_levels, *lay, reinterpret_cast<char *>(net));
    return check_launch("sdf_prep");
}


namespace {

constexpr int kSmallKH = 1, kSmallNH = 1, kSmallNT3 = 2;   // 8 levels, 1 hidden layer, 13 outputs
constexpr int kFullKH = 2, kFullNH = 2, kFullNT3 = 9;      // 16 levels, 2 hidden layers, 65 outputs

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(sms, 1);
}

template <int GROUP>
int launch_encode(const SdfParams &P, cudaStream_t s) {
    if (P.active == 0) return ANGELO_OK;
    const dim3 grid((unsigned)((P.S + kEncThreads - 1) / kEncThreads), (unsigned)P.active);
    stencil_encode_kernel<GROUP><<<grid, kEncThreads, 0, s>>>(P);
    return check_launch("sdf_stencil_encode");
}

template <int GROUP>
int launch_scatter(const SdfParams &P, cudaStream_t s) {
    if (P.active == 0 || (GROUP != kCurv && P.d_table == nullptr)) return ANGELO_OK;
    const dim3 grid((unsigned)((P.S + kEncThreads - 1) / kEncThreads), (unsigned)P.active);
    stencil_scatter_kernel<GROUP><<<grid, kEncThreads, 0, s>>>(P);
    return check_launch("sdf_stencil_scatter");
}

template <typename K>
int persistent_grid(K k, size_t smem, const SdfParams &P, const char *what, int *grid) {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch(what);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem);
    if (per_sm < 1) {
        set_error("%s: %zu bytes of shared memory do not fit an SM", what, smem);
        return ANGELO_E_UNSUPPORTED;
    }
    const int64_t tiles = (P.S + 15) / 16;
    const int64_t want = (tiles + kWarps - 1) / kWarps;
    *grid = (int)std::min<int64_t>(want, (int64_t)sm_count() * per_sm);
    return ANGELO_OK;
}

template <int KH, int NH, int NT3, int GROUP>
int launch_mlp_fwd(const SdfParams &P, cudaStream_t s) {
    const size_t smem = TcFwdShape<KH, NH, NT3>::bytes;
    auto k = sdf_mlp_fwd_kernel<KH, NH, NT3, GROUP>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess)
        return check_launch("sdf_mlp_fwd(smem attribute)");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kTcThreads, smem);
    if (per_sm < 1) {
        set_error("sdf_mlp_fwd: %zu bytes of shared memory do not fit an SM", smem);
        return ANGELO_E_UNSUPPORTED;
    }
    // two CTAs per SM: their registers (2 x 512 x 64) and shared memory
    // (2 x 115 KB) fit, and each holds 256 of the SM's 512 tensor-memory
    // columns (the occupancy query answers 1 here); CTAs beyond what the SMs
    // hold run as a later wave of the persistent loop
    per_sm = 2;
    const int64_t tiles = (P.S + 127) / 128;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sm_count() * per_sm);
    k<<<grid, kTcThreads, smem, s>>>(P);
    return check_launch("sdf_mlp_fwd");
}

template <int KH, int NH, int NT3, int GROUP>
int launch_mlp_bwd(const SdfParams &P, cudaStream_t s) {
    const size_t smem = BwdShape<KH, NH, NT3>::bytes;
    auto k = sdf_mlp_bwd_kernel<KH, NH, NT3, GROUP>;
    int grid = 0;
    const int rc = persistent_grid(k, smem, P, "sdf_mlp_bwd", &grid);
    if (rc != ANGELO_OK) return rc;
    k<<<grid, kThreads, smem, s>>>(P);
    return check_launch("sdf_mlp_bwd");
}

template <int KH, int NH, int NT3>
int run_fwd(const SdfParams &P, cudaStream_t s) {
    int rc;
    if (P.with_grad) {
        if ((rc = launch_encode<kFD>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_mlp_fwd<KH, NH, NT3, kFD>(P, s)) != ANGELO_OK) return rc;
    } else {
        if ((rc = launch_encode<kPoint>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_mlp_fwd<KH, NH, NT3, kPoint>(P, s)) != ANGELO_OK) return rc;
    }
    if (P.with_laplace) {
        if ((rc = launch_encode<kCurv>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_mlp_fwd<KH, NH, NT3, kCurv>(P, s)) != ANGELO_OK) return rc;
    }
    return ANGELO_OK;
}

template <int KH, int NH, int NT3>
int run_bwd(const SdfParams &P, cudaStream_t s) {
    int rc;
    if (P.with_laplace) {
        if ((rc = launch_mlp_bwd<KH, NH, NT3, kCurv>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_scatter<kCurv>(P, s)) != ANGELO_OK) return rc;
    }
    if (P.with_grad) {
        if ((rc = launch_mlp_bwd<KH, NH, NT3, kFD>(P, s)) != ANGELO_OK) return rc;
        return launch_scatter<kFD>(P, s);
    }
    if ((rc = launch_mlp_bwd<KH, NH, NT3, kPoint>(P, s)) != ANGELO_OK) return rc;
    return launch_scatter<kPoint>(P, s);
}

// The two instantiated network shapes; the layout query accepts only these.
bool shape_small(const angelo_sdf_net_layout &nl) {
    return nl.k_tiles1 == kSmallKH + 1 && nl.n_hidden == kSmallNH && nl.n_tiles3 == kSmallNT3;
}
bool shape_full(const angelo_sdf_net_layout &nl) {
    return nl.k_tiles1 == kFullKH + 1 && nl.n_hidden == kFullNH && nl.n_tiles3 == kFullNT3;
}

int64_t n_evals(int with_grad, int with_laplace) { return with_laplace ? 13 : (with_grad ? 7 : 1); }

}  // namespace

extern "C" int64_t angelo_sdf_workspace_floats(const angelo_hashgrid_layout_t *lay, int64_t n,
                                               int32_t with_grad, int32_t with_laplace,
                                               int32_t backward) {
    if (lay == nullptr || n < 0 || lay->n_levels < 1 || lay->n_levels > ANGELO_MAX_LEVELS) return -1;
    const int64_t x = 2 * n_evals(with_grad, with_laplace) * lay->n_levels * n;
    return x + (backward ? kBState : kState) * n;
}

extern "C" int angelo_sdf_stencil_fwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                      const void *table, int32_t table_dtype,
                                      const angelo_sdf_net_layout *nl, const void *net,
                                      const float *pos, const float *rand_dirs, int64_t n,
                                      float radius, float eps, int32_t with_grad,
                                      int32_t with_laplace, int32_t with_feature, float *sdf,
                                      float *grad, float *feature, int64_t feat_stride,
                                      float *laplace, float *workspace, void *stream) {
    ANGELO_REQUIRE(lay && nl && net && table, "sdf_stencil_fwd: null argument");
    ANGELO_REQUIRE(n >= 0, "sdf_stencil_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(lay->n_levels == 8 * (nl->k_tiles1 - 1), "sdf_stencil_fwd: levels vs net");
    ANGELO_REQUIRE(active_levels >= 0 && active_levels <= lay->n_levels, "sdf_stencil_fwd: active");
    ANGELO_REQUIRE(pos && sdf && workspace, "sdf_stencil_fwd: null pos/sdf/workspace");
    ANGELO_REQUIRE(!with_laplace || with_grad, "sdf_stencil_fwd: laplace needs the gradient");
    ANGELO_REQUIRE(!with_grad || grad, "sdf_stencil_fwd: null grad");
    ANGELO_REQUIRE(!with_laplace || (laplace && rand_dirs), "sdf_stencil_fwd: null laplace/rand");
    ANGELO_REQUIRE(!with_feature || (feature && feat_stride >= nl->out_dim + 3),
                   "sdf_stencil_fwd: bad feature output");
    ANGELO_REQUIRE(eps > 0.f && radius > 0.f, "sdf_stencil_fwd: eps/radius");
    ANGELO_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 7) == 0, "sdf_stencil_fwd: workspace alignment");
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
    P.X = reinterpret_cast<float2 *>(workspace);
    P.state = workspace + 2 * n_evals(with_grad, with_laplace) * lay->n_levels * n;
    cudaStream_t s = as_stream(stream);
    if (shape_full(*nl)) return run_fwd<kFullKH, kFullNH, kFullNT3>(P, s);
    if (shape_small(*nl)) return run_fwd<kSmallKH, kSmallNH, kSmallNT3>(P, s);
    set_error("sdf_stencil_fwd: network shape not instantiated");
    return ANGELO_E_UNSUPPORTED;
}

extern "C" int64_t angelo_tc_timeouts(int32_t reset) {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_timeouts, sizeof(v)) != cudaSuccess) return -1;
    if (reset) {
        const unsigned int z = 0;
        if (cudaMemcpyToSymbol(g_tc_timeouts, &z, sizeof(z)) != cudaSuccess) return -1;
    }
    return (int64_t)v;
}

extern "C" int64_t angelo_sdf_grad_size(const angelo_sdf_net_layout *nl) {
    const int k1cols = 16 * nl->k_tiles1, outp = 16 * nl->k_tiles3b;
    return 64 * k1cols + 64 * 64 + outp * 64 + 64 + 64 + outp;
}

extern "C" int angelo_sdf_stencil_bwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                      const void *table, int32_t table_dtype,
                                      const angelo_sdf_net_layout *nl, const void *net,
                                      const float *pos, const float *rand_dirs, int64_t n,
                                      float radius, float eps, int32_t with_grad,
                                      int32_t with_laplace, const float *workspace,
                                      float *bwd_workspace, const float *g_sdf,
                                      const float *g_grad, const float *g_feature,
                                      int64_t gfeat_stride, const float *g_laplace,
                                      float *d_table, float *d_net, void *stream) {
    ANGELO_REQUIRE(lay && nl && net && table && pos && workspace && bwd_workspace && d_net,
                   "sdf_stencil_bwd: null argument");
    ANGELO_REQUIRE(n >= 0, "sdf_stencil_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(lay->n_levels == 8 * (nl->k_tiles1 - 1), "sdf_stencil_bwd: levels vs net");
    ANGELO_REQUIRE(active_levels >= 0 && active_levels <= lay->n_levels, "sdf_stencil_bwd: active");
    ANGELO_REQUIRE(!with_laplace || (with_grad && rand_dirs), "sdf_stencil_bwd: laplace inputs");
    ANGELO_REQUIRE(g_feature == nullptr || gfeat_stride >= nl->out_dim, "sdf_stencil_bwd: stride");
    ANGELO_REQUIRE(eps > 0.f && radius > 0.f, "sdf_stencil_bwd: eps/radius");
    ANGELO_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 7) == 0 &&
                       (reinterpret_cast<uintptr_t>(bwd_workspace) & 7) == 0,
                   "sdf_stencil_bwd: workspace alignment");
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
    const int64_t x = 2 * n_evals(with_grad, with_laplace) * lay->n_levels * n;
    P.X = reinterpret_cast<float2 *>(const_cast<float *>(workspace));
    P.state = const_cast<float *>(workspace) + x;
    P.dX = reinterpret_cast<float2 *>(bwd_workspace);
    P.bstate = bwd_workspace + x;
    P.g_sdf = g_sdf;
    P.g_grad = g_grad;
    P.g_feature = g_feature;
    P.gfeat_stride = gfeat_stride;
    P.g_laplace = g_laplace;
    P.d_table = d_table;
    P.d_net = d_net;
    cudaStream_t s = as_stream(stream);
    if (shape_full(*nl)) return run_bwd<kFullKH, kFullNH, kFullNT3>(P, s);
    if (shape_small(*nl)) return run_bwd<kSmallKH, kSmallNH, kSmallNT3>(P, s);
    set_error("sdf_stencil_bwd: network shape not instantiated");
    return ANGELO_E_UNSUPPORTED;
}
