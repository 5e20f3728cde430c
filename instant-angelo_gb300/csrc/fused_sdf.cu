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
//   sdf_mlp_fwd      CTA of 16 warps per 128-sample tile: the geometry MLP of
//                    every evaluation on tcgen05 tensor cores (bf16x3 split,
//                    fp32 accumulation in tensor memory) from X, then the
//                    stencil arithmetic (sdf, FD gradient, tangent shift,
//                    curvature) in fp32.
//   sdf_mlp_bwd      the same layout: recomputes the activations from X,
//                    back-propagates the stencil arithmetic and the MLP and
//                    writes dL/dX; dL/dW accumulates in tensor memory over the
//                    CTA's tiles (one atomic flush per CTA).  The curvature
//                    taps' pass also forms dL/d(shifted point): the xyz
//                    columns and the hash grid's positional derivative, from
//                    the Jacobian dX/dfrac the curvature encode kept.
//   stencil_scatter  thread per (sample, level): dL/dtable of the taps with the
//                    same corner sharing (one atomic per distinct corner, warp-
//                    aggregated at coarse levels); both tap groups in one
//                    launch.
//
// Order: forward   encode(FD) -> mlp_fwd(FD) -> encode(curv) -> mlp_fwd(curv)
//        backward  mlp_bwd(curv) -> mlp_bwd(FD) -> scatter(FD and curv, one launch)
// (the curvature MLP backward takes the hash grid's positional derivative
// of its taps from the Jacobian the curvature encode kept, so the FD pass
// has dL/dshifted before the scatters run)
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include "mlp.cuh"
#include "tc.cuh"
#include "tc_mlp.cuh"

using namespace angelo;

// angelo_sdf_net_layout (include/angelo_gb.h): k_tiles1 = first-layer k-tiles
// of 16 columns (1 + levels/8), n_tiles3 = output width in tiles of 8,
// k_tiles3b = output width in tiles of 16; byte offsets of the fp32 biases,
// the fp32 output row 0 and the three tensor-core operands.

namespace {

constexpr int kEncThreads = 128;
// resident blocks per SM the encode and scatter kernels are compiled for
// (their register budget: 65536 / (128 x blocks) = 64 per thread at 8).
// Both wait on memory (random table gathers; L2 atomics), so more warps in
// flight pay more than the few registers they give up: measured on the
// samples of one training step (292k), 8 blocks took the backward call from
// 3.51 to 3.26 ms and the forward from 1.83 to 1.77 ms (6 and 10-12 less)
#ifndef ANGELO_ENCODE_MIN_BLOCKS
#define ANGELO_ENCODE_MIN_BLOCKS 8
#endif
#ifndef ANGELO_SCATTER_MIN_BLOCKS
#define ANGELO_SCATTER_MIN_BLOCKS 8
#endif
// both tap groups' table scatters in one launch (1) or one launch each (0)
#ifndef ANGELO_SCATTER_MERGED
#define ANGELO_SCATTER_MERGED 1
#endif
constexpr int kState = 16;      // per sample: sdf of the 13 evaluations, shifted point (3)
constexpr int kBState = 8;      // per sample, backward: dL/dshifted (3), dL/dnormal from curvature (3)
constexpr uint32_t kAggregateRes = 300;  // levels up to this resolution aggregate their atomics

enum Group { kPoint = 0, kFD = 1, kCurv = 2 };

// ------------------------------------------------------------------- prep
// Effective fp32 weights (after weight normalisation) -> bf16 hi/lo
// tensor-core operands.  W1 columns are permuted from the reference order
// [xyz(3), hash(2L)] to the kernel order [hash(2L), xyz(3), 0...].

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

// fp32 biases (zero padded) and row 0 of the output layer
__global__ void sdf_prep_vec_kernel(const float *__restrict__ b1, const float *__restrict__ b2,
                                    const float *__restrict__ W3, const float *__restrict__ b3,
                                    angelo_sdf_net_layout lay, char *__restrict__ net) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int NT3 = lay.n_tiles3;
    float *fb1 = reinterpret_cast<float *>(net + lay.off_b1);
    float *fb2 = reinterpret_cast<float *>(net + lay.off_b2);
    float *fb3 = reinterpret_cast<float *>(net + lay.off_b3);
    float *fr0 = reinterpret_cast<float *>(net + lay.off_w3row0);
    if (j < 64) {
        fb1[j] = b1[j];
    } else if (j < 128) {
        fb2[j - 64] = lay.n_hidden == 2 ? b2[j - 64] : 0.f;
    } else if (j < 128 + 8 * NT3) {
        const int o = j - 128;
        fb3[o] = o < lay.out_dim ? b3[o] : 0.f;
    } else if (j < 192 + 8 * NT3) {
        fr0[j - 128 - 8 * NT3] = W3[j - 128 - 8 * NT3];
    }
}

// tcgen05 operands of the three layers (Y = X W^T, kernel column order):
// element (n, k) at kmajor_offset(n, k, K) of the region's hi half, its lo
// part at the same offset of the lo half; bf16 or fp16 parts as the layout's
// operand_format says.
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
    const Split sp = lay.operand_format == ANGELO_OPERAND_FP16 ? split2h(v, 0.0f) : split2(v, 0.0f);
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
    int feat_vec4, gfeat_vec4;   // feature / dL/dfeature rows 16-byte aligned: 4-float accesses
    // forward workspace
    float2 *X;        // encodings, X[(e * n_levels + l) * S + s]
    float2 *J;        // curvature taps: d(encoding)/d(cell fraction),
                      // J[((k * n_levels + l) * 3 + axis) * S + s], k = tap 0..5
    float *state;     // (S, kState): sdf of the 13 evaluations, shifted point
    int32_t *perm;    // curvature pass: sample order by dead-tap pattern (may be null)
    int32_t *perm_blk;  // its per-block bucket counts (8 x ceil(S / 256))
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

// ------------------------------------------- curvature pass: dead tap pairs
// The curvature stencil is evaluated at contracted coordinates treated as
// world coordinates (models/geometry.py:246,264-265), so on every axis where
// the shifted point lies beyond r + eps both taps clamp to the same point:
// their SDFs are equal (the FD difference is exactly 0) and their backward
// contributions are 0.  The curvature pass orders its samples by that
// dead-axis pattern (a stable partition into 8 buckets), so that whole
// 128-sample tiles share it and the MLP kernels skip a tap whose pair is dead
// on every row of the tile; results are unchanged.

constexpr int kPermThreads = 256;

__device__ __forceinline__ int dead_pattern(const SdfParams &P, int64_t s) {
    const float *st = P.state + s * kState + 13;
    int p = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) p |= (int)coincident_taps(st[d], P.radius, P.eps) << d;
    return p;
}

// per block of kPermThreads samples: the count of each pattern,
// blk[pattern * nblk + block]
__global__ void __launch_bounds__(kPermThreads) perm_count_kernel(const __grid_constant__ SdfParams P, int nblk) {
    const int64_t s = (int64_t)blockIdx.x * kPermThreads + threadIdx.x;
    const int p = s < P.S ? dead_pattern(P, s) : -1;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int c = __syncthreads_count(p == b);
        if (threadIdx.x == 0) P.perm_blk[b * nblk + blockIdx.x] = c;
    }
}

// one block: exclusive prefix sum of the counts in pattern-major order
__global__ void __launch_bounds__(1024) perm_scan_kernel(int32_t *blk, int total) {
    __shared__ int32_t wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t carry = 0;
    for (int base = 0; base < total; base += 1024) {
        const int i = base + threadIdx.x;
        const int32_t v = i < total ? blk[i] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const int32_t before = (warp > 0 ? wsum[warp - 1] : 0) + x - v;
        if (i < total) blk[i] = carry + before;
        carry += wsum[31];
        __syncthreads();
    }
}

// position of each sample: its pattern's base in this block + its rank among
// the block's samples of that pattern (in sample order)
__global__ void __launch_bounds__(kPermThreads) perm_write_kernel(const __grid_constant__ SdfParams P, int nblk) {
    __shared__ int32_t wcnt[8][kPermThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s = (int64_t)blockIdx.x * kPermThreads + threadIdx.x;
    const int p = s < P.S ? dead_pattern(P, s) : -1;
    int rank = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const unsigned m = __ballot_sync(0xffffffffu, p == b);
        if (lane == 0) wcnt[b][warp] = __popc(m);
        if (p == b) rank = __popc(m & ((1u << lane) - 1u));
    }
    __syncthreads();
    if (p >= 0) {
        int32_t off = P.perm_blk[p * nblk + blockIdx.x] + rank;
        for (int w = 0; w < warp; ++w) off += wcnt[p][w];
        P.perm[off] = (int32_t)s;
    }
}

// ---------------------------------------------------------------- encode

template <int GROUP>
__global__ void __launch_bounds__(kEncThreads, ANGELO_ENCODE_MIN_BLOCKS)
    stencil_encode_kernel(const __grid_constant__ SdfParams P) {
    const int l = blockIdx.y;
    // position p of the pass; the curvature pass visits its samples in the
    // dead-tap order and keeps X and J by position, so that the MLP kernels'
    // rows (consecutive positions) read them coalesced
    const int64_t pidx = (int64_t)blockIdx.x * kEncThreads + threadIdx.x;
    if (pidx >= P.S) return;
    const int64_t s = (GROUP == kCurv && P.perm) ? (int64_t)P.perm[pidx] : pidx;
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
            // every tap's encoding and Jacobian are written, dead taps too:
            // dead and live taps are mixed across a warp's samples, and
            // skipping the dead ones' stores leaves partly written sectors
            // that cost more than the full stores (measured: forward call
            // +0.04 ms on one step's samples)
            float xc[3];
            int m, delta;
            tap_point(r, eps, base, e0 + k, xc, &m);
            const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
            const bool aligned = tap_aligned(p, pc, d, &delta);
            float2 f = make_float2(0.f, 0.f);
            float2 jac[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w = corner_weight(p, cc);
                const float2 v = corner_shared(aligned, delta, cc, d)
                                     ? centre_value(vc, delta, cc, d)
                                     : load_entry(P.table, P.tdtype, off + corner_index(P.lay, l, p, cc));
                f.x = __fmaf_rn(w, v.x, f.x);
                f.y = __fmaf_rn(w, v.y, f.y);
                if (GROUP == kCurv) {
                    // derivative of the trilinear weight along each axis
#pragma unroll
                    for (int dd = 0; dd < 3; ++dd) {
                        float wd = 1.f;
#pragma unroll
                        for (int kk = 0; kk < 3; ++kk)
                            if (kk != dd) wd *= (cc >> kk) & 1 ? p.f[kk] : 1.f - p.f[kk];
                        wd = (cc >> dd) & 1 ? wd : -wd;
                        jac[dd].x = __fmaf_rn(wd, v.x, jac[dd].x);
                        jac[dd].y = __fmaf_rn(wd, v.y, jac[dd].y);
                    }
                }
            }
            P.X[xidx(P, e0 + k, l, pidx)] = f;
            if (GROUP == kCurv) {
#pragma unroll
                for (int dd = 0; dd < 3; ++dd) P.J[((int64_t)(k * P.lay.n_levels + l) * 3 + dd) * P.S + pidx] = jac[dd];
            }
        }
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

// FP16: the operands (weights prepared with operand_format fp16 and the
// staged activations) are fp16 instead of bf16; with one pass per layer
// (nl.mma_passes == 1) only the hi parts are staged and multiplied.
template <int KH, int NH, int NT3, int GROUP, bool FP16>
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
    constexpr uint32_t id_hidden = tc::idesc_f32(128, 64, FP16);
    constexpr uint32_t id_out_main = tc::idesc_f32(128, N3, FP16), id_out_tap = tc::idesc_f32(128, 16, FP16);
    const bool with_lo = P.nl.mma_passes != 1;

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
    // position k of the pass -> sample (the curvature pass visits its samples
    // in P.perm's order); positions past S are padding rows
    auto item_pos = [&](int64_t k) { return (blockIdx.x + (k / ne) * (int64_t)gridDim.x) * 128 + row; };
    auto item_sample = [&](int64_t k) {
        const int64_t pk = item_pos(k);
        return (GROUP == kCurv && P.perm && pk < P.S) ? (int64_t)P.perm[pk] : pk;
    };
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
                const float2 f = (vk && l < P.active) ? __ldg(P.X + xidx(P, ek, l, GROUP == kCurv ? item_pos(k) : sk))
                                                      : make_float2(0.f, 0.f);
                x[2 * j] = f.x;
                x[2 * j + 1] = f.y;
            }
            stage16f<FP16>(a1h, a1l, row, 16 * slice, K1, x, with_lo);
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
            stage16f<FP16>(a1h, a1l, row, 16 * KH, K1, x, with_lo);
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
        // a curvature tap whose pair is dead on every row of the tile: its
        // SDF is the same for both taps, any value will do (0)
        bool skip = false;
        if (GROUP == kCurv)
            skip = !__syncthreads_or(v && !coincident_taps(base[(e - 7) >> 1], r_, eps));
        if (skip) {
            if (k + 1 < n_items) stage_x(k + 1);
            if (slice == 0) s13[e * 128 + row] = 0.f;
        } else {
            tc_publish();
            if (tid == 0) {
                tc_mma_p<K1 / 16>(tmem, op_k(sA1h, Sh::a1, K1), op_k(sW1h, Sh::w1, K1), id_hidden, false,
                                  P.nl.mma_passes);
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
                    stage16f<FP16>(a2h, a2l, row, 16 * slice, 64, z, with_lo);
                }
                tc_publish();
                if (tid == 0) {
                    if (layer + 1 < NH)
                        tc_mma_p<4>(tmem + 64, op_k(sA2h, Sh::a2, 64), op_k(sW2h, Sh::w2, 64), id_hidden, false,
                                    P.nl.mma_passes);
                    else if (GROUP != kCurv && e == 0 && P.with_feature)
                        tc_mma_p<4>(tmem + 128, op_k(sA2h, Sh::a2, 64), op_k(sW3h, Sh::w3, 64), id_out_main, false,
                                    P.nl.mma_passes);
                    else
                        tc_mma_p<4>(tmem + 128, op_k(sA2h, Sh::a2, 64), op_k(sW3h, Sh::w3, 64), id_out_tap, false,
                                    P.nl.mma_passes);
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
                        y[j] += bias[128 + 16 * q + j];
                        if (16 * q + j == 0) s13[row] = y[j];
                    }
                    if (v) {
                        float *frow = P.feature + s * P.feat_stride;
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            const int c = 16 * q + 4 * t;
                            if (P.feat_vec4 && c + 3 < od) {
                                *reinterpret_cast<float4 *>(frow + c) =
                                    make_float4(y[4 * t], y[4 * t + 1], y[4 * t + 2], y[4 * t + 3]);
                            } else {
#pragma unroll
                                for (int u = 0; u < 4; ++u)
                                    if (c + u < od) frow[c + u] = y[4 * t + u];
                            }
                        }
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

// ------------------------------------------------------ MLP backward (tcgen05)
// A CTA of 16 warps owns 128 consecutive samples through every evaluation of
// the group, with the forward kernel's thread layout (row r = tensor-memory
// lane r, four threads per row, one 16-column slice each).  Per evaluation
// the forward is recomputed and the backward runs as tensor-core rounds:
//
//   Z1 = X W1^T                     (two hidden layers:)  Z2 = H1 W2^T
//   dH of the last hidden layer: dY W3 for the point (a product), ds w3row0
//   for a stencil tap (rank one, in registers)
//   dH1 = dZ2 W2,  dW2 += dZ2^T H1,  db2 += dZ2^T 1
//   dX = dZ1 W1,   dW1 += dZ1^T X,   db1 += dZ1^T 1,  point: dW3^T += H^T dY
//
// A stencil tap adds ds H to row 0 of dW3 in fp32 (a warp reduce-scatter over
// the rows): the taps come in +h / -h pairs whose sum cancels to the
// difference of two nearby activations, which bf16x3 operands would resolve
// only to ~2^-17 of the activation.
// Each activation is staged once as a bf16 hi/lo K-major [sample][column]
// operand; the same bytes are the MN-major operand of the weight-gradient
// products over the 128 samples.  The weight gradients and the bias sums stay
// in tensor memory (M = 64 accumulators) for the CTA's whole loop and are
// added to the global gradient once.  Every round commits the product the
// next epilogue reads to mbarrier 0 and the weight-gradient products to
// mbarrier 1, so the epilogue overlaps them; operands are rewritten only after
// mbarrier 1 completed.

template <int KH, int NH, int NT3>
struct TcBwdShape {
    static constexpr int K1 = 16 * (KH + 1);
    static constexpr int N3 = 16 * ((NT3 + 1) / 2);
    // weights: bytes of one (hi or lo) half
    static constexpr uint32_t w1 = 64 * K1 * 2, w2 = NH == 2 ? 64 * 64 * 2 : 0, w3 = N3 * 64 * 2;
    // activation stagings, hi and lo side by side in a row: X [hi | lo] (the
    // hi column 16 KH + 3, a zero-weight pad, holds 1 for the bias sum),
    // H1 [hi | lo | 1-block] (column 128 = 1), H2 and Z [hi | lo], Y [hi | lo]
    static constexpr int CX = 2 * K1, CH1 = 144, CH = 128, CY = 2 * N3;
    static constexpr uint32_t x = 128 * CX * 2, h1 = 128 * CH1 * 2, h = 128 * CH * 2, y = 128 * CY * 2;
    static constexpr uint32_t off_w1 = 0, off_w2 = off_w1 + 2 * w1, off_w3 = off_w2 + 2 * w2,
                              off_x = off_w3 + 2 * w3,
                              off_h1 = off_x + x,                            // H1, then dZ1 (two layers)
                              off_h2 = off_h1 + h1,                          // H2 (two layers)
                              off_z = off_h2 + (NH == 2 ? h : 0),            // dZ of the last layer
                              off_y = off_z + h,                             // dY
                              off_vec = off_y + y,                           // b1, b2, W3 row 0
                              off_ds = off_vec + 3 * 64 * 4,                 // dL/dsdf [7][128]
                              off_db3 = off_ds + 7 * 128 * 4,
                              off_w3g = off_db3 + N3 * 4,                    // taps' dW3 row 0
                              off_bar = off_w3g + 64 * 4,
                              off_dsh = off_bar + 32,                        // dL/dshifted [128][3]
                              bytes = off_dsh + 128 * 3 * 4;
    // tensor-memory columns: per evaluation A, B; CTA-resident gradients: dW1
    // and dW2 (+ bias sums) as M = 128 products, rows hi then lo units, columns
    // the operand's hi then lo (four blocks summed at the end); dW3^T (M = 64)
    static constexpr uint32_t tA = 0, tB = 64, tW1 = 128, tW2 = tW1 + CX, tW3 = tW2 + (NH == 2 ? CH1 : 0),
                              used = tW3 + N3, tmem_cols = used <= 256 ? 256 : 512;
};

// dL/dsdf of the evaluations of GROUP of sample s (ds[e - e0]), from the
// incoming gradients and the stencil state kept by the forward; the curvature
// group stores dL/dnormal of the curvature for the FD pass (bstate 3..5).
template <int GROUP>
__device__ __forceinline__ void sample_ds(const SdfParams &P, int64_t s, float (&ds)[7]) {
    const float r_ = P.radius, eps = P.eps;
    const float *st = P.state + s * kState;
#pragma unroll
    for (int i = 0; i < 7; ++i) ds[i] = 0.f;
    if (GROUP == kCurv) {
        // curvature (models/geometry.py:247-251) back to the six
        // shifted-stencil SDFs
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
            ds[2 * d] = h;
            ds[2 * d + 1] = -h;
        }
        return;
    }
    ds[0] = P.g_sdf ? P.g_sdf[s] : 0.f;
    if (GROUP == kFD) {
        // FD gradient (and, with curvature, the normal that set the tangent
        // shift) back to the six stencil SDFs
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
            const float h = coincident_taps(P.pos[s * 3 + d], r_, eps) ? 0.f : __fdiv_rn(0.5f * (dg[d] + gin), eps);
            ds[1 + 2 * d] = h;
            ds[2 + 2 * d] = -h;
        }
    }
}

template <int KH, int NH, int NT3, int GROUP>
__global__ void __launch_bounds__(kTcThreads, 1) sdf_mlp_bwd_tc_kernel(const __grid_constant__ SdfParams P) {
    using Sh = TcBwdShape<KH, NH, NT3>;
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
    float *vec = reinterpret_cast<float *>(smem + Sh::off_vec);   // b1 [64], b2 [64], W3 row 0 [64]
    for (int i = tid; i < 192; i += kTcThreads) {
        float v;
        if (i < 64) v = reinterpret_cast<const float *>(P.net + nl.off_b1)[i];
        else if (i < 128) v = NH == 2 ? reinterpret_cast<const float *>(P.net + nl.off_b2)[i - 64] : 0.f;
        else v = reinterpret_cast<const float *>(P.net + nl.off_w3row0)[i - 128];
        vec[i] = v;
    }
    char *xs = smem + Sh::off_x, *h1s = smem + Sh::off_h1, *h2s = smem + Sh::off_h2, *zs = smem + Sh::off_z,
         *ys = smem + Sh::off_y;
    // the constant block of H1's staging: column 128 = 1, 129 .. 143 = 0
    for (int i = tid; i < 128 * 16; i += kTcThreads)
        *reinterpret_cast<uint16_t *>(h1s + tc::kmajor_offset(i >> 4, 128 + (i & 15), Sh::CH1)) =
            (i & 15) == 0 ? (uint16_t)0x3F80u : (uint16_t)0u;
    float *ds = reinterpret_cast<float *>(smem + Sh::off_ds);
    float *db3 = reinterpret_cast<float *>(smem + Sh::off_db3);
    for (int i = tid; i < N3; i += kTcThreads) db3[i] = 0.f;
    float *w3g = reinterpret_cast<float *>(smem + Sh::off_w3g);
    for (int i = tid; i < 64; i += kTcThreads) w3g[i] = 0.f;
    float *dsh_s = reinterpret_cast<float *>(smem + Sh::off_dsh);   // curvature: per-row dL/dshifted
    for (int i = tid; i < 128 * 3; i += kTcThreads) dsh_s[i] = 0.f;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + Sh::off_bar);   // [0] epilogue, [1] round
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 2);
    if (warp == 0) {
        tc::tmem_alloc(slot, Sh::tmem_cols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
    }
    tc_publish();
    const uint32_t tmem = *slot;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    // the CTA-resident gradient accumulators start at zero
    tmem_zero(tmem + lane_off, Sh::tW1, Sh::used, slice);
    tc_publish();

    const uint32_t sW1 = tc::smem_addr(smem + Sh::off_w1), sW2 = tc::smem_addr(smem + Sh::off_w2),
                   sW3 = tc::smem_addr(smem + Sh::off_w3), sX = tc::smem_addr(xs), sH1 = tc::smem_addr(h1s),
                   sH2 = tc::smem_addr(h2s), sZ = tc::smem_addr(zs), sY = tc::smem_addr(ys);
    const TcOp W1k = op_k(sW1, Sh::w1, K1), W1t = op_t(sW1, Sh::w1, K1);
    const TcOp W2k = op_k(sW2, Sh::w2, 64), W2t = op_t(sW2, Sh::w2, 64), W3t = op_t(sW3, Sh::w3, 64);
    // per-row products read hi / lo (op_k2); weight gradients read the whole
    // staging row, hi and lo stacked (op_t): one product per K step
    const TcOp Xk = op_k2(sX, K1, Sh::CX), Xs = op_t(sX, 0u, Sh::CX);
    const TcOp H1k = op_k2(sH1, 64, Sh::CH1), H1s = op_t(sH1, 0u, Sh::CH1), H1t = op_t2(sH1, 64, Sh::CH1);
    const TcOp H2t = op_t2(sH2, 64, Sh::CH), Zk = op_k2(sZ, 64, Sh::CH), Zs = op_t(sZ, 0u, Sh::CH);
    const TcOp Yk = op_k2(sY, N3, Sh::CY), Yt = op_t2(sY, N3, Sh::CY);
    // dZ1 lives in the H1 staging with two hidden layers, in the dZ staging with one
    const TcOp D1k = NH == 2 ? H1k : Zk, D1s = NH == 2 ? H1s : Zs, HLt = NH == 2 ? H2t : H1t;
    constexpr uint32_t id_fwd = tc::idesc_bf16_f32(128, 64);
    constexpr uint32_t id_dh = tc::idesc_bf16_f32(128, 64, 0, 1), id_dx = tc::idesc_bf16_f32(128, K1, 0, 1);
    constexpr uint32_t id_w1 = tc::idesc_bf16_f32(128, Sh::CX, 1, 1), id_w2 = tc::idesc_bf16_f32(128, Sh::CH1, 1, 1);
    constexpr uint32_t id_w3 = tc::idesc_bf16_f32(64, N3, 1, 1);

    constexpr int e0 = GROUP == kCurv ? 7 : 0;
    constexpr int ne = GROUP == kPoint ? 1 : (GROUP == kFD ? 7 : 6);
    const float r_ = P.radius, eps = P.eps;
    const float inv2r = 1.0f / __fsub_rn(r_, -r_);
    const int od = nl.out_dim;
    uint32_t ph0 = 0, ph1 = 0;
    bool alive = true;
    const int64_t n_tiles = (P.S + 127) / 128;
    const int64_t my_tiles = (int64_t)blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t n_items = my_tiles * ne;
    float g1[16];            // softplus' of this thread's layer-1 slice, kept for dZ1
    float dsh[3] = {0.f, 0.f, 0.f};
    constexpr int kDsSlice = 3;   // slice that runs a tile's ds prologue (stages no input)
    // layer-1 operand of item k (slice q < KH: hash levels 8q .. 8q + 7; slice
    // KH: xyz) into registers; issued two rounds before it is staged
    // position k of the pass -> sample (the curvature pass in P.perm's order)
    auto item_pos = [&](int64_t k) { return (blockIdx.x + (k / ne) * (int64_t)gridDim.x) * 128 + row; };
    auto item_sample = [&](int64_t k) {
        const int64_t pk = item_pos(k);
        return (GROUP == kCurv && P.perm && pk < P.S) ? (int64_t)P.perm[pk] : pk;
    };
    // the row of X, J and dX: the position (the curvature pass keeps them by
    // position in its sample order), else the sample
    auto item_row = [&](int64_t k, int64_t sk) { return GROUP == kCurv ? item_pos(k) : sk; };
    auto load_x = [&](int64_t k, float (&xv)[16]) {
        const int64_t s = item_sample(k);
        const bool v = s < P.S;
        const int e = e0 + (int)(k % ne);
#pragma unroll
        for (int j = 0; j < 16; ++j) xv[j] = 0.f;
        if (slice < KH) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int l = 8 * slice + j;
                const float2 f = (v && l < P.active) ? __ldg(P.X + xidx(P, e, l, item_row(k, s))) : make_float2(0.f, 0.f);
                xv[2 * j] = f.x;
                xv[2 * j + 1] = f.y;
            }
        } else if (slice == KH) {
            float b[3], xc[3];
            int m;
            const float *src = GROUP == kCurv ? P.state + s * kState + 13 : P.pos + s * 3;
#pragma unroll
            for (int d = 0; d < 3; ++d) b[d] = v ? src[d] : 0.f;
            tap_point(r_, eps, b, e, xc, &m);
#pragma unroll
            for (int d = 0; d < 3; ++d) xv[d] = x2m1(xc[d]);
            xv[3] = 1.f;   // zero-weight pad column: dW1 gathers the bias sum there
        }
    };
    float xv[16];
    if (n_items > 0) load_x(0, xv);
    // after a tile's last curvature tap: the four slices of a row add their
    // dL/dshifted up in shared memory and slice 0 stores it
    auto curv_tail = [&](int64_t s, bool v) {
        if (v) {
#pragma unroll
            for (int d = 0; d < 3; ++d) atomicAdd(dsh_s + row * 3 + d, dsh[d]);
        }
        __syncthreads();
        if (slice == 0) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (v) P.bstate[s * kBState + d] = dsh_s[row * 3 + d];
                dsh_s[row * 3 + d] = 0.f;
            }
        }
    };
    bool pending1 = false;   // weight-gradient products committed to bar[1], not yet waited for
    for (int64_t k = 0; k < n_items; ++k) {
        const int64_t s = item_sample(k);
        const bool v = s < P.S;
        const int i = (int)(k % ne), e = e0 + i;
        const bool point = GROUP != kCurv && e == 0;
        int m = 7;
        bool dead = false;
        if (GROUP == kCurv) {
            // which coordinates of this tap passed the clamp (for dL/dshifted)
            float base[3], xc[3];
            const float *src = P.state + s * kState + 13;
#pragma unroll
            for (int d = 0; d < 3; ++d) base[d] = v ? src[d] : 0.f;
            tap_point(r_, eps, base, e, xc, &m);
            dead = !v || coincident_taps(base[(e - 7) >> 1], r_, eps);
        }
        // a curvature tap whose pair is dead on every row of the tile has no
        // contribution (its dL/dX is not written; the scatter skips dead taps
        // the same way): it neither waits for the tensor core nor stages
        bool skip = false;
        if (GROUP == kCurv) skip = !__syncthreads_or(!dead);
        if (!skip) {
            if (pending1) {
                if (!(alive = tc_wait_all(&bar[1], ph1))) break;
                ph1 ^= 1;
                pending1 = false;
            }
            if (slice <= KH) stage16_2(xs, row, 16 * slice, K1, Sh::CX, xv);
        }
        if (i == 0) {
            if (slice == kDsSlice) {
                float d7[7];
                if (v) sample_ds<GROUP>(P, s, d7);
                else
                    for (int j = 0; j < 7; ++j) d7[j] = 0.f;
                for (int j = 0; j < ne; ++j) ds[j * 128 + row] = d7[j];
            }
            dsh[0] = dsh[1] = dsh[2] = 0.f;
        }
        if (point) {
            // dY: the output row's gradient (dL/dfeature, column 0 also dL/dsdf)
            // and its column sums (db3)
            const float d0 = v && P.g_sdf ? P.g_sdf[s] : 0.f;
            for (int q = slice; q < N3 / 16; q += 4) {
                float yv[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) yv[j] = 0.f;
                if (v && P.g_feature) {
                    const float *grow = P.g_feature + s * P.gfeat_stride;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int c = 16 * q + 4 * t;
                        if (P.gfeat_vec4 && c + 3 < od) {
                            const float4 g4 = __ldg(reinterpret_cast<const float4 *>(grow + c));
                            yv[4 * t] = g4.x;
                            yv[4 * t + 1] = g4.y;
                            yv[4 * t + 2] = g4.z;
                            yv[4 * t + 3] = g4.w;
                        } else {
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                if (c + u < od) yv[4 * t + u] = grow[c + u];
                        }
                    }
                }
                if (q == 0) yv[0] += d0;
                stage16_2(ys, row, 16 * q, N3, Sh::CY, yv);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float a = yv[j];
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                    if (lane == 0 && a != 0.f) red_add(db3 + 16 * q + j, a);
                }
            }
        }
        if (skip) {
            if (k + 1 < n_items) load_x(k + 1, xv);
            if (i == ne - 1) curv_tail(s, v);
            continue;
        }
        tc_publish();
        // stage 1: Z1 (one hidden layer, point: also dH1 = dY W3)
        if (tid == 0) {
            tc_mma<K1 / 16>(tmem + Sh::tA, Xk, W1k, id_fwd, false);
            if (NH == 1 && point) tc_mma<N3 / 16>(tmem + Sh::tB, Yk, W3t, id_dh, false);
            tc::commit(&bar[0]);
        }
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        float hl[16];   // this slice of the last hidden layer's activations
        {
            float z[16];
            tc::ld16(tmem + lane_off + Sh::tA + 16 * slice, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) softplus100_both(z[j] + vec[16 * slice + j], &hl[j], &g1[j]);
            stage16_2(h1s, row, 16 * slice, 64, Sh::CH1, hl);
        }
        if (NH == 2) {
            tc_publish();
            // stage 2: Z2 (point: also dH2 = dY W3)
            if (tid == 0) {
                tc_mma<4>(tmem + Sh::tB, H1k, W2k, id_fwd, false);
                if (point) tc_mma<N3 / 16>(tmem + Sh::tA, Yk, W3t, id_dh, false);
                tc::commit(&bar[0]);
            }
            if (!(alive = tc_wait_all(&bar[0], ph0))) break;
            ph0 ^= 1;
        }
        {
            // last hidden layer: H (two layers: staged for dW3), dH, dZ
            float gl[16], dh[16];
            if (NH == 2) {
                float z[16];
                tc::ld16(tmem + lane_off + Sh::tB + 16 * slice, z);
#pragma unroll
                for (int j = 0; j < 16; ++j) softplus100_both(z[j] + vec[64 + 16 * slice + j], &hl[j], &gl[j]);
                if (point) stage16_2(h2s, row, 16 * slice, 64, Sh::CH, hl);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) gl[j] = g1[j];
            }
            if (point) {
                tc::ld16(tmem + lane_off + (NH == 2 ? Sh::tA : Sh::tB) + 16 * slice, dh);
            } else {
                const float d = ds[i * 128 + row];
                float part[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    dh[j] = d * vec[128 + 16 * slice + j];
                    part[j] = d * hl[j];
                }
                int col;
                const float sum = warp_colsum16(part, lane, &col);
                if ((lane & 1) == 0 && sum != 0.f) red_add(w3g + 16 * slice + col, sum);
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) dh[j] *= gl[j];
            stage16_2(zs, row, 16 * slice, 64, Sh::CH, dh);
        }
        // the next item's encodings, in flight during this item's last rounds
        if (k + 1 < n_items) load_x(k + 1, xv);
        tc_publish();
        if (NH == 2) {
            // stage 3: dH1 (epilogue), then dW2, db2, dW3
            if (tid == 0) {
                tc_mma<4>(tmem + Sh::tA, Zk, W2t, id_dh, false);
                tc::commit(&bar[0]);
                tc_mma1<8>(tmem + Sh::tW2, Zs, H1s, id_w2, true);   // dW2 and db2
                if (point) tc_mma<8>(tmem + Sh::tW3, HLt, Yt, id_w3, true);
                tc::commit(&bar[1]);
            }
            if (!(alive = tc_wait_all(&bar[0], ph0))) break;
            ph0 ^= 1;
            float dz[16];
            tc::ld16(tmem + lane_off + Sh::tA + 16 * slice, dz);
#pragma unroll
            for (int j = 0; j < 16; ++j) dz[j] *= g1[j];
            // H1 is read by dW2: rewrite it as dZ1 after the round completed
            if (!(alive = tc_wait_all(&bar[1], ph1))) break;
            ph1 ^= 1;
            stage16_2(h1s, row, 16 * slice, 64, Sh::CH1, dz);
            tc_publish();
        }
        // last stage: dX (epilogue), then dW1, db1 (one hidden layer: dW3)
        if (tid == 0) {
            tc_mma<4>(tmem + Sh::tB, D1k, W1t, id_dx, false);
            tc::commit(&bar[0]);
            tc_mma1<8>(tmem + Sh::tW1, D1s, Xs, id_w1, true);   // dW1 and db1
            if (NH == 1 && point) tc_mma<8>(tmem + Sh::tW3, HLt, Yt, id_w3, true);
            tc::commit(&bar[1]);
        }
        pending1 = true;
        if (!(alive = tc_wait_all(&bar[0], ph0))) break;
        ph0 ^= 1;
        constexpr int CPS = 4 * KH;   // dL/dX columns of a slice
        float dxs[CPS];
        const int64_t xr = item_row(k, s);   // this item's row of dX and J
        {
            // dL/dX of hash levels (CPS / 2) slice .. : all four slices
            tc::ldn(tmem + lane_off + Sh::tB + CPS * slice, dxs);
#pragma unroll
            for (int j = 0; j < CPS / 2; ++j) {
                const int l = (CPS / 2) * slice + j;
                if (v && l < P.active) P.dX[xidx(P, e, l, xr)] = make_float2(dxs[2 * j], dxs[2 * j + 1]);
            }
        }
        if (GROUP == kCurv) {
            // dL/dshifted: the xyz columns x*2-1 (slice 0) and the hash grid's
            // positional derivative dL/dX . dX/dfrac * scale of this slice's
            // levels, from the Jacobian the forward encode kept; both
            // through the clamp (mask m) and the contraction (1 / 2r)
            if (slice == 0) {
                float dx[8];
                tc::ld8(tmem + lane_off + Sh::tB + 16 * KH, dx);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if ((m >> d) & 1) dsh[d] += 2.f * dx[d] * inv2r;
            }
            {
                // this slice's dL/dX (dxs, loaded by every lane above: the
                // load is warp-collective); only live rows use it
                const float *dx = dxs;
                const int k6 = e - 7;
#pragma unroll
                for (int j = 0; j < CPS / 2; ++j) {
                    const int l = (CPS / 2) * slice + j;
                    // a dead tap has no Jacobian (and dL/dX = 0)
                    if (dead || l >= P.active) continue;
                    const float sc = P.lay.scales[l] * inv2r;
#pragma unroll
                    for (int dd = 0; dd < 3; ++dd) {
                        if (!((m >> dd) & 1)) continue;
                        const float2 jv = __ldg(P.J + ((int64_t)(k6 * P.lay.n_levels + l) * 3 + dd) * P.S + xr);
                        dsh[dd] += sc * (dx[2 * j] * jv.x + dx[2 * j + 1] * jv.y);
                    }
                }
            }
            if (i == ne - 1) curv_tail(s, v);
        }
    }
    if (alive && pending1) alive = tc_wait_all(&bar[1], ph1);
    if (alive) {
        // add the CTA's gradients.  dW1, dW2: lane r = row r of an M = 128
        // product (unit r % 64, hi rows then lo rows), column = operand column
        // (hi then lo part; X's pad column 16 KH + 3 and H1's column 128 carry
        // the bias sums).  dW3^T: M = 64, row 16 (warp % 4) + lane, lanes < 16.
        const int r128 = 32 * (warp & 3) + lane, u128 = r128 & 63, u64 = 16 * (warp & 3) + lane;
        float *dW2 = P.d_net + 64 * K1, *dW3 = dW2 + 64 * 64, *db1 = dW3 + N3 * 64, *db2 = db1 + 64,
              *dB3 = db2 + 64;
        for (uint32_t b = slice; b < (Sh::used - Sh::tW1) / 16; b += 4) {
            const uint32_t c0 = Sh::tW1 + 16 * b;
            float w[16];
            __syncwarp();
            tc::ld16(tmem + lane_off + c0, w);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const uint32_t c = c0 + j;
                float *dst = nullptr;
                if (c < Sh::tW2) {
                    const int k = (int)(c - Sh::tW1) % K1;
                    dst = k == 16 * KH + 3 ? db1 + u128 : P.d_net + u128 * K1 + k;
                } else if (c < Sh::tW3) {
                    const int k = (int)(c - Sh::tW2);
                    dst = k < 128 ? dW2 + u128 * 64 + (k & 63) : (k == 128 ? db2 + u128 : nullptr);
                } else if (lane < 16) {
                    dst = dW3 + (c - Sh::tW3) * 64 + u64;
                }
                if (dst && w[j] != 0.f) atomicAdd(dst, w[j]);
            }
        }
        for (int o = tid; o < N3; o += kTcThreads)
            if (db3[o] != 0.f) atomicAdd(dB3 + o, db3[o]);
        for (int h = tid; h < 64; h += kTcThreads)
            if (w3g[h] != 0.f) atomicAdd(dW3 + h, w3g[h]);
    }
    if (!alive && tid == 0) atomicAdd(&g_tc_timeouts, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, Sh::tmem_cols);
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

// dL/dtable of one (sample, level) of tap group GROUP: thread (blockIdx.x,
// threadIdx.x) = sample, blockIdx.y = level
template <int GROUP>
__device__ __forceinline__ void scatter_body(const SdfParams &P) {
    const int l = blockIdx.y;
    // position s of the pass (the curvature pass: its dead-tap order, in which
    // dL/dX is kept; the sample is perm[s])
    const int64_t s = (int64_t)blockIdx.x * kEncThreads + threadIdx.x;
    const bool valid = s < P.S;
    const int64_t pv = valid ? s : P.S - 1;   // lanes past the end stay for the warp-collective adds
    const int64_t sv = (GROUP == kCurv && P.perm) ? (int64_t)P.perm[pv] : pv;
    const float r = P.radius, eps = P.eps;
    const float *src = GROUP == kCurv ? P.state + sv * kState + 13 : P.pos + sv * 3;
    const float base[3] = {src[0], src[1], src[2]};
    const float sc = P.lay.scales[l];
    const uint64_t off = P.lay.offsets[l];
    float2 *dt = reinterpret_cast<float2 *>(P.d_table);
    float xcc[3];
    clamped_centre(r, base, xcc);
    const LevelPos pc = level_pos(xcc[0], xcc[1], xcc[2], sc);
    float2 acc[8];
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) acc[cc] = make_float2(0.f, 0.f);
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
            // a curvature tap whose pair is dead contributes nothing (and its
            // dL/dX is not written when its whole tile was dead)
            if (GROUP == kCurv && coincident_taps(base[d], r, eps)) continue;
            const float2 gx = valid ? P.dX[xidx(P, e0 + k, l, s)] : make_float2(0.f, 0.f);
            const bool live = valid && (gx.x != 0.f || gx.y != 0.f);
            float xc[3];
            int m, delta;
            tap_point(r, eps, base, e0 + k, xc, &m);
            const LevelPos p = level_pos(xc[0], xc[1], xc[2], sc);
            const bool aligned = tap_aligned(p, pc, d, &delta);
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {
                const float w = corner_weight(p, cc);
                const float2 v = make_float2(w * gx.x, w * gx.y);
                if (corner_shared(aligned, delta, cc, d)) centre_add(acc, delta, cc, d, v);
                else if (live && dt) atomicAdd(dt + off + corner_index(P.lay, l, p, cc), v);
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
}


template <int GROUP>
__global__ void __launch_bounds__(kEncThreads, ANGELO_SCATTER_MIN_BLOCKS)
    stencil_scatter_kernel(const __grid_constant__ SdfParams P) {
    scatter_body<GROUP>(P);
}

// Both tap groups in one launch: blockIdx.z 0 = the point and its FD taps,
// 1 = the curvature taps (their scatters are independent once the
// curvature taps' positional derivative is taken in their MLP backward)
__global__ void __launch_bounds__(kEncThreads, ANGELO_SCATTER_MIN_BLOCKS)
    stencil_scatter_both_kernel(const __grid_constant__ SdfParams P) {
    if (blockIdx.z == 0) scatter_body<kFD>(P);
    else scatter_body<kCurv>(P);
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
    L.off_b1 = take(64 * 4);
    L.off_b2 = take(64 * 4);
    L.off_b3 = take(8 * L.n_tiles3 * 4);
    L.off_w3row0 = take(64 * 4);
    L.off_tcw1 = take(2 * 64 * (16 * L.k_tiles1) * 2);
    L.off_tcw2 = take(n_hidden == 2 ? 2 * 64 * 64 * 2 : 0);
    L.off_tcw3 = take(2 * (16 * L.k_tiles3b) * 64 * 2);
    L.bytes = o;
    L.mma_passes = 3;
    L.operand_format = ANGELO_OPERAND_BF16;
    *out = L;
    return ANGELO_OK;
}

extern "C" int angelo_sdf_prep(const angelo_sdf_net_layout *lay, int32_t n_levels, int32_t in_dim,
                               const float *W1, const float *b1, const float *W2, const float *b2,
                               const float *W3, const float *b3, void *net, void *stream) {
    ANGELO_REQUIRE(lay && W1 && b1 && W3 && b3 && net, "sdf_prep: null pointer");
    ANGELO_REQUIRE(lay->n_hidden == 1 || (W2 && b2), "sdf_prep: missing hidden layer 2");
    ANGELO_REQUIRE(in_dim == 3 + 2 * n_levels, "sdf_prep: in_dim %d != 3 + 2*levels", in_dim);
    ANGELO_REQUIRE(lay->operand_format == ANGELO_OPERAND_BF16 || lay->operand_format == ANGELO_OPERAND_FP16,
                   "sdf_prep: operand_format %d", lay->operand_format);
    const int K1 = lay->k_tiles1, nh = lay->n_hidden;
    sdf_prep_vec_kernel<<<1, 192 + 8 * lay->n_tiles3, 0, as_stream(stream)>>>(
        b1, b2, W3, b3, *lay, reinterpret_cast<char *>(net));
    const int tc_elems = 64 * 16 * K1 + (nh == 2 ? 64 * 64 : 0) + 16 * lay->k_tiles3b * 64;
    sdf_prep_tc_kernel<<<blocks_for(tc_elems, 256), 256, 0, as_stream(stream)>>>(
        W1, W2, W3, in_dim, 2 * n_levels, *lay, reinterpret_cast<char *>(net));
    return check_launch("sdf_prep");
}


namespace {

constexpr int kSmallKH = 1, kSmallNH = 1, kSmallNT3 = 2;   // 8 levels, 1 hidden layer, 13 outputs
constexpr int kFullKH = 2, kFullNH = 2, kFullNT3 = 9;      // 16 levels, 2 hidden layers, 65 outputs


int64_t perm_blocks(int64_t n) { return (n + kPermThreads - 1) / kPermThreads; }

// the curvature pass's sample order, in the forward workspace after the
// Jacobians
void set_perm(SdfParams &P, float *workspace, int64_t n, int levels) {
    float *p = workspace + 2 * 13 * (int64_t)levels * n + kState * n + 2 * 6 * 3 * (int64_t)levels * n;
    P.perm = reinterpret_cast<int32_t *>(p);
    P.perm_blk = P.perm + n;
}

int launch_perm(const SdfParams &P, cudaStream_t s) {
    const int nblk = (int)perm_blocks(P.S);
    perm_count_kernel<<<nblk, kPermThreads, 0, s>>>(P, nblk);
    perm_scan_kernel<<<1, 1024, 0, s>>>(P.perm_blk, 8 * nblk);
    perm_write_kernel<<<nblk, kPermThreads, 0, s>>>(P, nblk);
    return check_launch("sdf_curvature_order");
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
    if (P.active == 0 || P.d_table == nullptr) return ANGELO_OK;
    const dim3 grid((unsigned)((P.S + kEncThreads - 1) / kEncThreads), (unsigned)P.active);
    stencil_scatter_kernel<GROUP><<<grid, kEncThreads, 0, s>>>(P);
    return check_launch("sdf_stencil_scatter");
}

int launch_scatter_both(const SdfParams &P, cudaStream_t s) {
    if (P.active == 0 || P.d_table == nullptr) return ANGELO_OK;
    const dim3 grid((unsigned)((P.S + kEncThreads - 1) / kEncThreads), (unsigned)P.active, 2);
    stencil_scatter_both_kernel<<<grid, kEncThreads, 0, s>>>(P);
    return check_launch("sdf_stencil_scatter");
}

template <int KH, int NH, int NT3, int GROUP, bool FP16>
int launch_mlp_fwd_fmt(const SdfParams &P, cudaStream_t s) {
    const size_t smem = TcFwdShape<KH, NH, NT3>::bytes;
    auto k = sdf_mlp_fwd_kernel<KH, NH, NT3, GROUP, FP16>;
    static PersistentLaunch cfg;
    const int rc = persistent_setup(k, smem, kTcThreads, cfg, "sdf_mlp_fwd");
    if (rc != ANGELO_OK) return rc;
    // two CTAs per SM: their registers (2 x 512 x 64) and shared memory
    // (2 x 115 KB) fit, and each holds 256 of the SM's 512 tensor-memory
    // columns (the occupancy query answers 1 here); CTAs beyond what the SMs
    // hold run as a later wave of the persistent loop
    const int64_t tiles = (P.S + 127) / 128;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)cfg.sms * 2);
    k<<<grid, kTcThreads, smem, s>>>(P);
    return check_launch("sdf_mlp_fwd");
}

template <int KH, int NH, int NT3, int GROUP>
int launch_mlp_fwd(const SdfParams &P, cudaStream_t s) {
    return P.nl.operand_format == ANGELO_OPERAND_FP16 ? launch_mlp_fwd_fmt<KH, NH, NT3, GROUP, true>(P, s)
                                                      : launch_mlp_fwd_fmt<KH, NH, NT3, GROUP, false>(P, s);
}

template <int KH, int NH, int NT3, int GROUP>
int launch_mlp_bwd(const SdfParams &P, cudaStream_t s) {
    using Sh = TcBwdShape<KH, NH, NT3>;
    auto k = sdf_mlp_bwd_tc_kernel<KH, NH, NT3, GROUP>;
    static PersistentLaunch cfg;
    const int rc = persistent_setup(k, Sh::bytes, kTcThreads, cfg, "sdf_mlp_bwd");
    if (rc != ANGELO_OK) return rc;
    // each CTA holds Sh::tmem_cols of the SM's 512 tensor-memory columns
    const int per_sm = std::min(cfg.per_sm, (int)(512 / Sh::tmem_cols));
    const int64_t tiles = (P.S + 127) / 128;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)cfg.sms * per_sm);
    k<<<grid, kTcThreads, Sh::bytes, s>>>(P);
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
        if ((rc = launch_perm(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_encode<kCurv>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_mlp_fwd<KH, NH, NT3, kCurv>(P, s)) != ANGELO_OK) return rc;
    }
    return ANGELO_OK;
}

template <int KH, int NH, int NT3>
int run_bwd(const SdfParams &P, cudaStream_t s) {
    int rc;
    if (P.with_laplace) {
        // the curvature taps' MLP backward leaves dL/dshifted (with the hash
        // grid's positional derivative) for the FD pass; both groups' table
        // scatters then run as one launch
        if ((rc = launch_mlp_bwd<KH, NH, NT3, kCurv>(P, s)) != ANGELO_OK) return rc;
        if ((rc = launch_mlp_bwd<KH, NH, NT3, kFD>(P, s)) != ANGELO_OK) return rc;
#if ANGELO_SCATTER_MERGED
        return launch_scatter_both(P, s);
#else
        if ((rc = launch_scatter<kFD>(P, s)) != ANGELO_OK) return rc;
        return launch_scatter<kCurv>(P, s);
#endif
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
    // the curvature taps' Jacobians and the curvature pass's sample order
    // (int32 per sample + 8 counts per 256 samples)
    const int64_t j = (with_laplace && !backward)
                          ? 2 * 6 * 3 * (int64_t)lay->n_levels * n + n + 8 * perm_blocks(n)
                          : 0;
    return x + (backward ? kBState : kState) * n + j;
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
    ANGELO_REQUIRE(nl->mma_passes == 1 || nl->mma_passes == 3, "sdf_stencil_fwd: mma_passes %d (1 or 3)",
                   nl->mma_passes);
    ANGELO_REQUIRE(nl->operand_format == ANGELO_OPERAND_BF16 || nl->operand_format == ANGELO_OPERAND_FP16,
                   "sdf_stencil_fwd: operand_format %d", nl->operand_format);
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
    P.feat_vec4 = (feat_stride % 4 == 0) && (reinterpret_cast<uintptr_t>(feature) % 16 == 0);
    P.laplace = laplace;
    P.X = reinterpret_cast<float2 *>(workspace);
    P.state = workspace + 2 * n_evals(with_grad, with_laplace) * lay->n_levels * n;
    P.J = with_laplace ? reinterpret_cast<float2 *>(P.state + kState * n) : nullptr;
    if (with_laplace) set_perm(P, workspace, n, lay->n_levels);
    cudaStream_t s = as_stream(stream);
    if (shape_full(*nl)) return run_fwd<kFullKH, kFullNH, kFullNT3>(P, s);
    if (shape_small(*nl)) return run_fwd<kSmallKH, kSmallNH, kSmallNT3>(P, s);
    set_error("sdf_stencil_fwd: network shape not instantiated");
    return ANGELO_E_UNSUPPORTED;
}

namespace angelo {
int64_t mlp_tc_timeouts(int reset);        // fused_mlp.cu
int64_t radiance_tc_timeouts(int reset);   // fused_render.cu
}

extern "C" int64_t angelo_tc_timeouts(int32_t reset) {
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_timeouts, sizeof(v)) != cudaSuccess) return -1;
    if (reset) {
        const unsigned int z = 0;
        if (cudaMemcpyToSymbol(g_tc_timeouts, &z, sizeof(z)) != cudaSuccess) return -1;
    }
    const int64_t r = angelo::radiance_tc_timeouts(reset);
    const int64_t m = angelo::mlp_tc_timeouts(reset);
    return (r < 0 || m < 0) ? -1 : (int64_t)v + r + m;
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
    ANGELO_REQUIRE(nl->operand_format == ANGELO_OPERAND_BF16,
                   "sdf_stencil_bwd: the backward runs in bf16x3 and needs weights prepared with "
                   "operand_format bf16 (got %d)", nl->operand_format);
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
    P.J = with_laplace ? reinterpret_cast<float2 *>(P.state + kState * n) : nullptr;
    if (with_laplace) set_perm(P, const_cast<float *>(workspace), n, lay->n_levels);
    P.dX = reinterpret_cast<float2 *>(bwd_workspace);
    P.bstate = bwd_workspace + x;
    P.g_sdf = g_sdf;
    P.g_grad = g_grad;
    P.g_feature = g_feature;
    P.gfeat_stride = gfeat_stride;
    P.gfeat_vec4 = (gfeat_stride % 4 == 0) && (reinterpret_cast<uintptr_t>(g_feature) % 16 == 0);
    P.g_laplace = g_laplace;
    P.d_table = d_table;
    P.d_net = d_net;
    cudaStream_t s = as_stream(stream);
    if (shape_full(*nl)) return run_bwd<kFullKH, kFullNH, kFullNT3>(P, s);
    if (shape_small(*nl)) return run_bwd<kSmallKH, kSmallNH, kSmallNT3>(P, s);
    set_error("sdf_stencil_bwd: network shape not instantiated");
    return ANGELO_E_UNSUPPORTED;
}
