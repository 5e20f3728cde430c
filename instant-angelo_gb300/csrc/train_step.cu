// The small per-step work around the fused NeuS kernels, each in one launch
// instead of a chain of elementwise kernels:
//
// * weight normalisation of the geometry MLP's layers (nn.utils.weight_norm,
//   dim 0, applied in VanillaMLP.make_linear, models/network_utils.py:132-133):
//   W = g * v / ||v||_row, and its backward
//     dg = (dW . v) / n,   dv = (g / n) dW - (g (dW . v) / n^3) v,   n = ||v||_row
//   for every layer at once (one warp per output row);
// * the training loss the step seeds (systems/neus.py:130-159): the rgb MSE
//   over the valid rays, the eikonal term mean((||grad|| - 1)^2) and the
//   curvature term mean(|laplace|), weighted and summed, with the gradients
//   of the total:
//     d rgb_c   = w_rgb 2 (c - t) valid / (3 n_valid)
//     d grad    = w_eik 2 (||g|| - 1) / S * g / ||g||    (0 where ||g|| = 0)
//     d laplace = w_curv sign(laplace) / S
//   The sums are reduced in a fixed order (block partials, then the last
//   block adds them in double), so the loss does not change between runs.
#include <math.h>

#include "common.cuh"

using namespace angelo;

namespace {

constexpr int kMaxWnLayers = 8;

struct WnLayers {
    int n;
    int row0[kMaxWnLayers + 1];   // first global row of each layer
    int cols[kMaxWnLayers];
    const float *v[kMaxWnLayers];
    const float *g[kMaxWnLayers];
    float *w[kMaxWnLayers];      // forward output
    const float *dw[kMaxWnLayers];
    float *dv[kMaxWnLayers];
    float *dg[kMaxWnLayers];
};

__device__ __forceinline__ int wn_layer(const WnLayers &L, int row) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < kMaxWnLayers; ++i)
        if (i < L.n && row >= L.row0[i]) k = i;
    return k;
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(0xffffffffu, x, d);
    return x;
}

__global__ void weight_norm_fwd_kernel(const WnLayers L) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (row >= L.row0[L.n]) return;
    const int k = wn_layer(L, row), r = row - L.row0[k], C = L.cols[k];
    const float *v = L.v[k] + (int64_t)r * C;
    float ss = 0.f;
    for (int c = lane; c < C; c += 32) ss = fmaf(v[c], v[c], ss);
    const float n = sqrtf(warp_sum(ss));
    const float g = L.g[k][r];
    float *w = L.w[k] + (int64_t)r * C;
    for (int c = lane; c < C; c += 32) w[c] = g * v[c] / n;
}

__global__ void weight_norm_bwd_kernel(const WnLayers L) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (row >= L.row0[L.n]) return;
    const int k = wn_layer(L, row), r = row - L.row0[k], C = L.cols[k];
    const float *v = L.v[k] + (int64_t)r * C;
    const float *dw = L.dw[k] + (int64_t)r * C;
    float ss = 0.f, dot = 0.f;
    for (int c = lane; c < C; c += 32) {
        ss = fmaf(v[c], v[c], ss);
        dot = fmaf(dw[c], v[c], dot);
    }
    const float n = sqrtf(warp_sum(ss));
    dot = warp_sum(dot);
    const float g = L.g[k][r];
    if (lane == 0) L.dg[k][r] = dot / n;
    const float a = g / n, b = g * dot / (n * n * n);
    float *dv = L.dv[k] + (int64_t)r * C;
    for (int c = lane; c < C; c += 32) dv[c] = a * dw[c] - b * v[c];
}

int wn_pack(int32_t n_layers, const int32_t *rows, const int32_t *cols, WnLayers &L) {
    ANGELO_REQUIRE(n_layers >= 1 && n_layers <= kMaxWnLayers, "weight_norm: %d layers (1..%d)", n_layers,
                   kMaxWnLayers);
    ANGELO_REQUIRE(rows && cols, "weight_norm: null shape arrays");
    L = WnLayers{};
    L.n = n_layers;
    L.row0[0] = 0;
    for (int i = 0; i < n_layers; ++i) {
        ANGELO_REQUIRE(rows[i] >= 1 && cols[i] >= 1, "weight_norm: layer %d is %d x %d", i, rows[i], cols[i]);
        L.row0[i + 1] = L.row0[i] + rows[i];
        L.cols[i] = cols[i];
    }
    return ANGELO_OK;
}

// ------------------------------------------------------------------- loss

constexpr int kLossThreads = 256;
constexpr int kLossBlocksMax = 1024;

struct LossArgs {
    const float *rgb_pred, *rgb_true;   // (R, 3)
    const uint8_t *valid;               // (R,) bool
    int64_t R;
    const float *grad;                  // (S, 3)
    const float *lap;                   // (S,) or null
    int64_t S;
    float w_rgb, w_eik, w_curv;
    double *partials;                   // [blocks][4]
    unsigned *counter;
    float *out;                         // total, rgb_mse, eikonal, curvature, n_valid
};

__device__ __forceinline__ float block_sum(float x, float *sh) {
    x = warp_sum(x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = x;
    __syncthreads();
    float t = 0.f;
    if (warp == 0) {
        t = lane < kLossThreads / 32 ? sh[lane] : 0.f;
        t = warp_sum(t);
    }
    return t;   // valid in thread 0
}

__global__ void __launch_bounds__(kLossThreads) loss_fwd_kernel(const LossArgs A) {
    __shared__ float sh[kLossThreads / 32];
    __shared__ bool last;
    float se = 0.f, nv = 0.f, eik = 0.f, curv = 0.f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.R; i += stride) {
        if (A.valid[i]) {
            nv += 1.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float d = A.rgb_pred[i * 3 + c] - A.rgb_true[i * 3 + c];
                se = fmaf(d, d, se);
            }
        }
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.S; i += stride) {
        const float gx = A.grad[i * 3], gy = A.grad[i * 3 + 1], gz = A.grad[i * 3 + 2];
        const float e = sqrtf(gx * gx + gy * gy + gz * gz) - 1.f;
        eik = fmaf(e, e, eik);
        if (A.lap) curv += fabsf(A.lap[i]);
    }
    const float s0 = block_sum(se, sh), s1 = block_sum(nv, sh), s2 = block_sum(eik, sh), s3 = block_sum(curv, sh);
    if (threadIdx.x == 0) {
        double *p = A.partials + (int64_t)blockIdx.x * 4;
        p[0] = s0;
        p[1] = s1;
        p[2] = s2;
        p[3] = s3;
        __threadfence();
        last = atomicAdd(A.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: each thread adds a fixed stride of the partials, then
    // a fixed tree over the threads (the same order on every run)
    __shared__ double shd[kLossThreads / 32][4];
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const double *p = A.partials + (int64_t)b * 4;
#pragma unroll
        for (int q = 0; q < 4; ++q) t[q] += __ldcg(p + q);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) t[q] += __shfl_xor_sync(0xffffffffu, t[q], d);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) shd[warp][q] = t[q];
    __syncthreads();
    if (threadIdx.x != 0) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        t[q] = 0.0;
        for (int w = 0; w < kLossThreads / 32; ++w) t[q] += shd[w][q];
    }
    const float l_rgb = (float)(t[0] / (t[1] * 3.0));   // 0 / 0 = NaN without valid rays
    const float l_eik = A.S > 0 ? (float)(t[2] / (double)A.S) : NAN;
    const float l_curv = A.lap ? (A.S > 0 ? (float)(t[3] / (double)A.S) : NAN) : 0.f;
    float total = A.w_rgb * l_rgb + A.w_eik * l_eik;
    if (A.lap && A.w_curv > 0.f) total += A.w_curv * l_curv;
    A.out[0] = total;
    A.out[1] = l_rgb;
    A.out[2] = l_eik;
    A.out[3] = l_curv;
    A.out[4] = (float)t[1];
    *A.counter = 0u;   // ready for the next launch on this stream
}

struct LossBwdArgs {
    const float *rgb_pred, *rgb_true;
    const uint8_t *valid;
    int64_t R;
    const float *grad, *lap;
    int64_t S;
    float w_rgb, w_eik, w_curv;
    const float *stats;    // the forward's out (n_valid at [4])
    const float *d_total;  // dL/dtotal (device scalar)
    float *d_rgb, *d_grad, *d_lap;
};

__global__ void __launch_bounds__(kLossThreads) loss_bwd_kernel(const LossBwdArgs A) {
    const float dt = *A.d_total;
    const float crgb = dt * A.w_rgb * 2.f / (3.f * A.stats[4]);
    const float ceik = A.S > 0 ? dt * A.w_eik * 2.f / (float)A.S : 0.f;
    const float ccurv = A.S > 0 ? dt * A.w_curv / (float)A.S : 0.f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.R; i += stride) {
        const bool v = A.valid[i] != 0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            A.d_rgb[i * 3 + c] = v ? crgb * (A.rgb_pred[i * 3 + c] - A.rgb_true[i * 3 + c]) : 0.f;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.S; i += stride) {
        const float gx = A.grad[i * 3], gy = A.grad[i * 3 + 1], gz = A.grad[i * 3 + 2];
        const float n = sqrtf(gx * gx + gy * gy + gz * gz);
        const float k = n > 0.f ? ceik * (n - 1.f) / n : 0.f;
        A.d_grad[i * 3] = k * gx;
        A.d_grad[i * 3 + 1] = k * gy;
        A.d_grad[i * 3 + 2] = k * gz;
        if (A.d_lap) {
            const float l = A.lap[i];
            A.d_lap[i] = l > 0.f ? ccurv : (l < 0.f ? -ccurv : 0.f);
        }
    }
}

unsigned loss_blocks(int64_t n) {
    const int64_t b = (n + kLossThreads - 1) / kLossThreads;
    return (unsigned)(b < 1 ? 1 : (b > kLossBlocksMax ? kLossBlocksMax : b));
}

}  // namespace

extern "C" int angelo_weight_norm_fwd(int32_t n_layers, const int32_t *rows, const int32_t *cols,
                                      const float *const *v, const float *const *g, float *const *w,
                                      void *stream) {
    WnLayers L;
    if (int rc = wn_pack(n_layers, rows, cols, L)) return rc;
    ANGELO_REQUIRE(v && g && w, "weight_norm_fwd: null pointer arrays");
    for (int i = 0; i < n_layers; ++i) {
        ANGELO_REQUIRE(v[i] && g[i] && w[i], "weight_norm_fwd: layer %d has a null tensor", i);
        L.v[i] = v[i];
        L.g[i] = g[i];
        L.w[i] = w[i];
    }
    const int warps = 8;
    weight_norm_fwd_kernel<<<blocks_for(L.row0[n_layers], warps), 32 * warps, 0, as_stream(stream)>>>(L);
    return check_launch("weight_norm_fwd");
}

extern "C" int angelo_weight_norm_bwd(int32_t n_layers, const int32_t *rows, const int32_t *cols,
                                      const float *const *v, const float *const *g, const float *const *dw,
                                      float *const *dv, float *const *dg, void *stream) {
    WnLayers L;
    if (int rc = wn_pack(n_layers, rows, cols, L)) return rc;
    ANGELO_REQUIRE(v && g && dw && dv && dg, "weight_norm_bwd: null pointer arrays");
    for (int i = 0; i < n_layers; ++i) {
        ANGELO_REQUIRE(v[i] && g[i] && dw[i] && dv[i] && dg[i], "weight_norm_bwd: layer %d has a null tensor", i);
        L.v[i] = v[i];
        L.g[i] = g[i];
        L.dw[i] = dw[i];
        L.dv[i] = dv[i];
        L.dg[i] = dg[i];
    }
    const int warps = 8;
    weight_norm_bwd_kernel<<<blocks_for(L.row0[n_layers], warps), 32 * warps, 0, as_stream(stream)>>>(L);
    return check_launch("weight_norm_bwd");
}

extern "C" int64_t angelo_loss_workspace_size(void) {
    return (int64_t)kLossBlocksMax * 4 * 8 + 256;
}

extern "C" int angelo_neus_loss_fwd(const float *rgb_pred, const float *rgb_true, const uint8_t *valid, int64_t n_rays,
                                    const float *sdf_grad, const float *laplace, int64_t n_samples, float w_rgb,
                                    float w_eikonal, float w_curvature, void *workspace, float *out, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && n_samples >= 0, "neus_loss_fwd: negative sizes");
    ANGELO_REQUIRE(workspace && out, "neus_loss_fwd: null workspace or output");
    ANGELO_REQUIRE(n_rays == 0 || (rgb_pred && rgb_true && valid), "neus_loss_fwd: null ray tensors");
    ANGELO_REQUIRE(n_samples == 0 || sdf_grad, "neus_loss_fwd: null sdf_grad");
    LossArgs A;
    A.rgb_pred = rgb_pred;
    A.rgb_true = rgb_true;
    A.valid = valid;
    A.R = n_rays;
    A.grad = sdf_grad;
    A.lap = laplace;
    A.S = n_samples;
    A.w_rgb = w_rgb;
    A.w_eik = w_eikonal;
    A.w_curv = w_curvature;
    A.counter = reinterpret_cast<unsigned *>(workspace);
    A.partials = reinterpret_cast<double *>(reinterpret_cast<char *>(workspace) + 256);
    A.out = out;
    loss_fwd_kernel<<<loss_blocks(n_rays > n_samples ? n_rays : n_samples), kLossThreads, 0, as_stream(stream)>>>(A);
    return check_launch("neus_loss_fwd");
}

extern "C" int angelo_neus_loss_bwd(const float *rgb_pred, const float *rgb_true, const uint8_t *valid,
                                    int64_t n_rays, const float *sdf_grad, const float *laplace, int64_t n_samples,
                                    float w_rgb, float w_eikonal, float w_curvature, const float *stats,
                                    const float *d_total, float *d_rgb, float *d_grad, float *d_laplace,
                                    void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && n_samples >= 0, "neus_loss_bwd: negative sizes");
    ANGELO_REQUIRE(stats && d_total, "neus_loss_bwd: null stats or d_total");
    ANGELO_REQUIRE(n_rays == 0 || (rgb_pred && rgb_true && valid && d_rgb), "neus_loss_bwd: null ray tensors");
    ANGELO_REQUIRE(n_samples == 0 || (sdf_grad && d_grad), "neus_loss_bwd: null sample tensors");
    ANGELO_REQUIRE(!d_laplace || laplace, "neus_loss_bwd: d_laplace without laplace");
    LossBwdArgs A;
    A.rgb_pred = rgb_pred;
    A.rgb_true = rgb_true;
    A.valid = valid;
    A.R = n_rays;
    A.grad = sdf_grad;
    A.lap = laplace;
    A.S = n_samples;
    A.w_rgb = w_rgb;
    A.w_eik = w_eikonal;
    A.w_curv = w_curvature;
    A.stats = stats;
    A.d_total = d_total;
    A.d_rgb = d_rgb;
    A.d_grad = d_grad;
    A.d_lap = d_laplace;
    const int64_t n = n_rays > n_samples ? n_rays : n_samples;
    if (n == 0) return ANGELO_OK;
    loss_bwd_kernel<<<loss_blocks(n), kLossThreads, 0, as_stream(stream)>>>(A);
    return check_launch("neus_loss_bwd");
}
