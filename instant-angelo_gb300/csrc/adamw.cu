// AdamW step of the reference's optimizer (systems/utils.py:314-325 builds
// torch.optim.AdamW(lr, betas, eps) per parameter group) as one streaming
// pass per parameter tensor: read param, grad, first and second moment, write
// param and both moments (28 bytes per fp32 parameter, HBM-bound).
//
// The update is decoupled weight decay followed by the Adam step (Loshchilov
// and Hutter, "Decoupled Weight Decay Regularization", algorithm 2):
//   p   <- p - lr * wd * p
//   m   <- m + (1 - beta1) (g - m)          (= beta1 m + (1 - beta1) g)
//   v   <- beta2 v + (1 - beta2) g^2
//   p   <- p - (lr / bc1) * m / (sqrt(v) / sqrt(bc2) + eps)
// with bc1 = 1 - beta1^t, bc2 = 1 - beta2^t computed on the host per step.
// The first moment uses the interpolation form of torch.optim.AdamW's
// default CUDA path (foreach lerp); all arithmetic is fp32.
#include <algorithm>

#include "common.cuh"

using namespace angelo;

namespace {

struct AdamArgs {
    float lr, beta1, beta2, eps, wd;
    float step_size;       // lr / bc1
    float bc2_sqrt;        // sqrt(bc2)
};

__device__ __forceinline__ void adamw_one(float &p, float g, float &m, float &v, const AdamArgs &a) {
    p = p - a.lr * a.wd * p;
    m = m + (1.0f - a.beta1) * (g - m);
    v = a.beta2 * v + (1.0f - a.beta2) * g * g;
    const float denom = sqrtf(v) / a.bc2_sqrt + a.eps;
    p = p - a.step_size * m / denom;
}

__global__ void adamw_vec4_kernel(float4 *__restrict__ p, const float4 *__restrict__ g,
                                  float4 *__restrict__ m, float4 *__restrict__ v, int64_t n4,
                                  AdamArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 pp = p[i], mm = m[i], vv = v[i];
        const float4 gg = __ldcs(g + i);
        adamw_one(pp.x, gg.x, mm.x, vv.x, a);
        adamw_one(pp.y, gg.y, mm.y, vv.y, a);
        adamw_one(pp.z, gg.z, mm.z, vv.z, a);
        adamw_one(pp.w, gg.w, mm.w, vv.w, a);
        p[i] = pp;
        m[i] = mm;
        v[i] = vv;
    }
}

__global__ void adamw_scalar_kernel(float *__restrict__ p, const float *__restrict__ g,
                                    float *__restrict__ m, float *__restrict__ v, int64_t n,
                                    AdamArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float pp = p[i], mm = m[i], vv = v[i];
        adamw_one(pp, g[i], mm, vv, a);
        p[i] = pp;
        m[i] = mm;
        v[i] = vv;
    }
}

bool aligned16(const void *x) { return (reinterpret_cast<uintptr_t>(x) & 15) == 0; }

// Many small tensors in one launch: block b of the grid takes chunk
// b - blk0[k] (kMultiChunk elements) of tensor k, each tensor with its own
// hyper-parameters; the per-element update is adamw_one, as above.
constexpr int kMultiMax = 32, kMultiChunk = 2048;

struct MultiAdam {
    int n;
    int64_t blk0[kMultiMax + 1];
    float *p[kMultiMax];
    const float *g[kMultiMax];
    float *m[kMultiMax];
    float *v[kMultiMax];
    int64_t size[kMultiMax];
    AdamArgs a[kMultiMax];
};

__global__ void adamw_multi_kernel(const __grid_constant__ MultiAdam M) {
    int k = 0;
    for (int i = 1; i < M.n; ++i)
        if ((int64_t)blockIdx.x >= M.blk0[i]) k = i;
    const int64_t base = ((int64_t)blockIdx.x - M.blk0[k]) * kMultiChunk;
    const int64_t end = base + kMultiChunk < M.size[k] ? base + kMultiChunk : M.size[k];
    const AdamArgs a = M.a[k];
    for (int64_t i = base + threadIdx.x; i < end; i += blockDim.x) {
        float pp = M.p[k][i], mm = M.m[k][i], vv = M.v[k][i];
        adamw_one(pp, M.g[k][i], mm, vv, a);
        M.p[k][i] = pp;
        M.m[k][i] = mm;
        M.v[k][i] = vv;
    }
}

}  // namespace

extern "C" int angelo_adamw_step(float *param, const float *grad, float *exp_avg, float *exp_avg_sq,
                                 int64_t n, float lr, float beta1, float beta2, float eps,
                                 float weight_decay, float bias_correction1,
                                 float bias_correction2, void *stream) {
    ANGELO_REQUIRE(n >= 0, "adamw_step: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(param && grad && exp_avg && exp_avg_sq, "adamw_step: null pointer");
    ANGELO_REQUIRE(bias_correction1 > 0.f && bias_correction2 > 0.f, "adamw_step: bias corrections");
    AdamArgs a;
    a.lr = lr;
    a.beta1 = beta1;
    a.beta2 = beta2;
    a.eps = eps;
    a.wd = weight_decay;
    a.step_size = lr / bias_correction1;
    a.bc2_sqrt = sqrtf(bias_correction2);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s = as_stream(stream);
    const int threads = 256;
    const int64_t cap = (int64_t)std::max(sms, 1) * 8;   // 8 CTAs of 256 per SM, grid-stride
    int64_t head = 0;
    if (aligned16(param) && aligned16(grad) && aligned16(exp_avg) && aligned16(exp_avg_sq)) {
        const int64_t n4 = n / 4;
        if (n4 > 0) {
            const int64_t blocks = std::min<int64_t>((n4 + threads - 1) / threads, cap);
            adamw_vec4_kernel<<<(unsigned)blocks, threads, 0, s>>>(
                reinterpret_cast<float4 *>(param), reinterpret_cast<const float4 *>(grad),
                reinterpret_cast<float4 *>(exp_avg), reinterpret_cast<float4 *>(exp_avg_sq), n4, a);
        }
        head = n4 * 4;
    }
    if (head < n) {
        const int64_t rest = n - head;
        const int64_t blocks = std::min<int64_t>((rest + threads - 1) / threads, cap);
        adamw_scalar_kernel<<<(unsigned)blocks, threads, 0, s>>>(param + head, grad + head, exp_avg + head,
                                                                exp_avg_sq + head, rest, a);
    }
    return check_launch("adamw_step");
}

extern "C" int angelo_adamw_step_multi(int32_t n_tensors, float *const *params, const float *const *grads,
                                       float *const *exp_avg, float *const *exp_avg_sq, const int64_t *sizes,
                                       const float *lr, const float *beta1, const float *beta2, const float *eps,
                                       const float *weight_decay, const float *bias_correction1,
                                       const float *bias_correction2, void *stream) {
    ANGELO_REQUIRE(n_tensors >= 0, "adamw_step_multi: negative count");
    if (n_tensors == 0) return ANGELO_OK;
    ANGELO_REQUIRE(params && grads && exp_avg && exp_avg_sq && sizes && lr && beta1 && beta2 && eps &&
                       weight_decay && bias_correction1 && bias_correction2,
                   "adamw_step_multi: null array");
    cudaStream_t s = as_stream(stream);
    for (int32_t t0 = 0; t0 < n_tensors; t0 += kMultiMax) {
        MultiAdam M{};
        M.n = 0;
        int64_t blocks = 0;
        for (int32_t t = t0; t < n_tensors && t < t0 + kMultiMax; ++t) {
            ANGELO_REQUIRE(sizes[t] >= 0, "adamw_step_multi: tensor %d has negative size", t);
            if (sizes[t] == 0) continue;
            ANGELO_REQUIRE(params[t] && grads[t] && exp_avg[t] && exp_avg_sq[t],
                           "adamw_step_multi: tensor %d has a null pointer", t);
            ANGELO_REQUIRE(bias_correction1[t] > 0.f && bias_correction2[t] > 0.f,
                           "adamw_step_multi: tensor %d bias corrections", t);
            const int k = M.n++;
            M.blk0[k] = blocks;
            blocks += (sizes[t] + kMultiChunk - 1) / kMultiChunk;
            M.p[k] = params[t];
            M.g[k] = grads[t];
            M.m[k] = exp_avg[t];
            M.v[k] = exp_avg_sq[t];
            M.size[k] = sizes[t];
            AdamArgs &a = M.a[k];
            a.lr = lr[t];
            a.beta1 = beta1[t];
            a.beta2 = beta2[t];
            a.eps = eps[t];
            a.wd = weight_decay[t];
            a.step_size = lr[t] / bias_correction1[t];
            a.bc2_sqrt = sqrtf(bias_correction2[t]);
        }
        if (M.n == 0) continue;
        M.blk0[M.n] = blocks;
        ANGELO_REQUIRE(blocks < (1ll << 31), "adamw_step_multi: %lld blocks", (long long)blocks);
        adamw_multi_kernel<<<(unsigned)blocks, 256, 0, s>>>(M);
        if (int rc = check_launch("adamw_step_multi")) return rc;
    }
    return ANGELO_OK;
}
