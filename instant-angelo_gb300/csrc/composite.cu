// Plain compositing kernels: transmittance weights from alpha and
// accumulation along rays (nerfacc 0.3.3 render_weight_from_alpha and
// accumulate_along_rays at models/neus.py:234-240).  One thread per ray walks
// the ray's samples in order, so the float32 sums are deterministic.
#include "common.cuh"

using namespace angelo;

namespace {

__global__ void weights_fwd_kernel(const float *__restrict__ alpha, const int64_t *__restrict__ off,
                                   int64_t n_rays, float eps, float *__restrict__ w,
                                   float *__restrict__ trans) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float T = 1.0f;
    bool stopped = false;
    for (int64_t j = off[r]; j < off[r + 1]; ++j) {
        if (T < eps) stopped = true;
        if (trans) trans[j] = T;
        if (stopped) {
            w[j] = 0.0f;
            continue;
        }
        const float a = alpha[j];
        w[j] = __fmul_rn(a, T);
        T = __fmul_rn(T, __fsub_rn(1.0f, a));
    }
}

// w_j = a_j T_j m_j with T_j = prod_{k<j}(1-a_k), m_j = [T_j >= eps].
// dL/da_j = T_j (g_j m_j - R_j), R_j = sum_{k>j} g_k m_k a_k prod_{j<i<k}(1-a_i),
// evaluated back to front: R_{j-1} = g_j m_j a_j + (1-a_j) R_j.  T_j is the
// transmittance saved by the forward pass.
__global__ void weights_bwd_kernel(const float *__restrict__ alpha, const float *__restrict__ trans,
                                   const int64_t *__restrict__ off, int64_t n_rays, float eps,
                                   const float *__restrict__ gw, float *__restrict__ ga) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float R = 0.0f;
    for (int64_t j = off[r + 1] - 1; j >= off[r]; --j) {
        const float a = alpha[j], T = trans[j];
        const float g = T >= eps ? gw[j] : 0.0f;
        ga[j] = T * (g - R);
        R = g * a + (1.0f - a) * R;
    }
}

__global__ void accumulate_fwd_kernel(const float *__restrict__ w, const float *__restrict__ v,
                                      int C, const int64_t *__restrict__ off, int64_t n_rays,
                                      float *__restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int64_t j = off[r]; j < off[r + 1]; ++j) {
        const float wj = w[j];
        if (v == nullptr) {
            acc[0] += wj;
        } else {
            for (int c = 0; c < C; ++c) acc[c] += wj * v[j * C + c];
        }
    }
    for (int c = 0; c < C; ++c) out[r * C + c] = acc[c];
}

__global__ void accumulate_bwd_kernel(const float *__restrict__ w, const float *__restrict__ v,
                                      int C, const int64_t *__restrict__ off, int64_t n_rays,
                                      const float *__restrict__ dout, float *__restrict__ dw,
                                      float *__restrict__ dv) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float g[4];
    for (int c = 0; c < C; ++c) g[c] = dout[r * C + c];
    for (int64_t j = off[r]; j < off[r + 1]; ++j) {
        if (v == nullptr) {
            dw[j] = g[0];
        } else {
            float s = 0.f;
            for (int c = 0; c < C; ++c) {
                s += g[c] * v[j * C + c];
                if (dv) dv[j * C + c] = w[j] * g[c];
            }
            dw[j] = s;
        }
    }
}

// nerfacc 0.3.3 render_weight_from_density (the learned background,
// models/neus.py:171): per ray in sample order, with tau_j = sigma_j (t1_j -
// t0_j), w_j = (1 - e^-tau_j) e^-(tau_0 + .. + tau_{j-1}).
__global__ void density_weights_fwd_kernel(const float *__restrict__ t0, const float *__restrict__ t1,
                                           const float *__restrict__ sigma, const int64_t *__restrict__ off,
                                           int64_t n_rays, float *__restrict__ w) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float depth = 0.0f;
    for (int64_t j = off[r]; j < off[r + 1]; ++j) {
        const float tau = __fmul_rn(sigma[j], __fsub_rn(t1[j], t0[j]));
        w[j] = __fmul_rn(__fsub_rn(1.0f, expf(-tau)), expf(-depth));
        depth = __fadd_rn(depth, tau);
    }
}

// dL/dsigma_j = dt_j (g_j e^-(tau_0 + .. + tau_j) - sum_{k>j} g_k w_k),
// the suffix sum taken back to front.
__global__ void density_weights_bwd_kernel(const float *__restrict__ t0, const float *__restrict__ t1,
                                           const float *__restrict__ sigma, const float *__restrict__ w,
                                           const int64_t *__restrict__ off, int64_t n_rays,
                                           const float *__restrict__ gw, float *__restrict__ gs) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float total = 0.0f;
    for (int64_t j = off[r]; j < off[r + 1]; ++j) total += sigma[j] * (t1[j] - t0[j]);
    float after = 0.0f;   // sum_{k>j} g_k w_k
    float depth = total;  // tau_0 + .. + tau_j, walking back
    for (int64_t j = off[r + 1] - 1; j >= off[r]; --j) {
        const float dt = t1[j] - t0[j];
        gs[j] = dt * (gw[j] * expf(-depth) - after);
        after += gw[j] * w[j];
        depth -= sigma[j] * dt;
    }
}

}  // namespace

extern "C" int angelo_density_weights_fwd(const float *t_starts, const float *t_ends, const float *sigmas,
                                          const int64_t *offsets, int64_t n_rays, float *weights,
                                          void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "density_weights_fwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(t_starts && t_ends && sigmas && offsets && weights, "density_weights_fwd: null pointer");
    density_weights_fwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        t_starts, t_ends, sigmas, offsets, n_rays, weights);
    return check_launch("density_weights_fwd");
}

extern "C" int angelo_density_weights_bwd(const float *t_starts, const float *t_ends, const float *sigmas,
                                          const float *weights, const int64_t *offsets, int64_t n_rays,
                                          const float *dweights, float *dsigmas, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "density_weights_bwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(t_starts && t_ends && sigmas && weights && offsets && dweights && dsigmas,
                   "density_weights_bwd: null pointer");
    density_weights_bwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        t_starts, t_ends, sigmas, weights, offsets, n_rays, dweights, dsigmas);
    return check_launch("density_weights_bwd");
}

extern "C" int angelo_weights_fwd(const float *alpha, const int64_t *offsets, int64_t n_rays,
                                  float early_stop_eps, float *weights, float *trans,
                                  void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "weights_fwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(alpha && offsets && weights, "weights_fwd: null pointer");
    weights_fwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        alpha, offsets, n_rays, early_stop_eps, weights, trans);
    return check_launch("weights_fwd");
}

extern "C" int angelo_weights_bwd(const float *alpha, const float *trans, const int64_t *offsets,
                                  int64_t n_rays, float early_stop_eps, const float *dweights,
                                  float *dalpha, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0, "weights_bwd: negative n_rays");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(alpha && trans && offsets && dweights && dalpha, "weights_bwd: null pointer");
    weights_bwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        alpha, trans, offsets, n_rays, early_stop_eps, dweights, dalpha);
    return check_launch("weights_bwd");
}

extern "C" int angelo_accumulate_fwd(const float *weights, const float *values, int32_t channels,
                                     const int64_t *offsets, int64_t n_rays, float *out,
                                     void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && channels >= 1 && channels <= 4, "accumulate_fwd: bad sizes");
    ANGELO_REQUIRE(values != nullptr || channels == 1, "accumulate_fwd: channels without values");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(weights && offsets && out, "accumulate_fwd: null pointer");
    accumulate_fwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        weights, values, channels, offsets, n_rays, out);
    return check_launch("accumulate_fwd");
}

extern "C" int angelo_accumulate_bwd(const float *weights, const float *values, int32_t channels,
                                     const int64_t *offsets, int64_t n_rays, const float *dout,
                                     float *dweights, float *dvalues, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && channels >= 1 && channels <= 4, "accumulate_bwd: bad sizes");
    ANGELO_REQUIRE(values != nullptr || channels == 1, "accumulate_bwd: channels without values");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(weights && offsets && dout && dweights, "accumulate_bwd: null pointer");
    accumulate_bwd_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        weights, values, channels, offsets, n_rays, dout, dweights, dvalues);
    return check_launch("accumulate_bwd");
}
