// Degree-4 real spherical harmonics of a direction (the tcnn
// SphericalHarmonics encoding reached through get_encoding at
// models/texture.py:17,24-25).  The constants are the real-SH normalisations
// sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!) folded with the Legendre factors, in
// the sign convention of the Instant-NGP encoder.
#include "common.cuh"

using namespace angelo;

#include "sh.cuh"

namespace {

__global__ void sh4_fwd_kernel(const float *__restrict__ dirs, int64_t n, int from_unit,
                               float *__restrict__ out, int64_t stride, int64_t col) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float o[16];
    sh4_eval(sh_in(dirs[i * 3], from_unit), sh_in(dirs[i * 3 + 1], from_unit),
             sh_in(dirs[i * 3 + 2], from_unit), o);
    float *dst = out + i * stride + col;
#pragma unroll
    for (int k = 0; k < 16; ++k) dst[k] = o[k];
}

__global__ void sh4_bwd_kernel(const float *__restrict__ dirs, int64_t n, int from_unit,
                               const float *__restrict__ dout, int64_t stride, int64_t col,
                               float *__restrict__ ddirs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) g[k] = dout[i * stride + col + k];
    float d[3];
    sh4_grad(sh_in(dirs[i * 3], from_unit), sh_in(dirs[i * 3 + 1], from_unit),
             sh_in(dirs[i * 3 + 2], from_unit), g, d);
    // chain rule through v*2-1 (and (d+1)/2 when from_unit): factor 2 or 1
    const float f = from_unit ? 1.0f : 2.0f;
    ddirs[i * 3 + 0] = d[0] * f;
    ddirs[i * 3 + 1] = d[1] * f;
    ddirs[i * 3 + 2] = d[2] * f;
}

}  // namespace

extern "C" int angelo_sh4_fwd(const float *dirs, int64_t n, int32_t from_unit, float *out,
                              int64_t out_stride, int64_t out_col, void *stream) {
    ANGELO_REQUIRE(n >= 0, "sh4_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(dirs && out && out_stride >= out_col + 16, "sh4_fwd: bad arguments");
    sh4_fwd_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(dirs, n, from_unit, out,
                                                                     out_stride, out_col);
    return check_launch("sh4_fwd");
}

extern "C" int angelo_sh4_bwd(const float *dirs, int64_t n, int32_t from_unit, const float *dout,
                              int64_t dout_stride, int64_t dout_col, float *ddirs, void *stream) {
    ANGELO_REQUIRE(n >= 0, "sh4_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(dirs && dout && ddirs && dout_stride >= dout_col + 16, "sh4_bwd: bad arguments");
    sh4_bwd_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(dirs, n, from_unit, dout,
                                                                     dout_stride, dout_col, ddirs);
    return check_launch("sh4_bwd");
}
