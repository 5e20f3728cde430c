// Degree-4 real spherical harmonics (the tcnn SphericalHarmonics encoding the
// reference reaches through get_encoding at models/texture.py:17,24-25).
// The constants are the real-SH normalisations sqrt((2l+1)/(4 pi)
// (l-|m|)!/(l+|m|)!) folded with the Legendre factors, in the sign convention
// of the Instant-NGP encoder.
#pragma once

namespace angelo {

// 1/(2 sqrt(pi)), sqrt(3)/(2 sqrt(pi)), sqrt(15)/(2 sqrt(pi)), sqrt(5)/(4 sqrt(pi)),
// sqrt(15)/(4 sqrt(pi)), sqrt(70)/(8 sqrt(pi)), sqrt(105)/(2 sqrt(pi)),
// sqrt(42)/(8 sqrt(pi)), sqrt(7)/(4 sqrt(pi)), sqrt(105)/(4 sqrt(pi))
constexpr float kSH0 = 0.28209479177387814f;
constexpr float kSH1 = 0.48860251190291987f;
constexpr float kSH2a = 1.0925484305920792f;
constexpr float kSH2b = 0.31539156525252005f;
constexpr float kSH2c = 0.54627421529603959f;
constexpr float kSH3a = 0.59004358992664352f;
constexpr float kSH3b = 2.8906114426405538f;
constexpr float kSH3c = 0.45704579946446572f;
constexpr float kSH3d = 0.3731763325901154f;
constexpr float kSH3e = 1.4453057213202769f;

__device__ __forceinline__ void sh4_eval(float x, float y, float z, float *o) {
    const float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
    o[0] = kSH0;
    o[1] = -kSH1 * y;
    o[2] = kSH1 * z;
    o[3] = -kSH1 * x;
    o[4] = kSH2a * xy;
    o[5] = -kSH2a * yz;
    o[6] = kSH2b * (3.0f * z2 - 1.0f);
    o[7] = -kSH2a * xz;
    o[8] = kSH2c * (x2 - y2);
    o[9] = kSH3a * y * (-3.0f * x2 + y2);
    o[10] = kSH3b * xy * z;
    o[11] = kSH3c * y * (1.0f - 5.0f * z2);
    o[12] = kSH3d * z * (5.0f * z2 - 3.0f);
    o[13] = kSH3c * x * (1.0f - 5.0f * z2);
    o[14] = kSH3e * z * (x2 - y2);
    o[15] = kSH3a * x * (-x2 + 3.0f * y2);
}

// d/dx, d/dy, d/dz of sum_k g_k * Y_k(x, y, z).
__device__ __forceinline__ void sh4_grad(float x, float y, float z, const float *g, float *d) {
    const float x2 = x * x, y2 = y * y, z2 = z * z;
    float dx = 0.f, dy = 0.f, dz = 0.f;
    dy += -kSH1 * g[1];
    dz += kSH1 * g[2];
    dx += -kSH1 * g[3];
    dx += kSH2a * y * g[4];
    dy += kSH2a * x * g[4];
    dy += -kSH2a * z * g[5];
    dz += -kSH2a * y * g[5];
    dz += kSH2b * 6.0f * z * g[6];
    dx += -kSH2a * z * g[7];
    dz += -kSH2a * x * g[7];
    dx += kSH2c * 2.0f * x * g[8];
    dy += -kSH2c * 2.0f * y * g[8];
    dx += kSH3a * y * (-6.0f * x) * g[9];
    dy += kSH3a * (-3.0f * x2 + 3.0f * y2) * g[9];
    dx += kSH3b * y * z * g[10];
    dy += kSH3b * x * z * g[10];
    dz += kSH3b * x * y * g[10];
    dy += kSH3c * (1.0f - 5.0f * z2) * g[11];
    dz += kSH3c * y * (-10.0f * z) * g[11];
    dz += kSH3d * (15.0f * z2 - 3.0f) * g[12];
    dx += kSH3c * (1.0f - 5.0f * z2) * g[13];
    dz += kSH3c * x * (-10.0f * z) * g[13];
    dx += kSH3e * z * 2.0f * x * g[14];
    dy += kSH3e * z * (-2.0f * y) * g[14];
    dz += kSH3e * (x2 - y2) * g[14];
    dx += kSH3a * (-3.0f * x2 + 3.0f * y2) * g[15];
    dy += kSH3a * x * 6.0f * y * g[15];
    d[0] = dx;
    d[1] = dy;
    d[2] = dz;
}

// Input mapping of the reference: v01 = (d + 1)/2 (models/texture.py:24),
// then the encoder's v01*2 - 1.
__device__ __forceinline__ float sh_in(float v, int from_unit) {
    if (from_unit) v = __fdiv_rn(__fadd_rn(v, 1.0f), 2.0f);
    return __fsub_rn(__fmul_rn(v, 2.0f), 1.0f);
}

}  // namespace angelo
