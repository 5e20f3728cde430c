/*
 * oracle.c -- CPU restatement of the third-party arithmetic on the NeuS /
 * Neuralangelo hot path of Instant-angelo.  TEST INFRASTRUCTURE ONLY: nothing
 * in the product library links, loads or calls this file; the tests, the
 * smoke check and the CPU-baseline leg of bench.py use it as the checker.
 *
 * The reference reaches this arithmetic through two packages that are not
 * vendored in the reference tree:
 *   - tiny-cuda-nn (unpinned, installed from git HEAD: README.md:26,
 *     docker/dockerfile:26), used as tcnn.Encoding(otype=HashGrid) at
 *     models/network_utils.py:47 and otype=SphericalHarmonics at
 *     models/network_utils.py:91 (called from models/texture.py:17).
 *   - nerfacc==0.3.3 (requirements.txt:3), used at models/neus.py:11-12,
 *     63-68, 109, 210-220, 234-240.
 * Both are restated here from their published algorithms (the Instant-NGP
 * paper, Mueller et al. 2022, App. A; nerfacc 0.3 documentation).  Every
 * assumption about their exact float sequencing is listed in
 * oracle/ASSUMPTIONS.md.  The functions use IEEE float32 with no FP
 * contraction except where an explicit fmaf() is written (the Makefile
 * passes -ffp-contract=off), so that integer outputs (hash indices, cell
 * indices, per-ray counts, offsets) and the float32 encode are reproducible
 * bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define OR_MAX_LEVELS 32

/* ---------------------------------------------------------------- hash grid */

/* Per-level layout of a tcnn-style hash grid with 3 input dims.
 * scale_l  = exp2f(l * log2f(b)) * base - 1      (float32, tcnn grid_scale)
 * res_l    = ceilf(scale_l) + 1                   (tcnn grid_resolution)
 * params_l = min(next_multiple(res_l^3, 8), 2^log2T); offsets are prefix sums.
 * Returns the total number of table entries (each holds F features). */
uint32_t or_hashgrid_layout(int n_levels, int log2_hashmap_size, int base_resolution,
                            float per_level_scale, uint32_t *offsets, uint32_t *resolutions,
                            float *scales) {
    const float log2s = log2f(per_level_scale);
    const uint32_t hashmap = 1u << log2_hashmap_size;
    const uint32_t max_params = 0xffffffffu / 2;
    uint32_t off = 0;
    for (int l = 0; l < n_levels; ++l) {
        float s = exp2f((float)l * log2s);
        s = s * (float)base_resolution;
        s = s - 1.0f;
        const uint32_t r = (uint32_t)ceilf(s) + 1u;
        uint32_t params;
        const float rf = (float)r;
        if (rf * rf * rf > (float)max_params) params = max_params;
        else params = r * r * r;
        params = (params + 7u) / 8u * 8u;
        if (params > hashmap) params = hashmap;
        offsets[l] = off;
        resolutions[l] = r;
        scales[l] = s;
        off += params;
    }
    offsets[n_levels] = off;
    return off;
}

/* tcnn grid_index for 3 dims, coherent-prime hash (factors 1, 2654435761,
 * 805459861).  stride is uint32 and wraps exactly as in the reference. */
static uint32_t or_grid_index(uint32_t hashmap_size, uint32_t res, const uint32_t pg[3]) {
    uint32_t stride = 1, index = 0;
    for (int d = 0; d < 3 && stride <= hashmap_size; ++d) {
        index += pg[d] * stride;
        stride *= res;
    }
    if (hashmap_size < stride) {
        index = (pg[0] * 1u) ^ (pg[1] * 2654435761u) ^ (pg[2] * 805459861u);
    }
    return index % hashmap_size;
}

/* Cell position and fractional offset for one level and one dim:
 * pos = fmaf(scale, x, 0.5); g = (uint32)(int)floorf(pos); frac = pos - floor. */
static void or_pos_fract(float x, float scale, uint32_t *g, float *frac) {
    float pos = fmaf(scale, x, 0.5f);
    float f = floorf(pos);
    *g = (uint32_t)(int32_t)f;
    *frac = pos - f;
}

/* Corner indices (entry index within the level, before the *F feature
 * stride) and trilinear weights, for n points and all levels.
 * idx/w are laid out [n][L][8]; corner c has bit d set when it is the +1
 * corner along dim d (tcnn loop order).  cells (optional, [n][L][3]) receives
 * the floor cell of each level as a signed integer. */
void or_hashgrid_index(const float *x, int64_t n, int n_levels, const uint32_t *offsets,
                       const uint32_t *resolutions, const float *scales, uint32_t *idx, float *w,
                       int32_t *cells) {
    for (int64_t i = 0; i < n; ++i) {
        for (int l = 0; l < n_levels; ++l) {
            uint32_t g[3];
            float fr[3];
            for (int d = 0; d < 3; ++d) or_pos_fract(x[i * 3 + d], scales[l], &g[d], &fr[d]);
            if (cells)
                for (int d = 0; d < 3; ++d) cells[(i * n_levels + l) * 3 + d] = (int32_t)g[d];
            const uint32_t hs = offsets[l + 1] - offsets[l];
            for (int c = 0; c < 8; ++c) {
                uint32_t pl[3];
                float wt = 1.0f;
                for (int d = 0; d < 3; ++d) {
                    if ((c & (1 << d)) == 0) { wt = wt * (1.0f - fr[d]); pl[d] = g[d]; }
                    else { wt = wt * fr[d]; pl[d] = g[d] + 1u; }
                }
                idx[(i * n_levels + l) * 8 + c] = or_grid_index(hs, resolutions[l], pl);
                w[(i * n_levels + l) * 8 + c] = wt;
            }
        }
    }
}

/* float32 encode with an fp32 table laid out [entry][F] (level l starts at
 * entry offsets[l]).  Accumulation is result = fmaf(w, v, result) over the
 * corners in tcnn order.  Levels >= active_levels produce 0 (band mask). */
void or_hashgrid_encode(const float *x, int64_t n, int n_levels, int n_feat, const uint32_t *offsets,
                        const uint32_t *resolutions, const float *scales, const float *table,
                        int active_levels, float *out, int64_t out_stride) {
    for (int64_t i = 0; i < n; ++i) {
        for (int l = 0; l < n_levels; ++l) {
            float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (l < active_levels) {
                uint32_t g[3];
                float fr[3];
                for (int d = 0; d < 3; ++d) or_pos_fract(x[i * 3 + d], scales[l], &g[d], &fr[d]);
                const uint32_t hs = offsets[l + 1] - offsets[l];
                for (int c = 0; c < 8; ++c) {
                    uint32_t pl[3];
                    float wt = 1.0f;
                    for (int d = 0; d < 3; ++d) {
                        if ((c & (1 << d)) == 0) { wt = wt * (1.0f - fr[d]); pl[d] = g[d]; }
                        else { wt = wt * fr[d]; pl[d] = g[d] + 1u; }
                    }
                    const uint64_t e = (uint64_t)offsets[l] + or_grid_index(hs, resolutions[l], pl);
                    for (int f = 0; f < n_feat; ++f) acc[f] = fmaf(wt, table[e * n_feat + f], acc[f]);
                }
            }
            for (int f = 0; f < n_feat; ++f) out[i * out_stride + l * n_feat + f] = acc[f];
        }
    }
}

/* -------------------------------------------------------- spherical harmonics */

/* Real SH basis of degree 4 (16 values) of a direction given in [0,1]^3 as
 * the reference feeds it ((d+1)/2, models/texture.py:24); the encoder maps it
 * back with v*2-1.  Constants are the real-SH normalisations, e.g.
 * Y00 = 1/(2 sqrt(pi)), Y1m = sqrt(3)/(2 sqrt(pi)), ... (sign convention of
 * the tcnn / Instant-NGP encoder: -y, z, -x for degree 1). */
void or_sh4(const float *d01, int64_t n, double *out) {
    const double pi = 3.14159265358979323846;
    const double sp = sqrt(pi);
    const double c0 = 1.0 / (2.0 * sp);
    const double c1 = sqrt(3.0) / (2.0 * sp);
    const double c2a = sqrt(15.0) / (2.0 * sp);
    const double c2b = sqrt(5.0) / (4.0 * sp);
    const double c2c = sqrt(15.0) / (4.0 * sp);
    const double c3a = sqrt(70.0) / (8.0 * sp);
    const double c3b = sqrt(105.0) / (2.0 * sp);
    const double c3c = sqrt(42.0) / (8.0 * sp);
    const double c3d = sqrt(7.0) / (4.0 * sp);
    const double c3e = sqrt(105.0) / (4.0 * sp);
    for (int64_t i = 0; i < n; ++i) {
        const double x = (double)(d01[i * 3 + 0] * 2.0f - 1.0f);
        const double y = (double)(d01[i * 3 + 1] * 2.0f - 1.0f);
        const double z = (double)(d01[i * 3 + 2] * 2.0f - 1.0f);
        const double xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
        double *o = out + i * 16;
        o[0] = c0;
        o[1] = -c1 * y;
        o[2] = c1 * z;
        o[3] = -c1 * x;
        o[4] = c2a * xy;
        o[5] = -c2a * yz;
        o[6] = c2b * (3.0 * z2 - 1.0);
        o[7] = -c2a * xz;
        o[8] = c2c * (x2 - y2);
        o[9] = c3a * y * (-3.0 * x2 + y2);
        o[10] = c3b * xy * z;
        o[11] = c3c * y * (1.0 - 5.0 * z2);
        o[12] = c3d * z * (5.0 * z2 - 3.0);
        o[13] = c3c * x * (1.0 - 5.0 * z2);
        o[14] = c3e * z * (x2 - y2);
        o[15] = c3a * x * (-x2 + 3.0 * y2);
    }
}

/* ----------------------------------------------------------------- nerfacc */

/* Slab test; near/far = 1e10 when the ray misses; near clipped at 0. */
void or_ray_aabb(const float *o, const float *d, int64_t n, const float *aabb, float *t_min,
                 float *t_max) {
    for (int64_t i = 0; i < n; ++i) {
        const float *ro = o + i * 3, *rd = d + i * 3;
        float tmin = (aabb[0] - ro[0]) / rd[0];
        float tmax = (aabb[3] - ro[0]) / rd[0];
        if (tmin > tmax) { float t = tmin; tmin = tmax; tmax = t; }
        float tymin = (aabb[1] - ro[1]) / rd[1];
        float tymax = (aabb[4] - ro[1]) / rd[1];
        if (tymin > tymax) { float t = tymin; tymin = tymax; tymax = t; }
        float nr, fr;
        if (tmin > tymax || tymin > tmax) { nr = 1e10f; fr = 1e10f; goto done; }
        if (tymin > tmin) tmin = tymin;
        if (tymax < tmax) tmax = tymax;
        {
            float tzmin = (aabb[2] - ro[2]) / rd[2];
            float tzmax = (aabb[5] - ro[2]) / rd[2];
            if (tzmin > tzmax) { float t = tzmin; tzmin = tzmax; tzmax = t; }
            if (tmin > tzmax || tzmin > tmax) { nr = 1e10f; fr = 1e10f; goto done; }
            if (tzmin > tmin) tmin = tzmin;
            if (tzmax < tmax) tmax = tzmax;
            nr = tmin;
            fr = tmax;
        }
    done:
        t_min[i] = nr > 0.0f ? nr : 0.0f;
        t_max[i] = fr;
    }
}

/* nerfacc 0.3.3 grid_occupied_at: contraction 0 = AABB (nothing outside
 * roi), 1 = UN_BOUNDED_SPHERE (roi -> [-1,1]^3, |x| > 1 -> (2 - 1/|x|) x/|x|,
 * then x/4 + 1/2; models/neus.py:69-74 builds the background grid this way). */
static int or_occupied(const float xyz[3], const float *roi, const uint8_t *binary, const int res[3],
                       int contraction) {
    float u[3];
    if (contraction == 0) {
        for (int d = 0; d < 3; ++d)
            if (xyz[d] < roi[d] || xyz[d] > roi[3 + d]) return 0;
        for (int d = 0; d < 3; ++d) u[d] = (xyz[d] - roi[d]) / (roi[3 + d] - roi[d]);
    } else {
        for (int d = 0; d < 3; ++d) u[d] = ((xyz[d] - roi[d]) / (roi[3 + d] - roi[d])) * 2.0f - 1.0f;
        const float nrm = sqrtf(fmaf(u[2], u[2], fmaf(u[1], u[1], u[0] * u[0])));
        if (nrm > 1.0f) {
            const float sc = 2.0f - 1.0f / nrm;
            for (int d = 0; d < 3; ++d) u[d] = sc * (u[d] / nrm);
        }
        for (int d = 0; d < 3; ++d) u[d] = u[d] * 0.25f + 0.5f;
    }
    int ix[3];
    for (int d = 0; d < 3; ++d) {
        int v = (int)(u[d] * (float)res[d]);
        if (v < 0) v = 0;
        if (v > res[d] - 1) v = res[d] - 1;
        ix[d] = v;
    }
    const int64_t cell = (int64_t)ix[0] * res[1] * res[2] + (int64_t)ix[1] * res[2] + ix[2];
    return binary[cell] != 0;
}

static float or_sign(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }

static float or_calc_dt(float t, float cone, float dt_min, float dt_max) {
    float v = t * cone;
    if (v < dt_min) v = dt_min;
    if (v > dt_max) v = dt_max;
    return v;
}

/* DDA distance to the next occupancy-cell boundary (AABB contraction). */
static float or_dist_next_voxel(const float xyz[3], const float dir[3], const float inv_dir[3],
                                const float *roi, const int res[3]) {
    float t = 0.0f;
    for (int d = 0; d < 3; ++d) {
        const float ext = roi[3 + d] - roi[d];
        const float r = (float)res[d];
        const float u = ((xyz[d] - roi[d]) / ext) * r;
        const float tgt = floorf(u + 0.5f + 0.5f * or_sign(dir[d]));
        const float td = (((tgt - u) * inv_dir[d]) / r) * ext;
        t = d == 0 ? td : (td < t ? td : t);
    }
    return t > 0.0f ? t : 0.0f;
}

/* Ray marching with grid skipping (contraction AABB) or stepping (contracted
 * grids), cone_angle >= 0.
 * Pass 1 (offsets == NULL): counts[i] = number of samples of ray i.
 * Pass 2: writes ray index, t0, t1 of every sample at offsets[i] + j.
 * The sample point is xyz = fmaf(t_mid, dir, origin).  max_steps bounds the
 * loop; a ray that reaches it is cut there and flagged in *overflow. */
void or_march(const float *rays_o, const float *rays_d, const float *t_min, const float *t_max,
              int64_t n_rays, const float *roi, const uint8_t *binary, int rx, int ry, int rz,
              int contraction, float step, float cone, int64_t max_steps, int32_t *counts,
              const int64_t *offsets, int32_t *ray_indices, float *t_starts, float *t_ends,
              int32_t *overflow) {
    const int res[3] = {rx, ry, rz};
    for (int64_t i = 0; i < n_rays; ++i) {
        const float *o = rays_o + i * 3, *d = rays_d + i * 3;
        float inv[3];
        for (int k = 0; k < 3; ++k) inv[k] = 1.0f / d[k];
        const float near = t_min[i], far = t_max[i];
        const float dt_min = step, dt_max = 1e10f;
        int64_t j = 0, it = 0;
        float t0 = near;
        float dt = or_calc_dt(t0, cone, dt_min, dt_max);
        float t1 = t0 + dt;
        float tm = (t0 + t1) * 0.5f;
        while (tm < far) {
            if (++it > max_steps) { if (overflow) *overflow = 1; break; }
            float xyz[3];
            for (int k = 0; k < 3; ++k) xyz[k] = fmaf(tm, d[k], o[k]);
            if (or_occupied(xyz, roi, binary, res, contraction)) {
                if (offsets) {
                    const int64_t p = offsets[i] + j;
                    ray_indices[p] = (int32_t)i;
                    t_starts[p] = t0;
                    t_ends[p] = t1;
                }
                ++j;
                t0 = t1;
                t1 = t0 + or_calc_dt(t0, cone, dt_min, dt_max);
                tm = (t0 + t1) * 0.5f;
            } else if (contraction != 0) {
                /* a contracted grid is not skipped: the next step */
                t0 = t1;
                t1 = t0 + or_calc_dt(t0, cone, dt_min, dt_max);
                tm = (t0 + t1) * 0.5f;
            } else {
                const float tgt = tm + or_dist_next_voxel(xyz, d, inv, roi, res);
                float tt = tm;
                int64_t guard = 0;
                do { tt += dt_min; } while (tt < tgt && ++guard < max_steps);
                tm = tt;
                dt = or_calc_dt(tm, cone, dt_min, dt_max);
                t0 = tm - dt * 0.5f;
                t1 = tm + dt * 0.5f;
            }
        }
        if (!offsets) counts[i] = (int32_t)j;
    }
}

/* Rendering weights from alpha, per ray in sample order:
 * T_0 = 1, w_j = alpha_j * T_j, T_{j+1} = T_j * (1 - alpha_j); w_j = 0 once
 * T_j < early_stop_eps; samples with alpha < alpha_thre keep w = 0 and do
 * not attenuate T.  Also returns the transmittance T_j of each sample. */
void or_weights(const float *alpha, const int64_t *offsets, int64_t n_rays, float early_stop_eps,
                float alpha_thre, float *weights, float *trans) {
    for (int64_t r = 0; r < n_rays; ++r) {
        float T = 1.0f;
        int stopped = 0;
        for (int64_t j = offsets[r]; j < offsets[r + 1]; ++j) {
            if (T < early_stop_eps) stopped = 1;
            trans[j] = T;
            if (stopped || alpha[j] < alpha_thre) { weights[j] = 0.0f; continue; }
            weights[j] = alpha[j] * T;
            T = T * (1.0f - alpha[j]);
        }
    }
}

/* Occupancy bitfield from float occupancies: bit c of word c>>5 is set when
 * occ[c] > min(mean(occ), thre), mean accumulated in double. */
void or_occ_binary(const float *occ, int64_t n_cells, float thre, uint32_t *bits) {
    double s = 0.0;
    for (int64_t c = 0; c < n_cells; ++c) s += occ[c];
    float m = (float)(s / (double)n_cells);
    float t = m < thre ? m : thre;
    memset(bits, 0, (size_t)((n_cells + 31) / 32) * 4);
    for (int64_t c = 0; c < n_cells; ++c)
        if (occ[c] > t) bits[c >> 5] |= 1u << (c & 31);
}
