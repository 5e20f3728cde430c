// Plain multiresolution hash-grid encode / backward (the tcnn HashGrid seam of
// models/network_utils.py:47,56-59).  One thread per (point, level); the level
// is blockIdx.y so a warp's 32 points share a level's scale and table slice.
#include <math.h>

#include "common.cuh"

using namespace angelo;

extern "C" int angelo_hashgrid_layout(const angelo_hashgrid_desc *desc,
                                      angelo_hashgrid_layout_t *out) {
    ANGELO_REQUIRE(desc && out, "hashgrid_layout: null argument");
    ANGELO_REQUIRE(desc->n_levels >= 1 && desc->n_levels <= ANGELO_MAX_LEVELS,
                   "hashgrid_layout: n_levels %d outside [1, %d]", desc->n_levels,
                   ANGELO_MAX_LEVELS);
    ANGELO_REQUIRE(desc->n_features == 2, "hashgrid_layout: only 2 features per level");
    ANGELO_REQUIRE(desc->log2_hashmap_size >= 3 && desc->log2_hashmap_size <= 30,
                   "hashgrid_layout: log2_hashmap_size %d outside [3, 30]",
                   desc->log2_hashmap_size);
    ANGELO_REQUIRE(desc->base_resolution >= 1 && desc->per_level_scale >= 1.0f,
                   "hashgrid_layout: bad base resolution / scale");
    // float32 arithmetic in the order of tcnn's grid_scale(); volatile keeps
    // the host compiler from fusing the multiply and the subtraction.
    const float log2s = log2f(desc->per_level_scale);
    const uint32_t hashmap = 1u << desc->log2_hashmap_size;
    const uint32_t max_params = 0xffffffffu / 2;
    uint64_t off = 0;
    out->n_levels = desc->n_levels;
    out->n_features = desc->n_features;
    for (int l = 0; l < desc->n_levels; ++l) {
        volatile float s = exp2f((float)l * log2s);
        s = s * (float)desc->base_resolution;
        s = s - 1.0f;
        const uint32_t r = (uint32_t)ceilf(s) + 1u;
        const float rf = (float)r;
        uint32_t params = (rf * rf * rf > (float)max_params) ? max_params : r * r * r;
        params = (params + 7u) / 8u * 8u;
        if (params > hashmap) params = hashmap;
        out->offsets[l] = (uint32_t)off;
        out->resolutions[l] = r;
        out->scales[l] = s;
        off += params;
        ANGELO_REQUIRE(off < (1ull << 31), "hashgrid_layout: table larger than 2^31 entries");
    }
    out->offsets[desc->n_levels] = (uint32_t)off;
    return ANGELO_OK;
}

namespace {

// One thread per point over every level: the point's output row (x*2-1, then
// two features per level) is assembled in shared memory and written out a row
// per warp instruction, so that every sector of the output is written whole
// once.  (A launch dimension per level wrote 8 bytes into every row per level;
// with outputs larger than L2 those sectors were evicted partly written and
// read back from HBM once per level.)
constexpr int kFwdRows = 128;

__global__ void __launch_bounds__(kFwdRows) hashgrid_fwd_kernel(
    const __grid_constant__ angelo_hashgrid_layout_t lay, int active, const float *__restrict__ x,
    int64_t n, const void *__restrict__ table, int dtype, int include_xyz, float *__restrict__ out,
    int64_t out_stride, int64_t out_col) {
    extern __shared__ float rows[];
    const int width = (include_xyz ? 3 : 0) + 2 * lay.n_levels;
    const int pitch = width | 1;   // odd: one row per thread without bank conflicts
    const int64_t i0 = (int64_t)blockIdx.x * kFwdRows;
    const int t = threadIdx.x;
    const int64_t i = i0 + t;
    if (i < n) {
        const float x0 = x[i * 3 + 0], x1 = x[i * 3 + 1], x2 = x[i * 3 + 2];
        float *r = rows + t * pitch;
        if (include_xyz) {
            r[0] = __fsub_rn(__fmul_rn(x0, 2.0f), 1.0f);
            r[1] = __fsub_rn(__fmul_rn(x1, 2.0f), 1.0f);
            r[2] = __fsub_rn(__fmul_rn(x2, 2.0f), 1.0f);
            r += 3;
        }
        for (int l = 0; l < lay.n_levels; ++l) {
            float r0 = 0.0f, r1 = 0.0f;
            if (l < active) {
                const LevelPos p = level_pos(x0, x1, x2, lay.scales[l]);
                const uint64_t base = lay.offsets[l];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float w = corner_weight(p, c);
                    const float2 v = load_entry(table, dtype, base + corner_index(lay, l, p, c));
                    r0 = __fmaf_rn(w, v.x, r0);
                    r1 = __fmaf_rn(w, v.y, r1);
                }
            }
            r[2 * l] = r0;
            r[2 * l + 1] = r1;
        }
    }
    __syncthreads();
    const int warp = t >> 5, lane = t & 31;
    const int64_t nr = n - i0 < kFwdRows ? n - i0 : kFwdRows;
    for (int64_t q = warp; q < nr; q += kFwdRows / 32) {
        float *o = out + (i0 + q) * out_stride + out_col;
        const float *r = rows + q * pitch;
        for (int c = lane; c < width; c += 32) o[c] = r[c];
    }
}

__global__ void __launch_bounds__(256) hashgrid_bwd_table_kernel(
    const __grid_constant__ angelo_hashgrid_layout_t lay, int active, const float *__restrict__ x,
    int64_t n, int include_xyz, const float *__restrict__ dout, int64_t dout_stride,
    int64_t dout_col, float *__restrict__ dtable) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (l >= active) return;  // uniform over the block
    const bool valid = i < n;
    float g0 = 0.0f, g1 = 0.0f;
    LevelPos p{};
    if (valid) {
        const float *g = dout + i * dout_stride + dout_col + (include_xyz ? 3 : 0) + l * 2;
        g0 = g[0];
        g1 = g[1];
        p = level_pos(x[i * 3 + 0], x[i * 3 + 1], x[i * 3 + 2], lay.scales[l]);
    }
    const bool live = valid && (g0 != 0.0f || g1 != 0.0f);
    const uint64_t base = lay.offsets[l];
    float2 *dt = reinterpret_cast<float2 *>(dtable);
    // coarse levels: consecutive points share corners, so aggregate in the
    // warp first (the level, hence the branch, is uniform over the block)
    const bool coarse = lay.resolutions[l] <= 300u;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float w = live ? corner_weight(p, c) : 0.0f;
        const uint64_t e = live ? base + corner_index(lay, l, p, c) : 0;
        if (coarse) {
            aggregated_add2<1>(dt, e, w * g0, w * g1, live);
        } else if (live) {
            atomicAdd(dt + e, make_float2(w * g0, w * g1));
        }
    }
}

// dL/dx of the encoding: sum over levels/features of dL/denc * d enc/dx with
// d enc/dx_d = scale * sum_corners v * dw/dfrac_d (derivative of the
// trilinear weights), plus 2*dL/dxyz for the concatenated x*2-1.
__global__ void __launch_bounds__(128) hashgrid_bwd_input_kernel(
    const __grid_constant__ angelo_hashgrid_layout_t lay, int active, const float *__restrict__ x,
    int64_t n, const void *__restrict__ table, int dtype, int include_xyz,
    const float *__restrict__ dout, int64_t dout_stride, int64_t dout_col, float *__restrict__ dx) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x0 = x[i * 3 + 0], x1 = x[i * 3 + 1], x2 = x[i * 3 + 2];
    const float *g = dout + i * dout_stride + dout_col;
    float acc[3] = {0.0f, 0.0f, 0.0f};
    if (include_xyz) {
        acc[0] = 2.0f * g[0];
        acc[1] = 2.0f * g[1];
        acc[2] = 2.0f * g[2];
        g += 3;
    }
    for (int l = 0; l < active; ++l) {
        const float g0 = g[l * 2 + 0], g1 = g[l * 2 + 1];
        if (g0 == 0.0f && g1 == 0.0f) continue;
        const float s = lay.scales[l];
        const LevelPos p = level_pos(x0, x1, x2, s);
        const uint64_t base = lay.offsets[l];
        float dl[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float2 v = load_entry(table, dtype, base + corner_index(lay, l, p, c));
            const float gv = g0 * v.x + g1 * v.y;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                float w = 1.0f;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (k == d) continue;
                    w *= (c >> k) & 1 ? p.f[k] : 1.0f - p.f[k];
                }
                dl[d] += ((c >> d) & 1 ? w : -w) * gv;
            }
        }
        acc[0] += s * dl[0];
        acc[1] += s * dl[1];
        acc[2] += s * dl[2];
    }
    dx[i * 3 + 0] = acc[0];
    dx[i * 3 + 1] = acc[1];
    dx[i * 3 + 2] = acc[2];
}

__global__ void hashgrid_index_kernel(const __grid_constant__ angelo_hashgrid_layout_t lay,
                                      const float *__restrict__ x, int64_t n,
                                      uint32_t *__restrict__ idx, float *__restrict__ w) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (i >= n) return;
    const LevelPos p = level_pos(x[i * 3 + 0], x[i * 3 + 1], x[i * 3 + 2], lay.scales[l]);
    const int64_t o = (i * lay.n_levels + l) * 8;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        idx[o + c] = corner_index(lay, l, p, c);
        w[o + c] = corner_weight(p, c);
    }
}

int check_layout(const angelo_hashgrid_layout_t *lay, int active) {
    ANGELO_REQUIRE(lay != nullptr, "hash grid: null layout");
    ANGELO_REQUIRE(lay->n_levels >= 1 && lay->n_levels <= ANGELO_MAX_LEVELS,
                   "hash grid: bad n_levels %d", lay->n_levels);
    ANGELO_REQUIRE(lay->n_features == 2, "hash grid: only 2 features per level");
    ANGELO_REQUIRE(active >= 0 && active <= lay->n_levels, "hash grid: active_levels %d outside [0, %d]",
                   active, lay->n_levels);
    return ANGELO_OK;
}

}  // namespace

extern "C" int angelo_hashgrid_fwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                   const float *x, int64_t n, const void *table,
                                   int32_t table_dtype, int32_t include_xyz, float *out,
                                   int64_t out_stride, int64_t out_col, void *stream) {
    if (int e = check_layout(lay, active_levels)) return e;
    ANGELO_REQUIRE(n >= 0, "hashgrid_fwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(x && table && out, "hashgrid_fwd: null pointer");
    ANGELO_REQUIRE(table_dtype == ANGELO_DTYPE_F32 || table_dtype == ANGELO_DTYPE_F16,
                   "hashgrid_fwd: bad table dtype");
    ANGELO_REQUIRE(out_stride >= out_col + lay->n_levels * 2 + (include_xyz ? 3 : 0),
                   "hashgrid_fwd: out_stride too small");
    const int width = (include_xyz ? 3 : 0) + 2 * lay->n_levels;
    const size_t smem = (size_t)kFwdRows * (width | 1) * sizeof(float);
    hashgrid_fwd_kernel<<<blocks_for(n, kFwdRows), kFwdRows, smem, as_stream(stream)>>>(
        *lay, active_levels, x, n, table, table_dtype, include_xyz, out, out_stride, out_col);
    return check_launch("hashgrid_fwd");
}

extern "C" int angelo_hashgrid_bwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                                   const float *x, int64_t n, const void *table,
                                   int32_t table_dtype, int32_t include_xyz, const float *dout,
                                   int64_t dout_stride, int64_t dout_col, float *dtable,
                                   float *dx, void *stream) {
    if (int e = check_layout(lay, active_levels)) return e;
    ANGELO_REQUIRE(n >= 0, "hashgrid_bwd: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(x && dout, "hashgrid_bwd: null pointer");
    ANGELO_REQUIRE(dout_stride >= dout_col + lay->n_levels * 2 + (include_xyz ? 3 : 0),
                   "hashgrid_bwd: dout_stride too small");
    if (dtable && active_levels > 0) {
        dim3 grid(blocks_for(n, 256), active_levels);
        hashgrid_bwd_table_kernel<<<grid, 256, 0, as_stream(stream)>>>(
            *lay, active_levels, x, n, include_xyz, dout, dout_stride, dout_col, dtable);
        if (int e = check_launch("hashgrid_bwd(table)")) return e;
    }
    if (dx) {
        ANGELO_REQUIRE(table != nullptr, "hashgrid_bwd: dx needs the table");
        hashgrid_bwd_input_kernel<<<blocks_for(n, 128), 128, 0, as_stream(stream)>>>(
            *lay, active_levels, x, n, table, table_dtype, include_xyz, dout, dout_stride,
            dout_col, dx);
        if (int e = check_launch("hashgrid_bwd(input)")) return e;
    }
    return ANGELO_OK;
}

extern "C" int angelo_hashgrid_index(const angelo_hashgrid_layout_t *lay, const float *x,
                                     int64_t n, uint32_t *idx, float *w, void *stream) {
    if (int e = check_layout(lay, 0)) return e;
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(x && idx && w, "hashgrid_index: null pointer");
    dim3 grid(blocks_for(n, 256), lay->n_levels);
    hashgrid_index_kernel<<<grid, 256, 0, as_stream(stream)>>>(*lay, x, n, idx, w);
    return check_launch("hashgrid_index");
}
