// Ray-AABB clipping and occupancy-grid ray marching (the nerfacc 0.3.3 calls
// at models/neus.py:153 and models/neus.py:210-220).
//
// The per-ray march is a sequential float32 recurrence (t0 <- t1, t1 <- t0 +
// dt, DDA skips over empty cells) whose rounding fixes which samples exist, so
// each ray is marched by one thread exactly in the reference's order; the
// occupancy bitfield (res^3 bits, 256 KiB at 128^3) stays L1/L2 resident.
// Count, scan and fill are three launches, as in the reference; with a bound
// on the samples per ray, record (count + the samples into a per-ray scratch),
// scan and compact march each ray once.
#include <cmath>

#include "common.cuh"

using namespace angelo;

namespace {

// lanes per ray of the AABB grid's march (1: the sequential march itself)
#ifndef ANGELO_MARCH_AABB_LANES
#define ANGELO_MARCH_AABB_LANES 8
#endif
constexpr int kAabbLanes = ANGELO_MARCH_AABB_LANES;

// The march kernels map a group of G lanes to a ray (G = 32: a warp) or one
// thread to a ray (G = 1).  The launch picks the warp for the
// unbounded-sphere grid (the learned background: no empty-space skipping, so
// every round of the lookahead is a full run of 32 steps) and groups of 8 for
// the AABB grid, whose steps alternate between short runs of occupied steps
// and DDA skips: measured on the training step, the foreground's march took
// 0.25 ms per step one thread per ray, 0.23 with 4 lanes, 0.21 with 8 and
// 0.38 with 32; the background's went from ~0.19 to ~0.06 with 32.

struct Grid {
    float lo[3], hi[3];
    int res[3];
    // bit d set: the extent hi - lo (pow2_ext) or the resolution (pow2_res)
    // of axis d is a power of two, and a division by it is the exact
    // multiplication by its reciprocal: RN(x / 2^k) = RN(x * 2^-k), both the
    // correctly rounded value of the same real number
    int pow2_ext, pow2_res;
    float inv_ext[3], inv_res[3];
    const uint32_t *bits;
    int contraction;   // ANGELO_CONTRACT_*
};

__device__ __forceinline__ float div_ext(const Grid &g, int d, float x) {
    return ((g.pow2_ext >> d) & 1) ? __fmul_rn(x, g.inv_ext[d]) : __fdiv_rn(x, __fsub_rn(g.hi[d], g.lo[d]));
}
__device__ __forceinline__ float div_res(const Grid &g, int d, float x) {
    return ((g.pow2_res >> d) & 1) ? __fmul_rn(x, g.inv_res[d]) : __fdiv_rn(x, (float)g.res[d]);
}

__device__ __forceinline__ bool occupied(const Grid &g, const float xyz[3]) {
    float u[3];
    if (g.contraction == ANGELO_CONTRACT_AABB) {
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (xyz[d] < g.lo[d] || xyz[d] > g.hi[d]) return false;
        if (g.bits == nullptr) return true;
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = div_ext(g, d, __fsub_rn(xyz[d], g.lo[d]));
    } else {
        // unbounded sphere: roi -> [-1,1]^3; beyond the unit sphere
        // x <- (2 - 1/|x|) x/|x|; the radius-2 ball -> [0,1]^3
        if (g.bits == nullptr) return true;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            u[d] = __fsub_rn(__fmul_rn(div_ext(g, d, __fsub_rn(xyz[d], g.lo[d])), 2.0f), 1.0f);
        const float nrm = __fsqrt_rn(__fmaf_rn(u[2], u[2], __fmaf_rn(u[1], u[1], __fmul_rn(u[0], u[0]))));
        if (nrm > 1.0f) {
            const float sc = __fsub_rn(2.0f, __fdiv_rn(1.0f, nrm));
#pragma unroll
            for (int d = 0; d < 3; ++d) u[d] = __fmul_rn(sc, __fdiv_rn(u[d], nrm));
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = __fadd_rn(__fmul_rn(u[d], 0.25f), 0.5f);
    }
    int ix[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int v = (int)__fmul_rn(u[d], (float)g.res[d]);
        v = v < 0 ? 0 : (v > g.res[d] - 1 ? g.res[d] - 1 : v);
        ix[d] = v;
    }
    const int64_t c = ((int64_t)ix[0] * g.res[1] + ix[1]) * g.res[2] + ix[2];
    return (__ldg(g.bits + (c >> 5)) >> (c & 31)) & 1u;
}

__device__ __forceinline__ float sgn(float v) { return v > 0.f ? 1.f : (v < 0.f ? -1.f : 0.f); }

__device__ __forceinline__ float calc_dt(float t, float cone, float dt_min) {
    float v = __fmul_rn(t, cone);
    v = v < dt_min ? dt_min : v;
    return v > 1e10f ? 1e10f : v;
}

__device__ __forceinline__ float dist_next_voxel(const Grid &g, const float xyz[3],
                                                 const float dir[3], const float inv[3]) {
    float t = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float ext = __fsub_rn(g.hi[d], g.lo[d]);
        const float r = (float)g.res[d];
        const float u = __fmul_rn(div_ext(g, d, __fsub_rn(xyz[d], g.lo[d])), r);
        const float tgt = floorf(__fadd_rn(__fadd_rn(u, 0.5f), __fmul_rn(0.5f, sgn(dir[d]))));
        const float td = __fmul_rn(div_res(g, d, __fmul_rn(__fsub_rn(tgt, u), inv[d])), ext);
        t = d == 0 ? td : fminf(t, td);
    }
    return t > 0.f ? t : 0.f;
}

// One ray; emit(j, t0, t1) for each sample; returns the sample count.
template <typename Emit>
__device__ __forceinline__ int64_t march_ray(const Grid &g, const float o[3], const float d[3],
                                             float near, float far, float step, float cone,
                                             int64_t max_steps, int32_t *status, Emit emit) {
    float inv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) inv[k] = __fdiv_rn(1.0f, d[k]);
    int64_t j = 0, it = 0;
    float t0 = near;
    float t1 = __fadd_rn(t0, calc_dt(t0, cone, step));
    float tm = __fmul_rn(__fadd_rn(t0, t1), 0.5f);
    while (tm < far) {
        if (++it > max_steps) {
            if (status) atomicOr(status, 1);
            break;
        }
        float xyz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) xyz[k] = __fmaf_rn(tm, d[k], o[k]);
        if (occupied(g, xyz)) {
            emit(j, t0, t1);
            ++j;
            t0 = t1;
            t1 = __fadd_rn(t0, calc_dt(t0, cone, step));
            tm = __fmul_rn(__fadd_rn(t0, t1), 0.5f);
        } else if (g.contraction != ANGELO_CONTRACT_AABB) {
            // contracted grids are not skipped: the next step
            t0 = t1;
            t1 = __fadd_rn(t0, calc_dt(t0, cone, step));
            tm = __fmul_rn(__fadd_rn(t0, t1), 0.5f);
        } else {
            const float tgt = __fadd_rn(tm, dist_next_voxel(g, xyz, d, inv));
            float tt = tm;
            int64_t guard = 0;
            do {
                tt = __fadd_rn(tt, step);
            } while (tt < tgt && ++guard < max_steps);
            tm = tt;
            const float dt = calc_dt(tm, cone, step);
            t0 = __fsub_rn(tm, __fmul_rn(dt, 0.5f));
            t1 = __fadd_rn(tm, __fmul_rn(dt, 0.5f));
        }
    }
    return j;
}

// The same march with one warp per ray.  The recurrence stays sequential in
// its arithmetic, but the occupancy lookups need not wait for each other:
// each round, lane k takes the march state k steps ahead of the warp's state,
// assuming the next k steps are all of the current kind (advance within
// occupied cells, or DDA skips over empty ones), by applying the sequential
// update k times with the same rounding; all 32 lanes then look their cell up
// at once.  The first lane whose step is of the other kind (or past the far
// plane or the step limit) ends the round: the steps before it are the
// sequential march's steps, its state is where the next round starts.
// Samples come out in the sequential order with the same values.
struct MarchState {
    float t0, t1, tm;
};

__device__ __forceinline__ MarchState march_advance(const MarchState &s, float cone, float step) {
    MarchState r;
    r.t0 = s.t1;
    r.t1 = __fadd_rn(r.t0, calc_dt(r.t0, cone, step));
    r.tm = __fmul_rn(__fadd_rn(r.t0, r.t1), 0.5f);
    return r;
}

__device__ __forceinline__ MarchState march_skip(const Grid &g, const MarchState &s, const float o[3],
                                                 const float d[3], const float inv[3], float cone, float step,
                                                 int64_t max_steps) {
    float xyz[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) xyz[k] = __fmaf_rn(s.tm, d[k], o[k]);
    const float tgt = __fadd_rn(s.tm, dist_next_voxel(g, xyz, d, inv));
    float tt = s.tm;
    int64_t guard = 0;
    do {
        tt = __fadd_rn(tt, step);
    } while (tt < tgt && ++guard < max_steps);
    MarchState r;
    r.tm = tt;
    const float dt = calc_dt(tt, cone, step);
    r.t0 = __fsub_rn(tt, __fmul_rn(dt, 0.5f));
    r.t1 = __fadd_rn(tt, __fmul_rn(dt, 0.5f));
    return r;
}

// Every lane of a group of G lanes (G a power of two up to 32, groups
// aligned in the warp) calls this for the same ray; emit(j, t0, t1) is called
// by the lane that owns sample j.  Returns the sample count (the same in
// every lane of the group).
template <int G, typename Emit>
__device__ __forceinline__ int64_t march_ray_group(const Grid &g, const float o[3], const float d[3], float near,
                                                   float far, float step, float cone, int64_t max_steps,
                                                   int32_t *status, Emit emit) {
    const int lane = threadIdx.x & (G - 1);
    const int gbase = (threadIdx.x & 31) & ~(G - 1);   // the group's first lane in the warp
    const uint32_t gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << gbase);
    const uint32_t all = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
    const bool aabb = g.contraction == ANGELO_CONTRACT_AABB;
    float inv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) inv[k] = __fdiv_rn(1.0f, d[k]);
    MarchState S;
    S.t0 = near;
    S.t1 = __fadd_rn(S.t0, calc_dt(S.t0, cone, step));
    S.tm = __fmul_rn(__fadd_rn(S.t0, S.t1), 0.5f);
    bool skipping = false;   // the kind of step the round assumes
    int64_t j = 0, it = 0;
    while (true) {
        // this lane's state: `lane` steps of the assumed kind after S
        MarchState st = S;
        for (int k = 0; k < lane; ++k)
            st = skipping ? march_skip(g, st, o, d, inv, cone, step, max_steps) : march_advance(st, cone, step);
        const bool in_range = st.tm < far;
        const bool in_steps = it + lane + 1 <= max_steps;
        bool occ = false;
        if (in_range && in_steps) {
            float xyz[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) xyz[k] = __fmaf_rn(st.tm, d[k], o[k]);
            occ = occupied(g, xyz);
        }
        // the step's kind: contracted grids always advance (no skipping)
        const bool skip_here = aabb && !occ;
        const bool same = in_range && in_steps && skip_here == skipping;
        const uint32_t ok = (__ballot_sync(gmask, same) >> gbase) & all;
        const int first = ok == all ? G : __ffs(~ok) - 1;   // the first step that ends the run
        // the run's samples: lanes before `first` whose cell is occupied
        const uint32_t emits = (__ballot_sync(gmask, lane < first && occ) >> gbase) & all;
        if (lane < first && occ) emit(j + __popc(emits & ((1u << lane) - 1u)), st.t0, st.t1);
        j += __popc(emits);
        it += first;
        if (first == G) {
            // the whole run held: the next round starts one step after the
            // group's last lane
            MarchState nx = skipping ? march_skip(g, st, o, d, inv, cone, step, max_steps)
                                     : march_advance(st, cone, step);
            S.t0 = __shfl_sync(gmask, nx.t0, gbase + G - 1);
            S.t1 = __shfl_sync(gmask, nx.t1, gbase + G - 1);
            S.tm = __shfl_sync(gmask, nx.tm, gbase + G - 1);
            continue;
        }
        // the run ends at lane `first`: past the far plane, out of steps, or
        // a step of the other kind, which the next round starts with
        const bool f_range = __shfl_sync(gmask, in_range, gbase + first);
        const bool f_steps = __shfl_sync(gmask, in_steps, gbase + first);
        if (!f_range) break;
        if (!f_steps) {
            if (status && lane == 0) atomicOr(status, 1);
            break;
        }
        S.t0 = __shfl_sync(gmask, st.t0, gbase + first);
        S.t1 = __shfl_sync(gmask, st.t1, gbase + first);
        S.tm = __shfl_sync(gmask, st.tm, gbase + first);
        skipping = !skipping;
    }
    return j;
}

__global__ void ray_aabb_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                int64_t n, const float *__restrict__ aabb, float *__restrict__ tmin_out,
                                float *__restrict__ tmax_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *o = ro + i * 3, *d = rd + i * 3;
    float tmin = __fdiv_rn(aabb[0] - o[0], d[0]);
    float tmax = __fdiv_rn(aabb[3] - o[0], d[0]);
    if (tmin > tmax) { const float t = tmin; tmin = tmax; tmax = t; }
    float tymin = __fdiv_rn(aabb[1] - o[1], d[1]);
    float tymax = __fdiv_rn(aabb[4] - o[1], d[1]);
    if (tymin > tymax) { const float t = tymin; tymin = tymax; tymax = t; }
    float nr = 1e10f, fr = 1e10f;
    if (!(tmin > tymax || tymin > tmax)) {
        if (tymin > tmin) tmin = tymin;
        if (tymax < tmax) tmax = tymax;
        float tzmin = __fdiv_rn(aabb[2] - o[2], d[2]);
        float tzmax = __fdiv_rn(aabb[5] - o[2], d[2]);
        if (tzmin > tzmax) { const float t = tzmin; tzmin = tzmax; tzmax = t; }
        if (!(tmin > tzmax || tzmin > tmax)) {
            if (tzmin > tmin) tmin = tzmin;
            if (tzmax < tmax) tmax = tzmax;
            nr = tmin;
            fr = tmax;
        }
    }
    tmin_out[i] = nr > 0.f ? nr : 0.f;
    tmax_out[i] = fr;
}

template <int G>
__global__ void march_count_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                   const float *__restrict__ tmin, const float *__restrict__ tmax,
                                   int64_t n, Grid g, float step, float cone, int64_t max_steps,
                                   int32_t *__restrict__ counts, int32_t *status) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (i >= n) return;
    const float o[3] = {ro[i * 3], ro[i * 3 + 1], ro[i * 3 + 2]};
    const float d[3] = {rd[i * 3], rd[i * 3 + 1], rd[i * 3 + 2]};
    auto none = [](int64_t, float, float) {};
    const int64_t c = G > 1 ? march_ray_group<G>(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, none)
                            : march_ray(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, none);
    if ((threadIdx.x & (G - 1)) == 0) counts[i] = (int32_t)(c > 0x7fffffff ? 0x7fffffff : c);
}

template <int G>
__global__ void march_fill_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                  const float *__restrict__ tmin, const float *__restrict__ tmax,
                                  int64_t n, Grid g, float step, float cone, int64_t max_steps,
                                  const int64_t *__restrict__ offsets, int64_t capacity,
                                  int32_t *__restrict__ ray_idx, float *__restrict__ ts,
                                  float *__restrict__ te, int32_t *status) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (i >= n) return;
    const float o[3] = {ro[i * 3], ro[i * 3 + 1], ro[i * 3 + 2]};
    const float d[3] = {rd[i * 3], rd[i * 3 + 1], rd[i * 3 + 2]};
    const int64_t base = offsets[i];
    const int64_t limit = offsets[i + 1];
    bool dropped = false;
    auto emit = [&](int64_t j, float t0, float t1) {
        const int64_t p = base + j;
        if (p < capacity && p < limit) {
            ray_idx[p] = (int32_t)i;
            ts[p] = t0;
            te[p] = t1;
        } else {
            dropped = true;
        }
    };
    if (G > 1) march_ray_group<G>(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, emit);
    else march_ray(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, emit);
    if (dropped && status) atomicOr(status, 2);
}

// One march per ray: the count and the first per_ray samples into scratch.
template <int G>
__global__ void march_record_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                    const float *__restrict__ tmin, const float *__restrict__ tmax,
                                    int64_t n, Grid g, float step, float cone, int64_t max_steps,
                                    int32_t per_ray, float2 *__restrict__ scratch,
                                    int32_t *__restrict__ counts, int32_t *status) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    if (i >= n) return;
    const float o[3] = {ro[i * 3], ro[i * 3 + 1], ro[i * 3 + 2]};
    const float d[3] = {rd[i * 3], rd[i * 3 + 1], rd[i * 3 + 2]};
    float2 *dst = scratch + i * per_ray;
    auto emit = [&](int64_t j, float t0, float t1) {
        if (j < per_ray) dst[j] = make_float2(t0, t1);
    };
    const int64_t c = G > 1 ? march_ray_group<G>(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, emit)
                            : march_ray(g, o, d, tmin[i], tmax[i], step, cone, max_steps, status, emit);
    if ((threadIdx.x & (G - 1)) != 0) return;
    if (c > per_ray) atomicOr(status, 4);
    counts[i] = (int32_t)(c > 0x7fffffff ? 0x7fffffff : c);
}

// One CTA per ray copies its recorded samples to the packed outputs.
__global__ void march_compact_kernel(const float2 *__restrict__ scratch, int32_t per_ray,
                                     const int32_t *__restrict__ counts,
                                     const int64_t *__restrict__ offsets, int64_t capacity,
                                     int32_t *__restrict__ ray_idx, float *__restrict__ ts,
                                     float *__restrict__ te, int32_t *status) {
    const int64_t i = blockIdx.x;
    const int c = min(counts[i], per_ray);
    const int64_t base = offsets[i];
    bool dropped = false;
    for (int j = threadIdx.x; j < c; j += blockDim.x) {
        const int64_t p = base + j;
        if (p < capacity) {
            const float2 t = scratch[i * per_ray + j];
            ray_idx[p] = (int32_t)i;
            ts[p] = t.x;
            te[p] = t.y;
        } else {
            dropped = true;
        }
    }
    if (dropped && status) atomicOr(status, 2);
}

// ---------------------------------------------------------------- scan
// Three-phase exclusive scan of int32 counts into int64 offsets: per-block
// scans of 1024 counts (256 threads x 4), one block scanning the block sums,
// then the block offsets added back.

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *total) {
    __shared__ int64_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    const int64_t before = warp > 0 ? warp_sums[warp - 1] : 0;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const int32_t *__restrict__ in,
                                                                  int64_t n, int64_t *__restrict__ out,
                                                                  int64_t *__restrict__ tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? (int64_t)in[base + k] : 0;
        s += v[k];
    }
    int64_t total;
    int64_t run = block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(int64_t *__restrict__ sums,
                                                                 int64_t n_tiles,
                                                                 int64_t *__restrict__ grand) {
    int64_t carry = 0;
    for (int64_t start = 0; start < n_tiles; start += kScanThreads) {
        const int64_t i = start + threadIdx.x;
        const int64_t v = i < n_tiles ? sums[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan(v, &total);
        if (i < n_tiles) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_add_kernel(int64_t *__restrict__ out,
                                                                int64_t n,
                                                                const int64_t *__restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    const int64_t add = sums[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += kScanThreads)
        if (base + k < n) out[base + k] += add;
}

int make_grid(const angelo_grid_t *in, Grid *g) {
    ANGELO_REQUIRE(in != nullptr, "march: null grid");
    for (int d = 0; d < 3; ++d) {
        g->lo[d] = in->roi[d];
        g->hi[d] = in->roi[3 + d];
        g->res[d] = in->res[d];
        ANGELO_REQUIRE(in->res[d] >= 1 && in->res[d] <= 4096, "march: grid resolution %d",
                       in->res[d]);
    }
    g->bits = in->bits;
    g->pow2_ext = g->pow2_res = 0;
    for (int d = 0; d < 3; ++d) {
        // the same float32 subtraction as the device's; a power of two has
        // mantissa 0.5 under frexpf
        const float ext = g->hi[d] - g->lo[d];
        int e = 0;
        g->inv_ext[d] = g->inv_res[d] = 0.f;
        if (std::isfinite(ext) && ext > 0.f && std::frexp(ext, &e) == 0.5f && e - 1 >= -126 && e - 1 <= 126) {
            g->pow2_ext |= 1 << d;
            g->inv_ext[d] = std::ldexp(1.0f, 1 - e);
        }
        const float r = (float)g->res[d];
        if (std::frexp(r, &e) == 0.5f) {
            g->pow2_res |= 1 << d;
            g->inv_res[d] = std::ldexp(1.0f, 1 - e);
        }
    }
    ANGELO_REQUIRE(in->contraction == ANGELO_CONTRACT_AABB || in->contraction == ANGELO_CONTRACT_UNBOUNDED_SPHERE,
                   "march: contraction %d", in->contraction);
    g->contraction = in->contraction;
    return ANGELO_OK;
}

}  // namespace

extern "C" int angelo_ray_aabb(const float *rays_o, const float *rays_d, int64_t n,
                               const float *aabb6, float *t_min, float *t_max, void *stream) {
    ANGELO_REQUIRE(n >= 0, "ray_aabb: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && aabb6 && t_min && t_max, "ray_aabb: null pointer");
    ray_aabb_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(rays_o, rays_d, n, aabb6,
                                                                      t_min, t_max);
    return check_launch("ray_aabb");
}

extern "C" int angelo_march_count(const float *rays_o, const float *rays_d, const float *t_min,
                                  const float *t_max, int64_t n_rays, const angelo_grid_t *grid,
                                  float step, float cone_angle, int64_t max_steps, int32_t *counts,
                                  int32_t *status, void *stream) {
    Grid g;
    if (int e = make_grid(grid, &g)) return e;
    ANGELO_REQUIRE(n_rays >= 0 && step > 0.f && max_steps > 0, "march_count: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && t_min && t_max && counts, "march_count: null pointer");
    const bool warp = g.contraction != ANGELO_CONTRACT_AABB;
    if (warp)
        march_count_kernel<32><<<blocks_for(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, counts, status);
    else
        march_count_kernel<kAabbLanes><<<blocks_for(n_rays * kAabbLanes, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, counts, status);
    return check_launch("march_count");
}

extern "C" int64_t angelo_scan_workspace_size(int64_t n) {
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    return (tiles + 1) * (int64_t)sizeof(int64_t);
}

extern "C" int angelo_scan(const int32_t *counts, int64_t n, int64_t *offsets, void *workspace,
                           void *stream) {
    ANGELO_REQUIRE(n >= 0 && offsets && workspace, "scan: bad arguments");
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        if (cudaMemsetAsync(offsets, 0, sizeof(int64_t), s) != cudaSuccess)
            return check_launch("scan(memset)");
        return ANGELO_OK;
    }
    ANGELO_REQUIRE(counts != nullptr, "scan: null counts");
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    int64_t *sums = reinterpret_cast<int64_t *>(workspace);
    scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(counts, n, offsets, sums);
    scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, tiles, offsets + n);
    scan_add_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(offsets, n, sums);
    return check_launch("scan");
}

extern "C" int angelo_march_fill(const float *rays_o, const float *rays_d, const float *t_min,
                                 const float *t_max, int64_t n_rays, const angelo_grid_t *grid,
                                 float step, float cone_angle, int64_t max_steps,
                                 const int64_t *offsets, int64_t capacity, int32_t *ray_indices,
                                 float *t_starts, float *t_ends, int32_t *status, void *stream) {
    Grid g;
    if (int e = make_grid(grid, &g)) return e;
    ANGELO_REQUIRE(n_rays >= 0 && step > 0.f && max_steps > 0 && capacity >= 0,
                   "march_fill: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && t_min && t_max && offsets, "march_fill: null pointer");
    ANGELO_REQUIRE(capacity == 0 || (ray_indices && t_starts && t_ends), "march_fill: null output");
    const bool warp = g.contraction != ANGELO_CONTRACT_AABB;
    if (warp)
        march_fill_kernel<32><<<blocks_for(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, offsets, capacity,
        ray_indices, t_starts, t_ends, status);
    else
        march_fill_kernel<kAabbLanes><<<blocks_for(n_rays * kAabbLanes, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, offsets, capacity,
        ray_indices, t_starts, t_ends, status);
    return check_launch("march_fill");
}

extern "C" int angelo_march_record(const float *rays_o, const float *rays_d, const float *t_min,
                                   const float *t_max, int64_t n_rays, const angelo_grid_t *grid,
                                   float step, float cone_angle, int64_t max_steps, int32_t per_ray,
                                   float *scratch, int32_t *counts, int32_t *status, void *stream) {
    Grid g;
    if (int e = make_grid(grid, &g)) return e;
    ANGELO_REQUIRE(n_rays >= 0 && step > 0.f && max_steps > 0 && per_ray > 0, "march_record: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && t_min && t_max && counts && scratch && status,
                   "march_record: null pointer");
    ANGELO_REQUIRE((reinterpret_cast<uintptr_t>(scratch) & 7) == 0, "march_record: scratch alignment");
    const bool warp = g.contraction != ANGELO_CONTRACT_AABB;
    if (warp)
        march_record_kernel<32><<<blocks_for(n_rays * 32, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, per_ray,
        reinterpret_cast<float2 *>(scratch), counts, status);
    else
        march_record_kernel<kAabbLanes><<<blocks_for(n_rays * kAabbLanes, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, t_min, t_max, n_rays, g, step, cone_angle, max_steps, per_ray,
        reinterpret_cast<float2 *>(scratch), counts, status);
    return check_launch("march_record");
}

extern "C" int angelo_march_compact(const float *scratch, int32_t per_ray, const int32_t *counts,
                                    const int64_t *offsets, int64_t n_rays, int64_t capacity,
                                    int32_t *ray_indices, float *t_starts, float *t_ends, int32_t *status,
                                    void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && per_ray > 0 && capacity >= 0, "march_compact: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(scratch && counts && offsets, "march_compact: null pointer");
    ANGELO_REQUIRE(capacity == 0 || (ray_indices && t_starts && t_ends), "march_compact: null output");
    ANGELO_REQUIRE(n_rays < (1LL << 31), "march_compact: too many rays");
    march_compact_kernel<<<(unsigned)n_rays, 128, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2 *>(scratch), per_ray, counts, offsets, capacity, ray_indices, t_starts,
        t_ends, status);
    return check_launch("march_compact");
}

// Offsets of a fill into a fixed sample capacity, clamped to that capacity:
// the fill drops every sample at or past `capacity`, so a consumer that walks
// [offsets[r], offsets[r+1]) must not walk past it either.
__global__ void offsets_clamp_kernel(int64_t *offsets, int64_t n, int64_t capacity) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && offsets[i] > capacity) offsets[i] = capacity;
}

extern "C" int angelo_offsets_clamp(int64_t *offsets, int64_t n_rays, int64_t capacity, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && capacity >= 0, "offsets_clamp: bad arguments");
    ANGELO_REQUIRE(offsets != nullptr, "offsets_clamp: null offsets");
    const int64_t n = n_rays + 1;
    offsets_clamp_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(offsets, n, capacity);
    return check_launch("offsets_clamp");
}

// ------------------------------------------------ learned background samples
// The background's sample points and its visibility test (models/neus.py:
// 141-170 with nerfacc's sigma_fn), each one launch instead of a chain of
// elementwise ops: the points in the order of the reference's torch ops, the
// visibility with the sequential float32 transmittance of the foreground's
// weights kernel, and the kept samples (a prefix of each ray) compacted by
// their scanned counts.

namespace {

// world point o + d (t0 + t1) / 2 of sample j (the reference's
// positions = t_origins + t_dirs * midpoints, models/neus.py:222-226, in its
// order of float32 operations); with a radius, its contraction to the
// radius-2 ball in [0, 1]^3 (UN_BOUNDED_SPHERE, models/geometry.py:22-28):
// [-r, r]^3 -> [-1, 1]^3, |x| > 1 -> (2 - 1/|x|) x/|x|, then x / 4 + 1/2;
// the midpoint too where mids is given
__global__ void sample_points_kernel(const float *__restrict__ ro, const float *__restrict__ rd,
                                     const int32_t *__restrict__ ri, const float *__restrict__ t0,
                                     const float *__restrict__ t1, int64_t n, float radius,
                                     float *__restrict__ pts, float *__restrict__ mids) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int64_t r = ri[j];
    const float mid = __fmul_rn(__fadd_rn(t0[j], t1[j]), 0.5f);
    if (mids) mids[j] = mid;
    float x[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) x[k] = __fadd_rn(ro[r * 3 + k], __fmul_rn(rd[r * 3 + k], mid));
    if (radius > 0.f) {
        const float two_r = __fsub_rn(radius, -radius);
#pragma unroll
        for (int k = 0; k < 3; ++k) x[k] = __fsub_rn(__fmul_rn(__fdiv_rn(__fsub_rn(x[k], -radius), two_r), 2.0f), 1.0f);
        const float mag = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x[0], x[0]), __fmul_rn(x[1], x[1])),
                                               __fmul_rn(x[2], x[2])));
        if (mag > 1.0f) {
            const float sc = __fsub_rn(2.0f, __fdiv_rn(1.0f, mag));
#pragma unroll
            for (int k = 0; k < 3; ++k) x[k] = __fmul_rn(sc, __fdiv_rn(x[k], mag));
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) x[k] = __fadd_rn(__fdiv_rn(x[k], 4.0f), 0.5f);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) pts[j * 3 + k] = x[k];
}

// per ray: density exp(out0 + bias) (trunc_exp), alpha = 1 - exp(-density dt),
// transmittance T by the sequential product (held once below eps); the count
// of samples with T >= eps (a prefix of the ray)
__global__ void bg_visibility_kernel(const float *__restrict__ out, int64_t out_stride, float bias,
                                     const float *__restrict__ t0, const float *__restrict__ t1,
                                     const int64_t *__restrict__ off, int64_t n_rays, float eps,
                                     int32_t *__restrict__ kept) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    float T = 1.0f;
    int32_t k = 0;
    for (int64_t j = off[r]; j < off[r + 1]; ++j) {
        if (T < eps) break;
        ++k;
        const float sigma = expf(__fadd_rn(out[j * out_stride], bias));
        const float a = __fsub_rn(1.0f, expf(-__fmul_rn(sigma, __fsub_rn(t1[j], t0[j]))));
        T = __fmul_rn(T, __fsub_rn(1.0f, a));
    }
    kept[r] = k;
}

// the kept samples (the first kept[r] of ray r) at their scanned offsets:
// ray index, t0, t1, contracted point, the MLP output row and the row index
// into the visibility pass's arrays
__global__ void bg_compact_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ kept,
                                  const int64_t *__restrict__ koff, int64_t n_rays,
                                  const int32_t *__restrict__ ri, const float *__restrict__ t0,
                                  const float *__restrict__ t1, const float *__restrict__ pts,
                                  const float *__restrict__ out, int32_t out_dim,
                                  int32_t *__restrict__ ri_k, float *__restrict__ t0_k,
                                  float *__restrict__ t1_k, float *__restrict__ pts_k,
                                  float *__restrict__ out_k, int32_t *__restrict__ rows_k) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n_rays) return;
    const int64_t src = off[r], dst = koff[r];
    for (int i = lane; i < kept[r]; i += 32) {
        const int64_t a = src + i, b = dst + i;
        ri_k[b] = ri[a];
        t0_k[b] = t0[a];
        t1_k[b] = t1[a];
        rows_k[b] = (int32_t)a;
#pragma unroll
        for (int k = 0; k < 3; ++k) pts_k[b * 3 + k] = pts[a * 3 + k];
        for (int c = 0; c < out_dim; ++c) out_k[b * out_dim + c] = out[a * out_dim + c];
    }
}

}  // namespace

extern "C" int angelo_bg_points(const float *rays_o, const float *rays_d, const int32_t *ray_indices,
                                const float *t_starts, const float *t_ends, int64_t n, float radius,
                                float *points, void *stream) {
    ANGELO_REQUIRE(n >= 0 && radius > 0.f, "bg_points: bad arguments");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && ray_indices && t_starts && t_ends && points, "bg_points: null pointer");
    sample_points_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(
        rays_o, rays_d, ray_indices, t_starts, t_ends, n, radius, points, nullptr);
    return check_launch("bg_points");
}

extern "C" int angelo_sample_points(const float *rays_o, const float *rays_d, const int32_t *ray_indices,
                                    const float *t_starts, const float *t_ends, int64_t n, float *points,
                                    float *midpoints, void *stream) {
    ANGELO_REQUIRE(n >= 0, "sample_points: bad arguments");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && ray_indices && t_starts && t_ends && points, "sample_points: null pointer");
    sample_points_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(
        rays_o, rays_d, ray_indices, t_starts, t_ends, n, 0.f, points, midpoints);
    return check_launch("sample_points");
}

extern "C" int angelo_bg_visibility(const float *out, int64_t out_stride, float density_bias,
                                    const float *t_starts, const float *t_ends, const int64_t *offsets,
                                    int64_t n_rays, float early_stop_eps, int32_t *kept, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && out_stride >= 1, "bg_visibility: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(out && t_starts && t_ends && offsets && kept, "bg_visibility: null pointer");
    bg_visibility_kernel<<<blocks_for(n_rays, 128), 128, 0, as_stream(stream)>>>(
        out, out_stride, density_bias, t_starts, t_ends, offsets, n_rays, early_stop_eps, kept);
    return check_launch("bg_visibility");
}

extern "C" int angelo_bg_compact(const int64_t *offsets, const int32_t *kept, const int64_t *kept_offsets,
                                 int64_t n_rays, const int32_t *ray_indices, const float *t_starts,
                                 const float *t_ends, const float *points, const float *out, int32_t out_dim,
                                 int32_t *ray_indices_k, float *t_starts_k, float *t_ends_k, float *points_k,
                                 float *out_k, int32_t *rows_k, void *stream) {
    ANGELO_REQUIRE(n_rays >= 0 && out_dim >= 1, "bg_compact: bad arguments");
    if (n_rays == 0) return ANGELO_OK;
    ANGELO_REQUIRE(offsets && kept && kept_offsets && ray_indices && t_starts && t_ends && points && out,
                   "bg_compact: null input");
    ANGELO_REQUIRE(n_rays < (1ll << 26), "bg_compact: too many rays");
    bg_compact_kernel<<<blocks_for(n_rays * 32, 256), 256, 0, as_stream(stream)>>>(
        offsets, kept, kept_offsets, n_rays, ray_indices, t_starts, t_ends, points, out, out_dim, ray_indices_k,
        t_starts_k, t_ends_k, points_k, out_k, rows_k);
    return check_launch("bg_compact");
}
