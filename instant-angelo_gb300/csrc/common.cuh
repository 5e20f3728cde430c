// Shared helpers of libangelo_gb.so: status codes, error string, launch
// checks and the per-level hash-grid arithmetic used by several kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

#include "angelo_gb.h"

namespace angelo {

// Thread-local message behind angelo_last_error_string().
void set_error(const char *fmt, ...);

inline int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return ANGELO_E_CUDA;
    }
    return ANGELO_OK;
}

#define ANGELO_REQUIRE(cond, ...)          \
    do {                                   \
        if (!(cond)) {                     \
            ::angelo::set_error(__VA_ARGS__); \
            return ANGELO_E_INVALID;       \
        }                                  \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned blocks_for(int64_t n, int threads) {
    return (unsigned)((n + threads - 1) / threads);
}

// Launch configuration of a persistent kernel with `smem` bytes of dynamic
// shared memory, set up once per device (attributes, occupancy, SM count)
// and reused by later launches on that device.
struct PersistentLaunch {
    int device = -1;
    int per_sm = 0;
    int sms = 0;
};

template <typename K>
inline int persistent_setup(K kernel, size_t smem, int threads, PersistentLaunch &c, const char *what) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch(what);
    if (c.device == dev) return ANGELO_OK;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess)
        return check_launch(what);
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (per_sm < 1) {
        set_error("%s: %zu bytes of shared memory do not fit an SM", what, smem);
        return ANGELO_E_UNSUPPORTED;
    }
    c.per_sm = per_sm;
    c.sms = sms > 0 ? sms : 1;
    c.device = dev;
    return ANGELO_OK;
}

// ------------------------------------------------------------- hash grid math
//
// tcnn HashGrid per-level arithmetic for 3 input dims (the reference's
// tcnn.Encoding at models/network_utils.py:47):
//   pos = fmaf(scale, x, 0.5); cell = (uint32)(int)floor(pos); frac = pos - floor
//   corner c (bit d set = +1 along dim d), weight = prod_d (bit ? frac : 1-frac)
//   index = dense x + y*res + z*res^2 while the stride fits the level, else
//           x*1 ^ y*2654435761 ^ z*805459861; then mod the level size.

__device__ __forceinline__ uint32_t grid_index(uint32_t hashmap_size, uint32_t res, uint32_t g0,
                                               uint32_t g1, uint32_t g2) {
    uint32_t stride = 1, index = 0;
    const uint32_t g[3] = {g0, g1, g2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (stride <= hashmap_size) {
            index += g[d] * stride;
            stride *= res;
        }
    }
    // The dense loop above stops adding once stride exceeds the level size,
    // exactly where the reference's loop condition stops.
    if (hashmap_size < stride) index = (g0 * 1u) ^ (g1 * 2654435761u) ^ (g2 * 805459861u);
    // index % hashmap_size without the integer division: hashed levels have a
    // power-of-two size; dense indices of points inside [0,1] stay below twice
    // the level size (level sizes are at most 2^30)
    if ((hashmap_size & (hashmap_size - 1u)) == 0u) return index & (hashmap_size - 1u);
    if (index < hashmap_size) return index;
    if (index < 2u * hashmap_size) return index - hashmap_size;
    return index % hashmap_size;
}

struct LevelPos {
    uint32_t g[3];
    float f[3];
};

__device__ __forceinline__ LevelPos level_pos(float x0, float x1, float x2, float scale) {
    LevelPos p;
    const float xs[3] = {x0, x1, x2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float pos = __fmaf_rn(scale, xs[d], 0.5f);
        const float fl = floorf(pos);
        p.g[d] = (uint32_t)(int32_t)fl;
        p.f[d] = __fsub_rn(pos, fl);
    }
    return p;
}

// Weight of corner c, multiplied in tcnn's order (dim 0, 1, 2) with no
// contraction so the float32 result is reproducible on the host.
__device__ __forceinline__ float corner_weight(const LevelPos &p, int c) {
    float w = 1.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) w = __fmul_rn(w, (c >> d) & 1 ? p.f[d] : __fsub_rn(1.0f, p.f[d]));
    return w;
}

__device__ __forceinline__ uint32_t corner_index(const angelo_hashgrid_layout_t &lay, int l,
                                                 const LevelPos &p, int c) {
    const uint32_t hs = lay.offsets[l + 1] - lay.offsets[l];
    return grid_index(hs, lay.resolutions[l], p.g[0] + (c & 1), p.g[1] + ((c >> 1) & 1),
                      p.g[2] + ((c >> 2) & 1));
}

// Warp-aggregated float2 atomic add into a hash table.  The lanes of one
// group (lane % STRIDE equal) are visited in lane order; a run of consecutive
// group lanes with the same entry is summed by a segmented suffix scan and
// only the run's first lane issues the atomic.  Consecutive samples along a
// ray fall into the same coarse cells, so at coarse levels a run covers most
// of the group.  Every lane of the warp must call this (warp-collective).
template <int STRIDE>
__device__ __forceinline__ void aggregated_add2(float2 *table, uint64_t entry, float v0, float v1,
                                                bool active) {
    const int lane = threadIdx.x & 31;
    const uint64_t key = active ? entry : ~0ull;
    const uint64_t prev = __shfl_up_sync(0xffffffffu, key, STRIDE);
    const bool head = lane < STRIDE || prev != key;
    const uint32_t heads = __ballot_sync(0xffffffffu, head);
    uint32_t group = 0;
#pragma unroll
    for (int i = 0; i < 32; i += STRIDE) group |= 1u << i;
    group <<= (lane % STRIDE);
    const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
    const int run = __popc(heads & group & upto);
#pragma unroll
    for (int o = STRIDE; o < 32; o <<= 1) {
        const float a = __shfl_down_sync(0xffffffffu, v0, o);
        const float b = __shfl_down_sync(0xffffffffu, v1, o);
        const int r2 = __shfl_down_sync(0xffffffffu, run, o);
        if (lane + o < 32 && r2 == run) {
            v0 += a;
            v1 += b;
        }
    }
    if (active && head && (v0 != 0.0f || v1 != 0.0f)) atomicAdd(table + entry, make_float2(v0, v1));
}

__device__ __forceinline__ float2 load_entry(const void *table, int dtype, uint64_t entry) {
    if (dtype == ANGELO_DTYPE_F32) {
        return __ldg(reinterpret_cast<const float2 *>(table) + entry);
    }
    const __half2 h = __ldg(reinterpret_cast<const __half2 *>(table) + entry);
    return __half22float2(h);
}

}  // namespace angelo
