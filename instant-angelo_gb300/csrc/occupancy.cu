// Occupancy-grid EMA update and bit packing (nerfacc 0.3.3 OccupancyGrid._update
// reached from models/neus.py:108-109).  The reference assigns
// occs[idx] = max(occs[idx]*decay, occ) with duplicate indices resolved by
// whichever write lands last; here duplicates are resolved by their maximum
// (the scatter-max the reference's own comment describes), and the mean that
// sets the threshold is summed in a fixed order, which makes the update
// deterministic.
#include "common.cuh"

using namespace angelo;

namespace {

// Workspace: n_cells int32 "new value" slots (bit pattern of a float >= 0,
// or -1 for untouched), one double for the sum, then one double per block of
// the EMA pass (its partial sum).  The partials are added in block order by
// one block, so the mean, and with it the threshold, is the same on every
// run.
constexpr int kOccThreads = 256;

__global__ void occ_clear_kernel(int32_t *upd, int64_t n_cells) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_cells) upd[i] = -1;
}

__global__ void occ_scatter_kernel(const int64_t *__restrict__ cells, const float *__restrict__ occ,
                                   int64_t k, int64_t n_cells, int32_t *upd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    const int64_t c = cells[i];
    if (c < 0 || c >= n_cells) return;
    // alpha values are clipped to [0, 1]: their float bits order like ints
    const float v = fmaxf(occ[i], 0.0f);
    atomicMax(upd + c, __float_as_int(v));
}

__global__ void __launch_bounds__(kOccThreads) occ_ema_kernel(float *__restrict__ occs,
                                                              const int32_t *__restrict__ upd,
                                                              int64_t n_cells, float decay,
                                                              double *partial) {
    __shared__ double part[8];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n_cells) {
        float o = occs[i];
        const int32_t u = upd[i];
        if (u >= 0) {
            o = fmaxf(o * decay, __int_as_float(u));
            occs[i] = o;
        }
        v = (double)o;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += part[w];
        partial[blockIdx.x] = t;
    }
}

// One block: thread j adds partials j, j + 256, ... in order, then a fixed
// tree over the 256 thread sums.
__global__ void __launch_bounds__(kOccThreads) occ_sum_kernel(const double *__restrict__ partial,
                                                              int64_t n_part, double *sum) {
    __shared__ double t[kOccThreads];
    double v = 0.0;
    for (int64_t j = threadIdx.x; j < n_part; j += kOccThreads) v += partial[j];
    t[threadIdx.x] = v;
    __syncthreads();
    for (int w = kOccThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) t[threadIdx.x] += t[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *sum = t[0];
}

// One warp per 32 cells: ballot of occs > min(mean, thre) is one word.
__global__ void occ_pack_kernel(const float *__restrict__ occs, int64_t n_cells,
                                const double *__restrict__ sum, float thre,
                                uint32_t *__restrict__ bits) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float mean = (float)(*sum / (double)n_cells);
    const float t = mean < thre ? mean : thre;
    const bool on = i < n_cells && occs[i] > t;
    const uint32_t word = __ballot_sync(0xffffffffu, on);
    if ((threadIdx.x & 31) == 0 && i < n_cells) bits[i >> 5] = word;
}

}  // namespace

extern "C" int64_t angelo_occ_workspace_size(int64_t n_cells) {
    const int64_t blocks = (n_cells + kOccThreads - 1) / kOccThreads;
    return ((n_cells * 4 + 15) / 16) * 16 + 16 + blocks * 8;
}

extern "C" int angelo_occ_update(float *occs, int64_t n_cells, const int64_t *cells,
                                 const float *occ, int64_t k, float decay, float thre,
                                 uint32_t *bits, void *workspace, void *stream) {
    ANGELO_REQUIRE(occs && bits && workspace && n_cells > 0 && k >= 0,
                   "occ_update: bad arguments");
    ANGELO_REQUIRE(k == 0 || (cells && occ), "occ_update: null samples");
    cudaStream_t s = as_stream(stream);
    int32_t *upd = reinterpret_cast<int32_t *>(workspace);
    double *sum = reinterpret_cast<double *>(reinterpret_cast<char *>(workspace) +
                                             ((n_cells * 4 + 15) / 16) * 16);
    double *partial = sum + 2;
    const unsigned blocks = blocks_for(n_cells, kOccThreads);
    occ_clear_kernel<<<blocks, kOccThreads, 0, s>>>(upd, n_cells);
    if (k > 0) occ_scatter_kernel<<<blocks_for(k, 256), 256, 0, s>>>(cells, occ, k, n_cells, upd);
    occ_ema_kernel<<<blocks, kOccThreads, 0, s>>>(occs, upd, n_cells, decay, partial);
    occ_sum_kernel<<<1, kOccThreads, 0, s>>>(partial, blocks, sum);
    occ_pack_kernel<<<blocks, kOccThreads, 0, s>>>(occs, n_cells, sum, thre, bits);
    return check_launch("occ_update");
}
