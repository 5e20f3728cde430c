// Allocation-free variant of angelo_scan (march.cu): the exclusive prefix sum
// that turns per-ray sample counts into packed sample offsets.
//
// Who needs it: a caller that must not allocate device memory at all -- for
// example a host application that hands this library only pre-sized input and
// output buffers from its own fixed memory pool, or code running where a
// cudaMalloc would synchronise the device or is not permitted -- cannot
// provide the workspace angelo_scan asks for.  This entry point keeps that
// workspace in a fixed array inside the library instead.
//
// Limits and behaviour (also stated in include/angelo_gb.h):
//   * at most ANGELO_SCAN_NOALLOC_MAX_N = 2^24 counts per call; larger inputs
//     are rejected with ANGELO_E_INVALID and a message, nothing is launched;
//   * the workspace is one file-scope __device__ array of 16385 int64 values
//     (128 KiB); every GPU that loads the library holds it until the process
//     exits;
//   * all calls share that array: two calls whose kernels overlap on the GPU
//     (different streams, or different host threads without ordering) race
//     and may both return wrong offsets; order them on one stream;
//   * the array keeps whatever the last call wrote; the kernels below write
//     every slot they read before reading it, so nothing needs clearing;
//   * every call made outside stream capture looks up the array's device
//     address (cudaGetSymbolAddress) with the calling device current; a
//     call under capture reuses the address of that device's last uncaptured
//     call, so the first call on a device must come before any stream
//     capture (a first call under capture is refused with ANGELO_E_INVALID).
// Nothing here calls cudaMalloc, cudaFree or any allocating library routine.
#include <mutex>

#include "common.cuh"

using namespace angelo;

namespace {

constexpr int kThreadsNA = 256;
constexpr int kItemsNA = 4;
constexpr int kTileNA = kThreadsNA * kItemsNA;
constexpr int64_t kMaxN = ANGELO_SCAN_NOALLOC_MAX_N;
constexpr int64_t kMaxTiles = kMaxN / kTileNA;  // 16384

// tile sums (kMaxTiles) + grand total slot
static __device__ __align__(256) int64_t g_noalloc_scan_ws[kMaxTiles + 1];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
int64_t *g_ws_ptr[kMaxDevices] = {};

__device__ __forceinline__ int64_t block_scan_na(int64_t v, int64_t *total) {
    __shared__ int64_t sums[kThreadsNA / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t s = lane < kThreadsNA / 32 ? sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kThreadsNA / 32) sums[lane] = s;
    }
    __syncthreads();
    const int64_t before = warp > 0 ? sums[warp - 1] : 0;
    *total = sums[kThreadsNA / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kThreadsNA) na_tiles(const int32_t *__restrict__ in, int64_t n,
                                                       int64_t *__restrict__ out, int64_t *ws) {
    const int64_t base = (int64_t)blockIdx.x * kTileNA + threadIdx.x * kItemsNA;
    int64_t v[kItemsNA];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kItemsNA; ++k) {
        v[k] = base + k < n ? (int64_t)in[base + k] : 0;
        s += v[k];
    }
    int64_t total;
    int64_t run = block_scan_na(s, &total);
#pragma unroll
    for (int k = 0; k < kItemsNA; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) ws[blockIdx.x] = total;  // every slot later read is written here
}

__global__ void __launch_bounds__(kThreadsNA) na_sums(int64_t *ws, int64_t n_tiles,
                                                      int64_t *__restrict__ grand) {
    int64_t carry = 0;
    for (int64_t start = 0; start < n_tiles; start += kThreadsNA) {
        const int64_t i = start + threadIdx.x;
        const int64_t v = i < n_tiles ? ws[i] : 0;
        int64_t total;
        const int64_t ex = block_scan_na(v, &total);
        if (i < n_tiles) ws[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kThreadsNA) na_add(int64_t *__restrict__ out, int64_t n,
                                                     const int64_t *ws) {
    const int64_t base = (int64_t)blockIdx.x * kTileNA;
    const int64_t add = ws[blockIdx.x];
    for (int k = threadIdx.x; k < kTileNA; k += kThreadsNA)
        if (base + k < n) out[base + k] += add;
}

// Device address of the workspace for the current device.  Looked up on
// every call that is not being captured into a graph (a lookup is cheap, and
// a context torn down and re-created, e.g. by cudaDeviceReset, may place the
// array elsewhere); a call under stream capture uses the address of the
// device's last uncaptured call, so the first call on a device must come
// before any capture.
int workspace_for_current_device(cudaStream_t s, int64_t **ws) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return check_launch("scan_noalloc(cudaGetDevice)");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess)
        return check_launch("scan_noalloc(cudaStreamIsCapturing)");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (cap != cudaStreamCaptureStatusNone && g_ws_ptr[dev] == nullptr) {
        set_error("scan_noalloc: the first call on device %d is under stream capture; "
                  "call it once outside capture first", dev);
        return ANGELO_E_INVALID;
    }
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_ws);
        if (e != cudaSuccess || p == nullptr) {
            set_error("scan_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return ANGELO_E_CUDA;
        }
        g_ws_ptr[dev] = reinterpret_cast<int64_t *>(p);
    }
    *ws = g_ws_ptr[dev];
    return ANGELO_OK;
}

}  // namespace

extern "C" int angelo_scan_noalloc(const int32_t *counts, int64_t n, int64_t *offsets,
                                   void *stream) {
    ANGELO_REQUIRE(n >= 0 && offsets != nullptr, "scan_noalloc: bad arguments");
    ANGELO_REQUIRE(n <= kMaxN,
                   "scan_noalloc: %lld counts exceed the fixed workspace limit of %lld; "
                   "use angelo_scan with a caller-provided workspace",
                   (long long)n, (long long)kMaxN);
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        if (cudaMemsetAsync(offsets, 0, sizeof(int64_t), s) != cudaSuccess)
            return check_launch("scan_noalloc(memset)");
        return ANGELO_OK;
    }
    ANGELO_REQUIRE(counts != nullptr, "scan_noalloc: null counts");
    int64_t *ws = nullptr;
    if (int e = workspace_for_current_device(s, &ws)) return e;
    const int64_t tiles = (n + kTileNA - 1) / kTileNA;
    na_tiles<<<(unsigned)tiles, kThreadsNA, 0, s>>>(counts, n, offsets, ws);
    na_sums<<<1, kThreadsNA, 0, s>>>(ws, tiles, offsets + n);
    na_add<<<(unsigned)tiles, kThreadsNA, 0, s>>>(offsets, n, ws);
    return check_launch("scan_noalloc");
}
