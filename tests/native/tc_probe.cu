// The tcgen05 building block of the fused MLP kernels as a callable GEMM:
// D (M x N, fp32) = A (M x K) * B (N x K)^T, M = 64 or 128, with both operands split into
// bf16 hi/lo parts in shared memory (no swizzle) and the three products
// lo*hi + hi*lo + hi*hi accumulated in tensor memory (bf16x3), one CTA of 4
// warps.  Each operand is staged K-major (8 x 8 core matrices, K contiguous)
// or MN-major (the same core matrices with M or N contiguous: the layout in
// which a row-major [sample][unit] staging buffer is the transposed operand
// of a GEMM over samples).  Used by the tests to pin the descriptor and
// accumulator layouts the fused kernels rely on.
//
// Test-only: this file builds libangelo_tcprobe.so (tests/native/build.py),
// not the product library; it reuses the product's tensor-core helpers
// (tc.cuh) so that the layouts it pins are the ones the kernels use.
#include <algorithm>
#include <cstdarg>

#include <cuda_bf16.h>

#include "common.cuh"
#include "tc.cuh"
#include "tc_probe.h"

// The probe library's own error message (common.cuh's status helpers write
// it); read with angelo_probe_last_error_string().
static thread_local char g_probe_err[512];

namespace angelo {
void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_probe_err, sizeof(g_probe_err), fmt, ap);
    va_end(ap);
}
}  // namespace angelo

extern "C" const char *angelo_probe_last_error_string(void) { return g_probe_err; }

using namespace angelo;

namespace {

constexpr uint32_t kWaitPolls = 1u << 24;

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    *hi = h;
    *lo = __float2bfloat16_rn(x - __bfloat162float(h));
}

__global__ void __launch_bounds__(128, 1)
    tc_gemm_x3_kernel(const float *__restrict__ A, const float *__restrict__ B, float *__restrict__ D, int N,
                      int K, int M, int a_mn, int b_mn, int variant, uint32_t ncols, int a_region,
                      int b_region, int *status) {
    extern __shared__ __align__(1024) char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    char *a_hi = smem, *a_lo = a_hi + a_region, *b_hi = a_lo + a_region, *b_lo = b_hi + b_region;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(b_lo + b_region);
    uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
    // K-major: element (r, k) at kmajor_offset(r, k, K); MN-major: the
    // transposed storage, kmajor_offset(k, r, rows)
    for (int i = tid; i < M * K; i += 128) {
        const int r = i / K, k = i % K;
        const uint32_t o = a_mn ? tc::kmajor_offset(k, r, M) : tc::kmajor_offset(r, k, K);
        split_bf16(A[i], reinterpret_cast<__nv_bfloat16 *>(a_hi + o), reinterpret_cast<__nv_bfloat16 *>(a_lo + o));
    }
    for (int i = tid; i < N * K; i += 128) {
        const int r = i / K, k = i % K;
        const uint32_t o = b_mn ? tc::kmajor_offset(k, r, N) : tc::kmajor_offset(r, k, K);
        split_bf16(B[i], reinterpret_cast<__nv_bfloat16 *>(b_hi + o), reinterpret_cast<__nv_bfloat16 *>(b_lo + o));
    }
    tc::fence_proxy_async_smem();
    if (warp == 0) {
        tc::tmem_alloc(slot, ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        const uint32_t id = tc::idesc_bf16_f32(M, N, a_mn, b_mn);
        // core-matrix strides: LBO along K, SBO along M (or N), for either
        // operand major; variant 1 exchanges the two fields
        const uint32_t a_k = tc::k_stride(a_mn, M, K), a_m = tc::mn_stride(a_mn, M, K);
        const uint32_t b_k = tc::k_stride(b_mn, N, K), b_m = tc::mn_stride(b_mn, N, K);
        const uint32_t a_lbo = variant == 0 ? a_k : a_m, a_sbo = variant == 0 ? a_m : a_k;
        const uint32_t b_lbo = variant == 0 ? b_k : b_m, b_sbo = variant == 0 ? b_m : b_k;
        for (int ks = 0; ks < K / 16; ++ks) {
            // one K step of 16: two K chunks (K-major) or two 8-row groups (MN-major)
            const uint32_t a_off = a_mn ? ks * 2 * (16u * (uint32_t)M) : ks * 256u;
            const uint32_t b_off = b_mn ? ks * 2 * (16u * (uint32_t)N) : ks * 256u;
            const uint64_t ah = tc::smem_desc(tc::smem_addr(a_hi) + a_off, a_lbo, a_sbo);
            const uint64_t al = tc::smem_desc(tc::smem_addr(a_lo) + a_off, a_lbo, a_sbo);
            const uint64_t bh = tc::smem_desc(tc::smem_addr(b_hi) + b_off, b_lbo, b_sbo);
            const uint64_t bl = tc::smem_desc(tc::smem_addr(b_lo) + b_off, b_lbo, b_sbo);
            tc::mma_bf16(tmem, al, bh, id, ks > 0 ? 1u : 0u);
            tc::mma_bf16(tmem, ah, bl, id, 1u);
            tc::mma_bf16(tmem, ah, bh, id, 1u);
        }
        tc::commit(mbar);
    }
    __syncwarp();
    const bool done = tc::mbar_wait(mbar, 0, kWaitPolls);
    if (!done) {
        if (lane == 0) atomicExch(status, 1);
    } else {
        // every tensor-memory lane (128 x N): for M = 128 lane i holds row i of D
        tc::fence_after_sync();
        const int row = warp * 32 + lane;
        const int width = M == 64 ? 2 * N : N;
        for (int c0 = 0; c0 < width; c0 += 16) {
            float v[16];
            tc::ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) D[(int64_t)row * width + c0 + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Bytes the tensor core may read from an operand of `rows` rows (its M or N)
// and K columns under either assignment of the two strides to LBO / SBO: the
// region is the larger extent, so that a read stays inside the operand's
// region whichever way the descriptor is interpreted.
int operand_region(int rows, int K, int mn_major) {
    const int staged = rows * K * 2;
    int swapped;
    if (mn_major)   // rows/8 MN chunks 16*rows apart, K steps of 32*rows, 2 K groups 128 apart
        swapped = (rows / 8 - 1) * 16 * rows + (K / 16 - 1) * 32 * rows + 256;
    else            // rows/8 row groups 128 apart, K steps of 256, 2 chunks 16*K apart
        swapped = (rows / 8 - 1) * 128 + (K / 16 - 1) * 256 + 16 * K + 128;
    const int r = std::max(staged, swapped);
    return (r + 1023) / 1024 * 1024;
}

// n back-to-back products M x N x 16 from one thread (operands zero, K-major,
// 16 K columns: LBO 128, SBO 256), timed with the SM clock
__global__ void __launch_bounds__(128, 1) tc_mma_rate_kernel(int M, int N, int n, long long *cycles, int *status) {
    extern __shared__ __align__(1024) char smem[];
    constexpr int kOperandBytes = 4096 + 8192;   // A: 128 x 16 bf16, B: 256 x 16 bf16
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kOperandBytes);
    uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
    for (int i = threadIdx.x * 16; i < kOperandBytes; i += 128 * 16)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x < 32) {
        tc::tmem_alloc(slot, 512);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) tc::mbar_init(mbar, 1);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    if (threadIdx.x == 0) {
        const uint64_t ad = tc::smem_desc(tc::smem_addr(smem), 128, 256);
        const uint64_t bd = tc::smem_desc(tc::smem_addr(smem + 4096), 128, 256);
        const uint32_t id = tc::idesc_bf16_f32(M, N);
        const long long t0 = clock64();
        for (int i = 0; i < n; ++i) tc::mma_bf16(tmem, ad, bd, id, i > 0 ? 1u : 0u);
        const long long t1 = clock64();
        tc::commit(mbar);
        const bool done = tc::mbar_wait(mbar, 0, kWaitPolls);
        cycles[0] = t1 - t0;
        cycles[1] = clock64() - t0;
        if (!done) atomicExch(status, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 512);
}

}  // namespace

extern "C" int angelo_tc_mma_rate(int32_t M, int32_t N, int32_t n, int64_t *cycles, int32_t *status,
                                  void *stream) {
    ANGELO_REQUIRE(cycles && status, "tc_mma_rate: null pointer");
    ANGELO_REQUIRE(M == 64 || M == 128, "tc_mma_rate: M %d (64 or 128)", M);
    ANGELO_REQUIRE(N >= 16 && N <= 256 && N % 16 == 0, "tc_mma_rate: N %d", N);
    ANGELO_REQUIRE(n >= 1 && n <= 4096, "tc_mma_rate: n %d", n);
    const int smem = 4096 + 8192 + 64;
    if (cudaFuncSetAttribute(tc_mma_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return check_launch("tc_mma_rate(smem attribute)");
    tc_mma_rate_kernel<<<1, 128, smem, as_stream(stream)>>>(M, N, n, reinterpret_cast<long long *>(cycles),
                                                           status);
    return check_launch("tc_mma_rate");
}

extern "C" int angelo_tc_gemm_x3(const float *A, const float *B, float *D, int32_t M, int32_t N,
                                 int32_t K, int32_t a_mn_major, int32_t b_mn_major, int32_t variant,
                                 int32_t *status, void *stream) {
    ANGELO_REQUIRE(A && B && D && status, "tc_gemm_x3: null pointer");
    ANGELO_REQUIRE(M == 64 || M == 128, "tc_gemm_x3: M %d (64 or 128)", M);
    ANGELO_REQUIRE(M == 128 || N <= 128, "tc_gemm_x3: N %d > 128 with M = 64", N);
    ANGELO_REQUIRE(N >= 16 && N <= 256 && N % 16 == 0, "tc_gemm_x3: N %d (16..256, multiple of 16)", N);
    ANGELO_REQUIRE(K >= 16 && K <= 64 && K % 16 == 0, "tc_gemm_x3: K %d (16..64, multiple of 16)", K);
    ANGELO_REQUIRE(variant == 0 || variant == 1, "tc_gemm_x3: variant %d", variant);
    ANGELO_REQUIRE((a_mn_major | b_mn_major) >= 0 && a_mn_major <= 1 && b_mn_major <= 1,
                   "tc_gemm_x3: operand majors");
    uint32_t ncols = 32;
    while (ncols < (uint32_t)(M == 64 ? 2 * N : N)) ncols <<= 1;
    const int a_region = operand_region(M, K, a_mn_major);
    const int b_region = operand_region(N, K, b_mn_major);
    const size_t smem = (size_t)2 * a_region + (size_t)2 * b_region + 64;
    ANGELO_REQUIRE(smem <= 227 * 1024, "tc_gemm_x3: %zu bytes of shared memory", smem);
    if (cudaFuncSetAttribute(tc_gemm_x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return check_launch("tc_gemm_x3(smem attribute)");
    tc_gemm_x3_kernel<<<1, 128, smem, as_stream(stream)>>>(A, B, D, N, K, M, a_mn_major, b_mn_major,
                                                           variant, ncols, a_region, b_region, status);
    return check_launch("tc_gemm_x3");
}
