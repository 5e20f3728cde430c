/*
 * tc_probe.h -- C ABI of libangelo_tcprobe.so, a test-only library (built by
 * tests/native/build.py, not part of libangelo_gb.so) that pins the tcgen05
 * descriptor and tensor-memory layouts the fused MLP kernels rely on and
 * measures the issue cost of their tensor-core instruction.  No counterpart
 * in the reference.  Status codes are those of angelo_gb.h.
 */
#ifndef ANGELO_TC_PROBE_H
#define ANGELO_TC_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char *angelo_probe_last_error_string(void);

/* A (M x K) * B (N x K)^T, M = 64 or 128, on the 5th-generation tensor
 * cores (tcgen05.mma, operands in shared memory, fp32 accumulation in tensor
 * memory) with both operands split into bf16 hi/lo (three products).  D
 * (128 x W, fp32, row-major, W = N for M = 128 and 2N for M = 64) receives
 * every tensor-memory lane of the accumulator's first W columns: for M = 128
 * lane i is row i of the product.
 * a_mn_major / b_mn_major stage the operand MN-major (0: K-major); variant 0
 * is the descriptor convention the fused kernels use, 1 exchanges the
 * descriptor's two core-matrix strides (a layout self-check).  N in 16..256
 * (multiple of 16; at most 128 for M = 64), K in 16..64 (multiple of 16).
 * *status (zeroed by the caller) becomes 1 if the completion wait timed out.
 * No counterpart in the reference: it pins the layouts the fused MLP kernels
 * rely on. */
int angelo_tc_gemm_x3(const float *A, const float *B, float *D, int32_t M, int32_t N, int32_t K,
                      int32_t a_mn_major, int32_t b_mn_major, int32_t variant, int32_t *status,
                      void *stream);

/* Issue cost of the tensor-core instruction the fused MLPs are built from:
 * one thread issues n (1..4096) back-to-back tcgen05.mma of shape M x N x 16
 * (bf16, fp32 accumulation; M 64 or 128, N 16..256, multiple of 16) on
 * zero operands.  cycles[0] = SM clocks spent issuing, cycles[1] = until
 * the last product completed.  *status (zeroed by the caller) becomes 1 if
 * the completion wait timed out.  No counterpart in the reference. */
int angelo_tc_mma_rate(int32_t M, int32_t N, int32_t n, int64_t *cycles, int32_t *status,
                       void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ANGELO_TC_PROBE_H */
