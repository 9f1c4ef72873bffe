/*
 * forge_gpu_selftest.h -- test hooks of libforge_gpu.so (not part of the drop-in boundary).
 *
 * Internal steps of the engine exposed for the test suite; no reference routine corresponds to
 * them and a host application has no use for them.
 */
#ifndef FORGE_GPU_SELFTEST_H
#define FORGE_GPU_SELFTEST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* D = A B^T on the tcgen05 tensor cores with TF32 inputs and FP32 accumulation; A (batch x M x K),
 * B (batch x N x K), D (batch x M x N), all row-major fp32 host arrays. */
int forge_gpu_selftest_tc_gemm(int64_t M, int64_t N, int64_t K, int64_t batch, const float* A, const float* B,
                               float* D);

/* The same GEMM (batch 1) with a failure injected: the TMA producer issues only K block 0, so the
 * MMA issuer's wait for block 1 runs out after spin_limit polls (1..2^26); the kernel flags the
 * error, drains its copies and MMAs, frees its TMEM and returns.  Returns FORGE_ERR_TIMEOUT; the
 * context stays usable.  K must exceed 32. */
int forge_gpu_selftest_tc_gemm_timeout(int64_t M, int64_t N, int64_t K, int64_t spin_limit, const float* A,
                                       const float* B, float* D);

/* Host only: the small dense step of the window refinement.  G, S: n x n Hermitian (complex,
 * column-major, interleaved re/im doubles), n <= 32.  Returns theta (ascending) and M = L^{-H} U,
 * with S = L L^H and L^{-1} G L^{-H} = U diag(theta) U^H, so that G M = S M diag(theta) and
 * M^H S M = I.  Returns 1 if S is not positive definite. */
int forge_selftest_rr_small(int64_t n, const double* G, const double* S, double* theta, double* M);

#ifdef __cplusplus
}
#endif
#endif /* FORGE_GPU_SELFTEST_H */
