/*
 * swe_gb300_mlp.h -- MLP surrogate of the augmented Riemann solver, on the
 * fifth-generation tensor cores of the GB300 (tcgen05, BF16 in, FP32 out).
 *
 * Same conventions as swe_gb300.h: plain C, int status (0 = OK, negative =
 * error, message via swe_mlp_last_error()).  The reference has no learned
 * solver; the surrogate stands beside the solvers of swe_gb300.h at their
 * call sites (src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410).
 */
#ifndef SWE_GB300_MLP_H
#define SWE_GB300_MLP_H

#ifdef __cplusplus
extern "C" {
#endif

const char *swe_mlp_last_error(void);

/* Tensor-core self-check: D[128 x n] = A[128 x k] * B[n x k]^T with A and B
 * rounded to BF16 and FP32 accumulation, one CTA, host arrays (row-major).
 * n: 16..128, k: 16..64, multiples of 16. */
int swe_mlp_gemm_check(int n, int k, const float *a, const float *b, float *d);

#ifdef __cplusplus
}
#endif

#endif
