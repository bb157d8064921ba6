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

#include "swe_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

const char *swe_mlp_last_error(void);

/* Parameters: W1[64][6], b1[64], W2[64][64], b2[64], W3[64][64], b3[64],
 * W4[4][64], b4[4] (row-major, rows = output neurons), FP32. */
#define SWE_MLP_NPARAMS 9028
int swe_mlp_param_count(void);

/* Edge arrays are structure-of-arrays host memory of n edges each:
 *   edges   = hL[n] hR[n] huL[n] huR[n] bL[n] bR[n]  (the argument order of
 *             solver::X<float>::computeNetUpdates at the reference's call
 *             sites, normal momentum)
 *   targets = hUpdL[n] hUpdR[n] huUpdL[n] huUpdR[n]  (net updates to learn)
 *   outputs = o0[n] o1[n] o2[n] o3[n]  (raw network outputs: speed
 *             corrections of the two waves in units of sqrt(g h), predicted
 *             strengths in units of h sqrt(g h)) */
typedef struct swe_mlp swe_mlp;

/* New surrogate on the current device: Glorot-uniform hidden weights from
 * `seed`, zero biases and a zero last layer (the untrained surrogate is the
 * f-wave solver with Roe speeds).  Allocates its device state. */
int swe_mlp_create(unsigned long long seed, swe_mlp **out);
void swe_mlp_destroy(swe_mlp *m);
int swe_mlp_get_params(swe_mlp *m, float *params);
/* SMs of the device and resident CTAs per SM of the inference kernels (each
 * holds 64 of the SM's 512 TMEM columns). */
int swe_mlp_launch_shape(swe_mlp *m, int *sms, int *forward_ctas_per_sm);
/* Sets the FP32 master parameters and clears the optimiser state. */
int swe_mlp_set_params(swe_mlp *m, const float *params);

/* Raw network outputs (BF16 operands, FP32 accumulation) of n edges. */
int swe_mlp_forward(swe_mlp *m, int n, const float *edges, float *outputs);

/* Surrogate solve of n edges: net updates (4 x n, same order as targets),
 * maximum wave speed, and used[e] = 1 where the surrogate's gate accepted
 * the edge, 0 where the augmented Riemann solver computed it instead (a side
 * shallower than 0.1 m, waves closer than 0.5 sqrt(g h), or predicted
 * strengths inconsistent with the closure). */
int swe_mlp_solve(swe_mlp *m, int n, const float *edges, float *updates, float *speed, unsigned char *used);

/* Mean training loss over n edges and its gradient (SWE_MLP_NPARAMS floats). */
int swe_mlp_loss_grad(swe_mlp *m, int n, const float *edges, const float *targets, float *loss, float *grad);

/* Adam training (beta 0.9 / 0.999, eps 1e-8) for `epochs` passes over the n
 * edges in shuffled mini-batches of `batch`; epoch_loss (may be NULL) gets the
 * mean loss of each epoch, measured during the pass. */
int swe_mlp_train(swe_mlp *m, int n, const float *edges, const float *targets, int epochs, int batch, float lr,
                  unsigned long long seed, float *epoch_loss);

/* The surrogate on a domain of swe_gb300.h (unsplit semantics, no local time
 * stepping).  Each of the nsteps steps runs setGhostLayer, an edge pass that
 * stores the net updates of every edge (the surrogate where its gate accepts,
 * the augmented Riemann solver elsewhere), the dt of each dt group from the
 * max wave speed (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456) and the
 * unsplit cell update (:458-492); the call ends with setGhostLayer of the
 * new state, as a regular step leaves it.  m == NULL runs the augmented solver on every
 * edge through the same kernels: bit-identical to steps of a domain created
 * with SWE_SOLVER_AUGRIE.  Like a regular step, groups whose time has reached
 * their advance target (swe_gpu_advance) sit the step out.
 * *surrogate_edges (may be NULL; the call then waits) counts the edges the
 * surrogate solved over the call.  Allocates the edge buffers (8 floats per
 * cell) on first use. */
int swe_gpu_surrogate_step(swe_gpu_domain *d, swe_mlp *m, int nsteps, long long *surrogate_edges);
/* Edges one step solves: x-edges (nx+1) ny plus y-edges nx (ny+1), all blocks. */
int swe_gpu_surrogate_edge_count(swe_gpu_domain *d, long long *edges);

/* Edge-state logger: after setGhostLayer of the current state, every
 * stride-th edge of the step's edge order with both sides at least 0.1 m deep
 * (up to capacity of them, in edge order) with its augmented-solver net
 * updates: edges (room for 6 x capacity floats) and targets (4 x capacity) are
 * returned packed as 6 x count and 4 x count rows -- training data for
 * swe_mlp_train as they stand. */
int swe_gpu_log_edges(swe_gpu_domain *d, int stride, int capacity, float *edges, float *targets, int *count);

/* Tensor-core self-check, one CTA, host arrays (row-major), operands rounded
 * to BF16, FP32 accumulation:
 *   mode 0: D[128 x w2] = X[128 x w1] Y[w2 x w1]^T   (both operands K-major)
 *   mode 1: D[w1 x w2]  = X[128 x w1]^T Y[128 x w2]  (both read transposed, K = 128)
 *   mode 2: D[128 x w2] = X[128 x w1] Y[w1 x w2]     (Y read transposed)
 * D is returned as 128 x w2 (mode 1: rows >= w1 undefined).
 * w1 in {16, 32, 64}; w2 16..128, a multiple of 16. */
int swe_mlp_gemm_check(int mode, int w1, int w2, const float *x, const float *y, float *d);

#ifdef __cplusplus
}
#endif

#endif
