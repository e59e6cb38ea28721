/*
 * icm.h -- drop-in CPU-API boundary of the GB300 ICM engine.
 *
 * Same names, signatures and argument meaning as the reference's
 * src/cpu/icm.h, so code written against the reference links against
 * libicm_gb300.so unchanged.  Here the computation runs on the GPU (sm_103a)
 * behind the same call; see icm_gpu.h for the explicit GPU API and
 * icm_gb300.h for the additions (batched tournaments, gradients, status).
 *
 * Model: Malmuth-Harville ICM by generating-function quadrature.  Player i
 * with stack S_i receives
 *   equity_i = sum_q w_q S_i a_i(q)/v_q * sum_{m<k} payout[m] [x^m] prod_{j!=i}(a_j + (1-a_j) x)
 * with a_j(q) = v_q^{S_j} over Q erfc-trapezoid nodes in probit space.
 */
#ifndef ICM_H
#define ICM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Equities for all n players.                      [reference src/cpu/icm.h:26]
 *   S[n] stacks (> 0), Q quadrature nodes (>= 1; 256 is the usual choice),
 *   payout[k] prize for places 1..k (1 <= k <= n), equity[n] output.
 * No status is returned (as in the reference); on failure equity is filled
 * with NaN, a message goes to stderr and icm_last_status() returns -1. */
void icm_equity(int n, const double *S, int Q,
                const double *payout, int k,
                double *equity);

/* Equities for the players listed in targets[0..n_targets).
 *                                                   [reference src/cpu/icm.h:33]
 * Only target entries are computed; every other entry is written as 0
 * (the reference's Python binding promises 0, python/tests/test_icm.py:132-141).
 * Tree branches without a target are pruned from the propagate pass. */
void icm_equity_subset(int n, const double *S, int Q,
                       const double *payout, int k,
                       double *equity,
                       const int *targets, int n_targets);

/* Library initialisation.                           [reference src/cpu/icm.h:41]
 * The reference loads FFTW wisdom from wisdom_path.  Here the path names the
 * autotuner table (the analogue of wisdom: per-level schoolbook/FFT choices
 * and block size); NULL or a missing file keeps the built-in defaults.
 * Also selects device 0 if no device was chosen with icm_gpu_init. */
void icm_init(const char *wisdom_path);

/* ---- engine introspection API of the reference (src/cpu/icm.h:45-83) ----
 * Kept so callers link; the GB300 library has one engine (the GPU tree), so
 * the context constructors return NULL, the engine getters return NULL and
 * icm_run_engine / icm_run_linear_batched return -1.0 without computing. */
typedef void (*IcmEngine)(int n, const double *a,
                          const double *payout, int k,
                          double *inner, void *ctx);

void *icm_tree_ctx_create(int n, int k);                           /* icm.h:48 */
void *icm_hybrid_ctx_create(int n, const double *S, int k, int B); /* icm.h:49 */
void *icm_linear_ctx_create(int n, int k);                         /* icm.h:50 */
void  icm_ctx_destroy(void *ctx, int engine_kind);                 /* icm.h:51 */
IcmEngine icm_engine_tree(void);                                   /* icm.h:54 */
IcmEngine icm_engine_hybrid(void);                                 /* icm.h:55 */
IcmEngine icm_engine_linear(void);                                 /* icm.h:56 */
double icm_run_engine(int n, const double *S, int Q,               /* icm.h:60 */
                      const double *payout, int k,
                      double *equity, IcmEngine engine, void *ctx);
double icm_run_linear_batched(int n, const double *S, int Q,       /* icm.h:65 */
                              const double *payout, int k,
                              double *equity, void *ctx);

#define ICM_ENGINE_TREE   0
#define ICM_ENGINE_LINEAR 1
#define ICM_ENGINE_HYBRID 2

/* Engine dispatch queries.                         [reference src/cpu/icm.h:80,83]
 * icm_select_engine returns the block size B the GPU tree will use for
 * (n, k) (never 0: there is no separate linear engine); icm_select_best_B
 * returns the same B. */
int icm_select_engine(int n, int k);
int icm_select_best_B(int n, int k);

/* Closed-form references.                          [reference src/cpu/icm.h:88-89]
 * V1_i = 1 + sum_{j!=i} S_i/(S_i+S_j)          (payout[m] = n-m)
 * V2_i = sum_{j<l; j,l!=i} S_i/(S_i+S_j+S_l)    (payout[m] = C(n-1-m, 2))
 * Computed on the host, O(n^2) and O(n^3). */
void icm_v1_exact(int n, const double *S, double *V1);
void icm_v2_exact(int n, const double *S, double *V2);

#ifdef __cplusplus
}
#endif

#endif /* ICM_H */
