/*
 * icm_gb300.h -- additions of the GB300 engine beyond the reference's API.
 *
 * None of these has a counterpart in the reference's headers; they extend
 * the drop-in surface of icm.h / icm_gpu.h without changing it.
 */
#ifndef ICM_GB300_H
#define ICM_GB300_H

#include <stddef.h>
#include <stdint.h>

#include "icm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status of the last icm_equity / icm_equity_subset call on this thread:
 * 0 = success, -1 = failure (message in icm_gpu_last_error()).  The
 * reference's void entry points have no status; this is how callers of the
 * drop-in learn that the GPU path failed. */
int icm_last_status(void);

/* Engine configuration (all optional).  Zero fields keep the default.
 *   block_size        players per leaf block B (default chosen per (n, k))
 *   fft_min_degree    child degree at which tree levels switch from
 *                     schoolbook to FFT products (default from the tuner)
 *   q_chunk           quadrature nodes processed per launch sequence
 *   coefficient_fft_only  1 = keep every FFT level on coefficients (no
 *                     spectral levels; for comparison and testing)
 *   max_device_bytes  cap on the plan's device memory
 *   disable_zero_prefix  1 = compute tree nodes whose players all have a
 *                     leaf factor of exactly 0 at a quadrature node (by
 *                     default they are written as monomials or skipped)
 *   enable_subtree    1 = run the leaf blocks and the bottom schoolbook
 *                     levels in one kernel per direction instead of level
 *                     by level (same arithmetic; measured slightly slower
 *                     on GB300, kept for comparison)
 *   small_max_n       largest n solved by the one-CTA-per-node small path
 *                     (whole pipeline in shared memory, one launch per
 *                     solve); 0 = the default k-dependent limit, -1 = never
 *   engine            0 = choose per (n, k); 1 = the tree engine (and the
 *                     small path); 2 = the linear engine (one warp per node,
 *                     O(n k); k <= 256, larger k uses the tree)
 *   quadrature        0 = the reference's erfc-trapezoid rule; 1 = tanh-sinh
 *                     on v in (0, 1) (nodes independent of the stacks; less
 *                     accurate for widely spread stacks)
 *   chunk_streams     streams a tree plan's node chunks are spread over
 *                     (pieces of consecutive nodes, same results); 0 = the
 *                     default (4 from n = 6000, else 2), 1 = one stream,
 *                     at most 4
 *   cta_points        complex points per CTA of the one-CTA FFT steps of a
 *                     single plan's spectral levels (1024, 2048, 4096 or
 *                     8192; 0 = the tuner table's per-level choice, else
 *                     4096); same results, only the CTA shape changes
 *   disable_tma       1 = the four-step column pass of the largest levels
 *                     gathers its tile with ordinary loads instead of a
 *                     tensor-map (TMA) copy (same results; read when a run
 *                     is enqueued)
 *   vjp_spectral_min_degree  levels of a VJP (icm_gb300_vjp_*,
 *                     icm_gb300_equity_vjp[_batched]) whose children have at
 *                     least this degree run spectrally, forward and adjoint (children
 *                     untruncated at k, as for forward plans); 0 = the
 *                     default (every level a forward plan would make
 *                     spectral), -1 = every level on coefficients; batch
 *                     members equal their single VJPs bit for bit either way */
typedef struct {
    int block_size;
    int fft_min_degree;
    int q_chunk;
    int coefficient_fft_only;
    size_t max_device_bytes;
    int disable_zero_prefix;
    int enable_subtree;
    int small_max_n;
    int engine;
    int quadrature;
    int chunk_streams;
    int cta_points;
    int disable_tma;
    int vjp_spectral_min_degree;
} IcmGb300Config;

/* Set the process-wide engine configuration used by plans created
 * afterwards (NULL restores the defaults).  Returns 0. */
int icm_gb300_set_config(const IcmGb300Config *cfg);

/* The engine's player order (host only, no device needed): perm[r] is the
 * index of the player of rank r by stack, descending, ties by index (the
 * reference's GPU order, src/gpu/gpu_plan.cu:405-409).  Returns 0, or -1 for
 * invalid arguments (n < 1, a stack not finite and positive). */
int icm_gb300_player_order(int n, const double *S, int *perm);

/* The geometry of a plan for (n, k) under the given block size and FFT
 * crossover (0 = the defaults), checked against the invariants the kernels
 * rely on (host only: FFT sizes cover every product and correlation without
 * wrap, spectral levels sit over untruncated children, truncation lengths
 * and strides).  flags: 1 = every FFT level on coefficients, 2 = a single
 * VJP plan's geometry (under vjp_spectral_min_degree).  Returns 0
 * when they hold (why: "kinds" and each parent level's kind from level 1 up,
 * 0 schoolbook, 1 FFT on coefficients, 2 spectral), 1 with the first
 * violation in why, -1 for bad arguments. */
int icm_gb300_check_geometry(int n, int k, int block_size, int fft_min_degree, int flags,
                             char *why, int why_len);

/* Test hook for error paths: the nth device allocation made by plans,
 * batches and VJPs from now on fails as if the allocator were exhausted
 * (the call that needed it returns -1 / NULL with the error text); 0 clears
 * a pending failure.  No device fault is involved. */
void icm_gb300_test_fail_allocation(int nth);

/* Batched tournaments: T independent tournaments of uneven size.
 *   n[t], k[t]        players and paid places of tournament t
 *   S, payout         concatenated stacks (sum n) and payouts (sum k)
 *   equity            concatenated output (sum n)
 * All tournaments share Q.  Every tree-level step of all tournaments runs as
 * one work-list launch; each tournament's equities equal those of a single
 * icm_gpu_equity call bit for bit.  Returns 0 / -1. */
int icm_gpu_equity_batched(int T, const int *n, const int *k,
                           const double *S, const double *payout, int Q,
                           double *equity, IcmGpuRunStats *stats);

/* Reusable batch (the batched analogue of IcmGpuPlan): sorts, tree geometry,
 * device buffers and work lists are built once; every run uploads the
 * payouts, replays the captured CUDA graph of the whole launch sequence
 * (recaptured when Q changes) and downloads the equities.
 *   batch_create      stacks concatenated as for icm_gpu_equity_batched;
 *                     NULL on failure (icm_gpu_last_error())
 *   batch_run         payouts concatenated (sum k), equities (sum n)
 *   batch_set_options use_graphs 0/1; profiling 1 = per-launch CUDA events
 *                     (graphs off while profiling), 0 = off, -1 = unchanged
 *   batch_info        members solved by work lists, tournaments solved by
 *                     their own plans (transforms beyond one CTA), players,
 *                     nodes per chunk, device ms of the last run, arena bytes
 *   batch_kernel_stats  as icm_gb300_plan_kernel_stats                      */
typedef struct IcmGb300Batch IcmGb300Batch;
IcmGb300Batch *icm_gb300_batch_create(int T, const int *n, const int *k, const double *S);
int icm_gb300_batch_run(IcmGb300Batch *batch, int Q, const double *payout, double *equity,
                        IcmGpuRunStats *stats);
void icm_gb300_batch_destroy(IcmGb300Batch *batch);
int icm_gb300_batch_set_options(IcmGb300Batch *batch, int use_graphs, int profiling);
int icm_gb300_batch_info(const IcmGb300Batch *batch, long *members, long *fallbacks, long *players,
                         int *q_chunk, double *device_ms, size_t *device_bytes);
int icm_gb300_batch_kernel_stats(const IcmGb300Batch *batch, int i, char *name, int name_len,
                                 double *ms, long *launches, double *flops);

/* Vector-Jacobian products of the equities.  No counterpart in the reference.
 *
 * For the loss L = sum_i cot[i] * equity_i(S, payout) (equity as from
 * icm_equity with the same n, S, Q, payout, k) these return
 *   grad_S[n]        dL/dS_i        (caller's player order)
 *   grad_payout[k]   dL/dpayout_m   (equity is linear in the payout, so
 *                    sum_m grad_payout[m] payout[m] = L)
 * by reverse mode through the quadrature, the per-player division, the
 * propagate and build passes of the tree and the leaf factors.  The forward
 * tree of each chunk of nodes is recomputed inside the call.
 *   flags = 0                the quadrature nodes are held fixed (they move
 *                            with max S only through the quadrature rule)
 *   flags = ICM_VJP_NODE_TERMS  also differentiate the nodes' dependence on
 *                            max S: the exact derivative of the Q-node
 *                            formula, equal to finite differences of it; it
 *                            adds the derivative of the quadrature error to
 *                            the largest stack's entry
 * Returns 0 / -1 (message in icm_gpu_last_error()).
 *   vjp_create/run/destroy   reusable plan for repeated calls on one S
 *   vjp_device_ms            CUDA-event time of the last run's kernels
 *   equity_vjp_batched       T tournaments, arrays concatenated as for
 *                            icm_gpu_equity_batched (cot and grad_S: sum n;
 *                            payout and grad_payout: sum k); every step of
 *                            the forward and adjoint passes of all
 *                            tournaments is one work-list launch, and each
 *                            tournament's gradients equal its single VJP's
 *                            bit for bit
 *   vjp_batch_create/run     the reusable form (an IcmGb300Batch: destroy,
 *                            set_options, info and kernel_stats as for
 *                            batches); runs replay one CUDA graph            */
#define ICM_VJP_NODE_TERMS 1
typedef struct IcmGb300Vjp IcmGb300Vjp;
int icm_gb300_equity_vjp(int n, const double *S, int Q, const double *payout, int k,
                         const double *cot, double *grad_S, double *grad_payout, int flags);
IcmGb300Vjp *icm_gb300_vjp_create(int n, const double *S, int k);
int icm_gb300_vjp_run(IcmGb300Vjp *plan, int Q, const double *payout, const double *cot,
                      double *grad_S, double *grad_payout, int flags, IcmGpuRunStats *stats);
void icm_gb300_vjp_destroy(IcmGb300Vjp *plan);
double icm_gb300_vjp_device_ms(const IcmGb300Vjp *plan);
int icm_gb300_equity_vjp_batched(int T, const int *n, const int *k, const double *S,
                                 const double *payout, int Q, const double *cot,
                                 double *grad_S, double *grad_payout, int flags);
IcmGb300Batch *icm_gb300_vjp_batch_create(int T, const int *n, const int *k, const double *S);
int icm_gb300_vjp_batch_run(IcmGb300Batch *batch, int Q, const double *payout, const double *cot,
                            double *grad_S, double *grad_payout, int flags, IcmGpuRunStats *stats);

/* Tuner table (the analogue of the reference's FFTW wisdom, reference
 * src/cpu/icm.c:184-192; icm_init(path) loads it too).  Entries map a size
 * class -- ceil(log2 n) and a k/n bucket (<= 1/64, <= 1/8, <= 1/2, > 1/2) --
 * to a leaf block size and the child degree where tree levels switch from
 * schoolbook to FFT products, and per tree level (the counterpart of the
 * reference planner's per-level tier choice, src/gpu/gpu_plan.cu:51-329)
 * whether an untruncated FFT level is carried in the frequency domain
 * (spectral = 1) or on coefficients (0) and the complex points per CTA of its
 * one-CTA FFT launches (0 = 4096); plans of that class use them unless
 * icm_gb300_set_config fixes the values.
 *   tuner_load/save   text file; return the number of entries or -1
 *   tuner_lookup      1 and the class's entry, 0 when the class has none
 *   tuner_lookup_level 1 and the class's entry for a tree level, 0 when it
 *                     has none (spectral 1, cta_points 0 then)
 *   autotune          times every candidate (block sizes 4, 8, 16; FFT
 *                     crossover 16, 32, 64, 128) on the given stacks and
 *                     payouts (best device time of `runs` solves after one
 *                     warm-up each) and records the fastest; then, on that
 *                     tree, times each spectral level's alternatives (1024,
 *                     2048, 8192 points per CTA; coefficients) bottom-up and
 *                     records those faster by more than 1%; returns the
 *                     block size, crossover and best time; 0 / -1           */
int icm_gb300_tuner_load(const char *path);
int icm_gb300_tuner_save(const char *path);
void icm_gb300_tuner_clear(void);
int icm_gb300_tuner_lookup(int n, int k, int *block_size, int *fft_min_degree);
int icm_gb300_tuner_lookup_level(int n, int k, int level, int *spectral, int *cta_points);
int icm_gb300_autotune(int n, const double *S, int Q, const double *payout, int k, int runs,
                       int *block_size, int *fft_min_degree, double *best_ms);

/* Subset state of a resident plan: later icm_gpu_equity_with_plan calls
 * compute only the target players' equities (non-targets are 0), pruning the
 * propagate below nodes with no target, as icm_gpu_equity_subset does for one
 * call (reference src/cpu/icm.c:2430-2473, 1733-1815); n_targets = 0 (or
 * targets = NULL) returns the plan to full-field runs.  Targets are original
 * player indices in [0, n).  Returns 0 / -1. */
int icm_gb300_plan_set_targets(IcmGpuPlan *plan, const int *targets, int n_targets);

/* One plan, part of the quadrature: equity[i] = the sum over the rule's
 * nodes q in [q_begin, q_end) of Q of player i's node contribution
 * (icm_gpu_equity_with_plan sums all Q).  The partial sums of a partition
 * of [0, Q) add up to the full equities (to rounding: the full run sums the
 * nodes in one fixed order); [0, Q) equals icm_gpu_equity_with_plan bit for
 * bit.  This is the node-range split a multi-GPU driver uses: each GPU takes
 * a range, one all-reduce sums the partials (icm_gb300/distributed.py).
 * Returns 0 / -1 (invalid range: 0 <= q_begin <= q_end <= Q). */
int icm_gb300_plan_equity_nodes(IcmGpuPlan *plan, int Q, const double *payout, int q_begin, int q_end,
                                double *equity, IcmGpuRunStats *stats);

/* Stream-ordered runs on device memory, for callers whose data already lives
 * on the GPU (a torch tensor, a CUDA buffer): the payouts, cotangents,
 * equities and gradients are device pointers (device memory of the library's
 * device or managed memory, else -1), and `stream` is the caller's CUDA
 * stream (cudaStream_t; NULL = the legacy default stream).  The run starts
 * after the work already queued on that stream, later work on the stream sees
 * the results, and the call returns without waiting for the GPU (the VJP with
 * ICM_VJP_NODE_TERMS waits once, for its host-side chain rule).  Arrays are
 * as in icm_gpu_equity_with_plan / icm_gb300_vjp_run (original player order,
 * payout[k], equity[n], cot[n], grad_S[n], grad_payout[k]).  The plan's
 * stacks stay on the host side (the player sort runs there).  The device time
 * of such a run is not recorded.  Returns 0 / -1. */
int icm_gb300_plan_equity_dev(IcmGpuPlan *plan, int Q, const double *d_payout, double *d_equity, void *stream);
/* The device the library runs on (the one icm_gpu_init chose; -1 before any
 * initialisation).  Returns 0 / -1 (null argument). */
int icm_gb300_current_device(int *device);

/* Four-step column passes launched through TMA tensor copies since the
 * library was loaded (all plans; a diagnostic for disable_tma). */
long icm_gb300_tma_launch_count(void);
int icm_gb300_vjp_run_dev(IcmGb300Vjp *plan, int Q, const double *d_payout, const double *d_cot,
                          double *d_grad_S, double *d_grad_payout, int flags, void *stream);

/* Work of each node of the rule for these stacks (host only, no GPU):
 * work[q] = the players outside node q's zero prefix (those whose leaf factor
 * is not exactly 0, the part of the tree the engine computes), 0 for nodes
 * of weight 0, which are skipped.  A multi-GPU driver cuts node ranges of
 * equal total work from it.  Returns 0 / -1. */
int icm_gb300_node_work(int n, const double *S, int Q, int *work);

/* Quadrature ladder: solves with Q0, 2 Q0, 4 Q0, ... nodes of the
 * reference's rule (never more than Qmax) until two successive results
 * agree per player to tol (relative, against a floor of 1e-12 of the
 * largest equity).  equity receives the finest result, *Q_used its node
 * count, *est_err the last difference (INFINITY if only Q0 ran).  The
 * default entry points keep the caller's Q; this is for callers that want
 * a stated accuracy where Q = 256 does not resolve the integrand.
 * Returns 0 / -1. */
int icm_gb300_equity_adaptive(int n, const double *S, const double *payout, int k, int Q0,
                              double tol, int Qmax, double *equity, int *Q_used, double *est_err);

/* Measured peak of this GPU's FP64 pipe: a register-resident DFMA loop over
 * all SMs, in GFLOP/s (2 flops per DFMA).  Returns 1 / 0. */
int icm_gpu_measure_fp64_gflops(double *gflops_out);

/* The leaf factors a = exp(arg) (0 below -700) of n arguments, computed on
 * the GPU exactly as the tree's leaves compute them (a check of the device
 * exponential against the host's).  Returns 0 / -1. */
int icm_gb300_leaf_factors(int n, const double *arg, double *out);

/* Number of kernels the last equity call launched (for benchmarks). */
long icm_gpu_last_launch_count(void);

/* Diagnostics for a plan (the analogue of the reference's instrumented
 * IcmGpuRunStats path, without synchronising between kernels):
 *   set_profiling   1 = bracket every kernel launch of later runs with CUDA
 *                   events on the plan's stream (timings accumulate until
 *                   profiling is set again)
 *   kernel_stats    entry i of the per-kernel table: name, total ms,
 *                   launches and algorithmic FP64 flops; returns the number
 *                   of entries (call with i = -1 to get the count)
 *   device_ms       CUDA-event time of the last run's kernel sequence       */
int icm_gb300_plan_set_profiling(IcmGpuPlan *plan, int enable);
int icm_gb300_plan_kernel_stats(const IcmGpuPlan *plan, int i, char *name, int name_len, double *ms,
                                long *launches, double *flops);
double icm_gb300_plan_device_ms(const IcmGpuPlan *plan);

/* Equities for callers that cannot allocate device memory.  No counterpart
 * in the reference.
 *
 * Same inputs, outputs and result as icm_equity (host arrays S[n],
 * payout[k] in, equity[n] out), but the call allocates nothing: no
 * cudaMalloc/cudaFree, no stream or event creation, no allocating library
 * routine.  It serves hosts that forbid device allocation after start-up
 * (services that size every buffer once so that a solve cannot fail or stall
 * on an allocator) and processes whose device memory belongs to another
 * allocator (a framework's caching pool that has reserved the GPU).  All
 * device-side data lives in one static scratch array of 32 MiB inside the
 * library, held by every GPU that loads the library until the process exits.
 *
 * Limits: n <= 4096 players and Q <= 4096 nodes; larger requests return -1
 * with the reason in icm_gpu_last_error() (use icm_equity for them).
 * The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; that first call should come
 * before any stream capture begins.  Calls share the scratch array: calls that
 * overlap on the GPU race.  The solve runs on the library's device, restores
 * the caller's current device, uses the legacy default stream and returns
 * after the equities are on the host; returns 0 / -1.  Results agree with
 * icm_equity's to rounding (coefficient-FFT tree levels throughout). */
int icm_gpu_equity_noalloc(int n, const double *S, int Q, const double *payout, int k,
                           double *equity);

#ifdef __cplusplus
}
#endif

#endif /* ICM_GB300_H */
