/*
 * icm_gpu.h -- drop-in GPU-API boundary of the GB300 ICM engine.
 *
 * Names, signatures, return conventions and struct layouts are those of the
 * reference's src/gpu/icm_gpu.h (structs must stay layout-identical so that
 * callers compiled against the reference header work unchanged).  Meanings
 * of the option fields that describe the reference's cuFFT tiers are noted
 * where the GB300 engine treats them differently.
 */
#ifndef ICM_GPU_H
#define ICM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct IcmGpuPlan IcmGpuPlan;

/* [reference src/gpu/icm_gpu.h:12-34] */
typedef struct {
    int device_id;              /* informational, overwritten by plan_create
                                   with the device chosen by icm_gpu_init */
    int use_cufftdx;            /* ignored: the engine has its own FP64 FFT */
    int enable_graphs;          /* 1 = capture the run's launch sequence (all
                                   node chunks) in a CUDA graph once per node
                                   count and replay it on later runs */
    int enable_q_pipeline;      /* ignored (all Q nodes of a chunk run
                                   level-synchronously in one launch per level) */
    int memory_strategy;        /* 1 = plain cudaMalloc for the plan's arena;
                                   any other value = the stream-ordered pool.
                                   The reference's selective recompute (3) has
                                   no counterpart: memory is bounded by the
                                   node chunk instead */
    int force_uncached_fused_levels; /* ignored: coefficient-FFT levels always
                                   cache the children's spectra */
    int force_uncached_cufft_levels; /* ignored (no cuFFT levels) */
    int fast_mode;              /* ignored */
    int verbose;                /* print the plan to stderr and report the
                                   per-stage device times in IcmGpuRunStats
                                   (block build, tree build, propagate, leaf
                                   extraction; events at stage boundaries) */
} IcmGpuOptions;

/* [reference src/gpu/icm_gpu.h:36-50] */
typedef struct {
    double total_ns;
    double sort_ns;
    double quadrature_overhead_ns;
    double block_build_ns;
    double tree_build_ns;
    double tree_propagate_cached_ns;
    double tree_propagate_recomputed_ns;
    double leaf_extract_ns;
    size_t peak_vram_bytes;
    int engine;                 /* 1 = hybrid tree (the only engine) */
    int B;
    int uncached_fused_levels;
    int uncached_cufft_levels;
} IcmGpuRunStats;

/* [reference src/gpu/icm_gpu.h:52-63] */
typedef struct {
    int n;
    int k;
    int B;
    int engine;                 /* 1 = hybrid tree */
    int n_levels;
    int n_tier1;                /* schoolbook levels */
    int n_tier2;                /* shared-memory FFT levels */
    int n_tier3;                /* multi-pass (global) FFT levels */
    int q_batch;                /* quadrature nodes per launch sequence */
    size_t planned_peak_vram_bytes;
} IcmGpuPlanSummary;

/* Lifecycle.                       [reference src/gpu/icm_gpu.h:66-68,74]
 * icm_gpu_init returns 1 on success and 0 on failure (the reference's
 * convention); the other calls return 0 on success and -1 on failure. */
int icm_gpu_init(int device_id);
void icm_gpu_shutdown(void);
const char *icm_gpu_last_error(void);
int icm_gpu_release_pooled_memory(void);

/* Plans.                            [reference src/gpu/icm_gpu.h:77-79]
 * A plan owns the sorted stacks, the tree geometry and all device buffers
 * for one tournament; it is reusable across payouts and Q. */
IcmGpuPlan *icm_gpu_plan_create(int n, const double *S, int k, const IcmGpuOptions *opts);
void icm_gpu_plan_destroy(IcmGpuPlan *plan);
int icm_gpu_plan_summary(const IcmGpuPlan *plan, IcmGpuPlanSummary *summary);

/* Execution.                        [reference src/gpu/icm_gpu.h:92-109]
 * Return 0 on success, -1 on failure (see icm_gpu_last_error).  stats is
 * optional; stats->total_ns is the wall time of the call including the
 * final device synchronisation. */
int icm_gpu_equity_with_plan(IcmGpuPlan *plan, int Q,
                             const double *payout, double *equity,
                             IcmGpuRunStats *stats);

int icm_gpu_equity(int n, const double *S, int Q,
                   const double *payout, int k,
                   double *equity, const IcmGpuOptions *opts,
                   IcmGpuRunStats *stats);

/* Subset: unlike the reference GPU path (which computes the full tree and
 * masks the output, reference src/gpu/icm_gpu.h:101-103), cold tree branches
 * are pruned from the propagate pass and cold blocks skip the divide.
 * Non-target entries are written as 0. */
int icm_gpu_equity_subset(int n, const double *S, int Q,
                          const double *payout, int k,
                          double *equity,
                          const int *targets, int n_targets,
                          const IcmGpuOptions *opts,
                          IcmGpuRunStats *stats);

/* Calibration helpers.              [reference src/gpu/icm_gpu.h:112-116]
 * Return 1 on success, 0 on failure.  The fused-pair probes time this
 * engine's shared-memory FFT build and propagate kernels for a batch of
 * parents with FFT size fft_n (ns per parent). */
int icm_gpu_measure_hbm_bandwidth_gbps(double *gbps_out);
int icm_gpu_measure_fused_pair_ns(int fft_n, int batch, int quick,
                                  double *build_ns_out, double *corr_ns_out);
int icm_gpu_measure_fused_r2c_pair_ns(int fft_n, int batch, int quick,
                                      double *build_ns_out, double *corr_ns_out);

#ifdef __cplusplus
}
#endif

#endif /* ICM_GPU_H */
