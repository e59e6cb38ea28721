// api.cpp -- the C ABI of libicm_gb300.so: the reference's icm.h / icm_gpu.h
// entry points (same names, arguments and return conventions) plus the
// additions in icm_gb300.h.  Plain pointers and sizes only.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "batch.h"
#include "engine.h"
#include "kernels.h"
#include "vjp.h"

using namespace icmg;

namespace {
thread_local std::string t_last_error;
thread_local int t_last_status = 0;
thread_local long t_launches = 0;

void set_error(const std::string &e) { t_last_error = e; }

bool ensure_device() {
    if (g_device >= 0) {
        cudaError_t e = cudaSetDevice(g_device);
        if (e != cudaSuccess) { set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e)); return false; }
        return true;
    }
    return icm_gpu_init(0) == 1;
}

double now_ns() {
    return (double)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// void entry points report failure through NaN output, stderr and
// icm_last_status() (the reference's icm_equity has no status to return)
void fail_void(int n, double *equity, const std::string &what) {
    t_last_status = -1;
    set_error(what);
    fprintf(stderr, "icm_gb300: %s\n", what.c_str());
    if (equity)
        for (int i = 0; i < n; ++i) equity[i] = std::nan("");
}

// The calling thread's last one-shot plan, kept when its arena is small:
// reused by the next call of the same shape under the same options, engine
// configuration and tuner table (the geometry depends on nothing else).
struct PlanCache {
    Plan *p = nullptr;
    IcmGpuOptions opts{};
    IcmGb300Config cfg{};
    long tune_gen = -1;
    int dev = -1;
};
thread_local PlanCache t_plan;
// Arenas of kept plans, summed over the process's threads, stay within this
// budget: a kept plan's arena cannot go back to the device's default pool for
// another thread's plan, and a thread that exits leaves its kept plan behind,
// so the budget bounds both.  icm_gpu_release_pooled_memory drops the calling
// thread's kept plan.
constexpr size_t kPlanCacheTotalBytes = (size_t)16 << 30;
std::atomic<size_t> g_plan_cache_bytes{0};

bool same_opts(const IcmGpuOptions &a, const IcmGpuOptions &b) {
    IcmGpuOptions x = a, y = b;
    x.device_id = y.device_id = 0;
    return std::memcmp(&x, &y, sizeof x) == 0;
}

void drop_cached_plan() {
    if (t_plan.p) {
        g_plan_cache_bytes.fetch_sub(t_plan.p->arena_bytes);
        plan_destroy(t_plan.p);
    }
    t_plan = PlanCache{};
}

Plan *cached_plan(int n, int k, const IcmGpuOptions *opts) {
    PlanCache &c = t_plan;
    if (!c.p) return nullptr;
    g_plan_cache_bytes.fetch_sub(c.p->arena_bytes);   // out of the cache while in use
    const IcmGpuOptions o = opts ? *opts : IcmGpuOptions{};
    Plan *p = nullptr;
    if (c.p->n == n && c.p->k == k && c.dev == g_device && c.tune_gen == g_tune_generation.load() &&
        same_opts(c.opts, o) && std::memcmp(&c.cfg, &g_config, sizeof c.cfg) == 0)
        p = c.p;
    else
        plan_destroy(c.p);
    c = PlanCache{};
    return p;   // taken out of the cache while in use
}

bool keep_plan(Plan *p, const IcmGpuOptions *opts) {
    drop_cached_plan();
    const size_t b = p->arena_bytes;
    size_t cur = g_plan_cache_bytes.load();
    do {
        if (cur + b > kPlanCacheTotalBytes) return false;
    } while (!g_plan_cache_bytes.compare_exchange_weak(cur, cur + b));
    t_plan.p = p;
    t_plan.opts = opts ? *opts : IcmGpuOptions{};
    t_plan.cfg = g_config;
    t_plan.tune_gen = g_tune_generation.load();
    t_plan.dev = g_device;
    return true;
}

int run_full(int n, const double *S, int Q, const double *payout, int k, double *equity, const int *targets,
             int n_targets, const IcmGpuOptions *opts, IcmGpuRunStats *stats) {
    if (!ensure_device()) return -1;
    std::string err;
    // small fields: no plan at all (only fields within the small path's largest
    // limit are classified here, so larger ones are sorted once, by the plan)
    const int small_cap = std::max(kSmallMaxN, g_config.small_max_n);
    if (n <= small_cap && (!opts || (!opts->verbose && opts->memory_strategy != 1))) {
        long nl = 0;
        const int r = small_solve(n, S, Q, payout, k, equity, targets, n_targets, stats, &nl, err);
        if (r < 0) { set_error(err); return -1; }
        if (r == 1) { t_launches = nl; return 0; }
    }
    // repeated calls of one shape reuse the thread's last plan (new stacks
    // only; a subset query sets its targets for the one run)
    Plan *p = cached_plan(n, k, opts);
    if (p) {
        if (plan_restack(p, S, err) != 0) {
            plan_destroy(p);
            set_error(err);
            return -1;
        }
    } else {
        p = plan_create(n, S, k, opts, err);
        if (!p) { set_error(err); return -1; }
    }
    int rc = 0;
    if (targets) rc = plan_set_targets(p, targets, n_targets, err);
    if (rc == 0) rc = plan_run(p, Q, payout, equity, stats, err);
    p->subset = false;
    t_launches = p->launches;
    if (rc != 0 || !keep_plan(p, opts)) plan_destroy(p);
    if (rc != 0) { set_error(err); return -1; }
    return 0;
}
}  // namespace

namespace icmg {
void api_set_error(const std::string &e) { set_error(e); }
}

// An entry point's work runs inside guarded(): a C++ exception (a host
// allocation that fails, a thread that cannot start) becomes the entry
// point's failure value with the message as the last error, instead of
// unwinding into C callers.
template <class R, class F>
static R guarded(const char *name, R fail, F &&f) {
    try {
        return f();
    } catch (const std::exception &e) {
        set_error(std::string(name) + ": " + e.what());
    } catch (...) {
        set_error(std::string(name) + ": unknown error");
    }
    return fail;
}

extern "C" {

// ------------------------------------------------------------ icm.h
void icm_init(const char *wisdom_path) {
    try {
        // The tuner table (the analogue of the reference's FFTW wisdom, read from
        // the given path; a missing file keeps the defaults, as the reference's
        // missing wisdom file does)
        if (wisdom_path) {
            std::string err;
            tune_load(wisdom_path, err);
        }
        if (g_device < 0) icm_gpu_init(0);
    } catch (const std::exception &e) {
        set_error(std::string("icm_init: ") + e.what());
    } catch (...) {
        set_error("icm_init: unknown error");
    }
}

void icm_equity(int n, const double *S, int Q, const double *payout, int k, double *equity) {
    try {
        t_last_status = 0;
        if (n < 1 || k < 1 || k > n || Q < 1 || !S || !payout || !equity) {
            fail_void(n, equity, "icm_equity: invalid arguments (need 1 <= k <= n, Q >= 1)");
            return;
        }
        if (run_full(n, S, Q, payout, k, equity, nullptr, 0, nullptr, nullptr) != 0)
            fail_void(n, equity, "icm_equity failed: " + t_last_error);
    } catch (const std::exception &e) {
        fail_void(n, equity, std::string("icm_equity: ") + e.what());
    } catch (...) {
        fail_void(n, equity, "icm_equity: unknown error");
    }
}

void icm_equity_subset(int n, const double *S, int Q, const double *payout, int k, double *equity,
                       const int *targets, int n_targets) {
    try {
        t_last_status = 0;
        if (n < 1 || k < 1 || k > n || Q < 1 || !S || !payout || !equity || !targets || n_targets < 1) {
            fail_void(n, equity, "icm_equity_subset: invalid arguments");
            return;
        }
        if (run_full(n, S, Q, payout, k, equity, targets, n_targets, nullptr, nullptr) != 0)
            fail_void(n, equity, "icm_equity_subset failed: " + t_last_error);
    } catch (const std::exception &e) {
        fail_void(n, equity, std::string("icm_equity_subset: ") + e.what());
    } catch (...) {
        fail_void(n, equity, "icm_equity_subset: unknown error");
    }
}

void *icm_tree_ctx_create(int, int) { return nullptr; }
void *icm_hybrid_ctx_create(int, const double *, int, int) { return nullptr; }
void *icm_linear_ctx_create(int, int) { return nullptr; }
void icm_ctx_destroy(void *, int) {}
IcmEngine icm_engine_tree(void) { return nullptr; }
IcmEngine icm_engine_hybrid(void) { return nullptr; }
IcmEngine icm_engine_linear(void) { return nullptr; }
double icm_run_engine(int, const double *, int, const double *, int, double *, IcmEngine, void *) {
    set_error("icm_run_engine: the GB300 library has a single GPU engine; use icm_equity");
    return -1.0;
}
double icm_run_linear_batched(int, const double *, int, const double *, int, double *, void *) {
    set_error("icm_run_linear_batched: the GB300 library has a single GPU engine; use icm_equity");
    return -1.0;
}
int icm_select_engine(int n, int k) { return select_block_size(n, k); }
int icm_select_best_B(int n, int k) { return select_block_size(n, k); }

// closed forms (reference src/cpu/icm.c:145-170), host-side
void icm_v1_exact(int n, const double *S, double *V1) {
    for (int i = 0; i < n; ++i) {
        double v = 1.0;
        for (int j = 0; j < n; ++j)
            if (j != i) v += S[i] / (S[i] + S[j]);
        V1[i] = v;
    }
}

void icm_v2_exact(int n, const double *S, double *V2) {
    for (int i = 0; i < n; ++i) {
        double v = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            for (int l = j + 1; l < n; ++l) {
                if (l == i) continue;
                v += S[i] / (S[i] + S[j] + S[l]);
            }
        }
        V2[i] = v;
    }
}

// ------------------------------------------------------------ icm_gpu.h
int icm_gpu_init(int device_id) {
    return guarded<int>("icm_gpu_init", 0, [&]() -> int {
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess) { set_error(std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e)); return 0; }
        if (count <= 0) { set_error("No CUDA devices found"); return 0; }
        if (device_id < 0) device_id = 0;
        if (device_id >= count) {
            set_error("Invalid CUDA device id " + std::to_string(device_id) + " (count=" + std::to_string(count) + ")");
            return 0;
        }
        e = cudaSetDevice(device_id);
        if (e != cudaSuccess) { set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e)); return 0; }
        fft_set_smem_limits();
        // keep freed plan arenas in this process's default pool for the next plan
        cudaMemPool_t pool = nullptr;
        if (cudaDeviceGetDefaultMemPool(&pool, device_id) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        g_device = device_id;
        return 1;
    });
}

void icm_gpu_shutdown(void) {
    if (g_device >= 0) {
        cudaSetDevice(g_device);
        cudaDeviceSynchronize();
        small_context_release();   // this thread's one-shot buffers and plan
        drop_cached_plan();
    }
}

const char *icm_gpu_last_error(void) { return t_last_error.c_str(); }

int icm_gpu_release_pooled_memory(void) {
    if (g_device < 0) return -1;
    small_context_release();   // this thread's one-shot buffers and plan
    drop_cached_plan();
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, g_device) != cudaSuccess) return -1;
    if (cudaMemPoolTrimTo(pool, 0) != cudaSuccess) return -1;
    return 0;
}

IcmGpuPlan *icm_gpu_plan_create(int n, const double *S, int k, const IcmGpuOptions *opts) {
    return guarded<IcmGpuPlan *>("icm_gpu_plan_create", nullptr, [&]() -> IcmGpuPlan * {
        if (g_device < 0) {
            set_error("icm_gpu_init must be called before icm_gpu_plan_create");
            return nullptr;
        }
        if (!ensure_device()) return nullptr;
        std::string err;
        Plan *p = plan_create(n, S, k, opts, err);
        if (!p) set_error(err);
        return reinterpret_cast<IcmGpuPlan *>(p);
    });
}

void icm_gpu_plan_destroy(IcmGpuPlan *plan) { plan_destroy(reinterpret_cast<Plan *>(plan)); }

int icm_gpu_plan_summary(const IcmGpuPlan *plan, IcmGpuPlanSummary *summary) {
    const Plan *p = reinterpret_cast<const Plan *>(plan);
    if (!p || !summary) return 0;
    memset(summary, 0, sizeof(*summary));
    summary->n = p->n;
    summary->k = p->k;
    summary->B = p->B;
    summary->engine = 1;
    summary->n_levels = p->L;
    for (int l = 1; l < p->L; ++l) {
        if (!p->lv[l].fft) summary->n_tier1++;
        else if (p->lv[l].fftn <= kSmemFftMax) summary->n_tier2++;
        else summary->n_tier3++;
    }
    summary->q_batch = p->qc;
    summary->planned_peak_vram_bytes = p->arena_bytes;
    return 1;
}

// a pointer the library's kernels and device copies may use: device memory of
// the library's device, or managed memory
static bool device_pointer(const void *ptr, const char *what, const char *fn) {
    cudaPointerAttributes a{};
    if (!ptr || cudaPointerGetAttributes(&a, ptr) != cudaSuccess ||
        !(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == g_device))) {
        cudaGetLastError();   // clear a failed query
        set_error(std::string(fn) + ": " + what + " is not device memory of the library's device");
        return false;
    }
    return true;
}

long icm_gb300_tma_launch_count(void) { return g_tma_launches.load(); }

int icm_gb300_current_device(int *device) {
    if (!device) return -1;
    *device = g_device;
    return 0;
}

int icm_gb300_plan_equity_dev(IcmGpuPlan *plan, int Q, const double *d_payout, double *d_equity, void *stream) {
    return guarded<int>("icm_gb300_plan_equity_dev", -1, [&]() -> int {
        Plan *p = reinterpret_cast<Plan *>(plan);
        const char *fn = "icm_gb300_plan_equity_dev";
        if (!p || Q < 1) { set_error(std::string(fn) + ": invalid arguments"); return -1; }
        if (!ensure_device()) return -1;
        if (!device_pointer(d_payout, "payout", fn) || !device_pointer(d_equity, "equity", fn)) return -1;
        std::string err;
        DevIO io;
        io.st = static_cast<cudaStream_t>(stream);
        const int rc = plan_run(p, Q, d_payout, d_equity, nullptr, err, 0, -1, &io);
        t_launches = p->launches;
        if (rc != 0) { set_error(std::string(fn) + ": " + err); return -1; }
        return 0;
    });
}

int icm_gb300_plan_set_targets(IcmGpuPlan *plan, const int *targets, int n_targets) {
    return guarded<int>("icm_gb300_plan_set_targets", -1, [&]() -> int {
        Plan *p = reinterpret_cast<Plan *>(plan);
        if (!p || n_targets < 0 || (n_targets > 0 && !targets)) {
            set_error("icm_gb300_plan_set_targets: invalid arguments");
            return -1;
        }
        if (n_targets == 0) {
            p->subset = false;
            return 0;
        }
        for (int t = 0; t < n_targets; ++t)
            if (targets[t] < 0 || targets[t] >= p->n) {
                set_error("icm_gb300_plan_set_targets: target " + std::to_string(targets[t]) + " outside [0, " +
                          std::to_string(p->n) + ")");
                return -1;
            }
        std::string err;
        if (!ensure_device()) return -1;
        if (plan_set_targets(p, targets, n_targets, err) != 0) {
            set_error("icm_gb300_plan_set_targets: " + err);
            return -1;
        }
        return 0;
    });
}

int icm_gpu_equity_with_plan(IcmGpuPlan *plan, int Q, const double *payout, double *equity,
                             IcmGpuRunStats *stats) {
    return guarded<int>("icm_gpu_equity_with_plan", -1, [&]() -> int {
        Plan *p = reinterpret_cast<Plan *>(plan);
        if (!p || !payout || !equity || Q <= 0) {
            set_error("icm_gpu_equity_with_plan invalid arguments");
            return -1;
        }
        if (!ensure_device()) return -1;
        std::string err;
        const int rc = plan_run(p, Q, payout, equity, stats, err);
        t_launches = p->launches;
        if (rc != 0) { set_error(err); return -1; }
        return 0;
    });
}

int icm_gb300_plan_equity_nodes(IcmGpuPlan *plan, int Q, const double *payout, int q_begin, int q_end,
                                double *equity, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gb300_plan_equity_nodes", -1, [&]() -> int {
        Plan *p = reinterpret_cast<Plan *>(plan);
        if (!p || !payout || !equity || Q <= 0 || q_begin < 0 || q_begin > q_end || q_end > Q) {
            set_error("icm_gb300_plan_equity_nodes invalid arguments");
            return -1;
        }
        if (!ensure_device()) return -1;
        std::string err;
        const int rc = plan_run(p, Q, payout, equity, stats, err, q_begin, q_end);
        t_launches = p->launches;
        if (rc != 0) { set_error(err); return -1; }
        return 0;
    });
}

int icm_gpu_equity(int n, const double *S, int Q, const double *payout, int k, double *equity,
                   const IcmGpuOptions *opts, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gpu_equity", -1, [&]() -> int {
        if (n <= 0 || k <= 0 || k > n || Q <= 0 || !S || !payout || !equity) {
            set_error("icm_gpu_equity invalid arguments");
            return -1;
        }
        const double t0 = now_ns();
        const int rc = run_full(n, S, Q, payout, k, equity, nullptr, 0, opts, stats);
        if (rc == 0 && stats) stats->total_ns = now_ns() - t0;   // includes plan creation
        return rc;
    });
}

int icm_gpu_equity_subset(int n, const double *S, int Q, const double *payout, int k, double *equity,
                          const int *targets, int n_targets, const IcmGpuOptions *opts, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gpu_equity_subset", -1, [&]() -> int {
        if (n <= 0 || k <= 0 || k > n || Q <= 0 || n_targets <= 0 || !targets || !S || !payout || !equity) {
            set_error("icm_gpu_equity_subset invalid arguments");
            return -1;
        }
        const double t0 = now_ns();
        const int rc = run_full(n, S, Q, payout, k, equity, targets, n_targets, opts, stats);
        if (rc == 0 && stats) stats->total_ns = now_ns() - t0;
        return rc;
    });
}

int icm_gpu_measure_hbm_bandwidth_gbps(double *gbps_out) {
    return guarded<int>("icm_gpu_measure_hbm_bandwidth_gbps", 0, [&]() -> int {
        if (!gbps_out || !ensure_device()) return 0;
        std::string err;
        if (measure_hbm_gbps(gbps_out, err) != 0) { set_error(err); return 0; }
        return 1;
    });
}

int icm_gpu_measure_fused_pair_ns(int fft_n, int batch, int quick, double *build_ns_out, double *corr_ns_out);
int icm_gpu_measure_fused_r2c_pair_ns(int fft_n, int batch, int quick, double *build_ns_out,
                                      double *corr_ns_out) {
    return icm_gpu_measure_fused_pair_ns(fft_n, batch, quick, build_ns_out, corr_ns_out);
}

// ------------------------------------------------------------ icm_gb300.h
int icm_last_status(void) { return t_last_status; }

int icm_gb300_player_order(int n, const double *S, int *perm) {
    return guarded<int>("icm_gb300_player_order", -1, [&]() -> int {
        if (n < 1 || !S || !perm) { set_error("icm_gb300_player_order: invalid arguments"); return -1; }
        for (int i = 0; i < n; ++i)
            if (!(S[i] > 0.0) || !std::isfinite(S[i])) {
                set_error("icm_gb300_player_order: stacks must be finite and positive");
                return -1;
            }
        std::vector<int> p;
        sort_players_desc(S, n, p);
        std::copy(p.begin(), p.end(), perm);
        return 0;
    });
}

int icm_gb300_node_work(int n, const double *S, int Q, int *work) {
    return guarded<int>("icm_gb300_node_work", -1, [&]() -> int {
        if (n < 1 || !S || Q < 1 || !work) { set_error("icm_gb300_node_work: invalid arguments"); return -1; }
        std::vector<double> Ss(S, S + n);
        for (double v : Ss)
            if (!(v > 0.0) || !std::isfinite(v)) {
                set_error("icm_gb300_node_work: stacks must be finite and positive");
                return -1;
            }
        std::sort(Ss.begin(), Ss.end(), [](double a, double b) { return a > b; });
        std::vector<double> logv, w;
        make_nodes(Q, Ss[0], logv, w);
        for (int q = 0; q < Q; ++q) work[q] = (w[q] == 0.0) ? 0 : n - zero_prefix(Ss.data(), n, logv[q]);
        return 0;
    });
}

void icm_gb300_test_fail_allocation(int nth) { set_alloc_failure(nth); }

int icm_gb300_check_geometry(int n, int k, int block_size, int fft_min_degree, int flags, char *why, int why_len) {
    return guarded<int>("icm_gb300_check_geometry", -1, [&]() -> int {
        if (n < 1 || k < 1 || k > n) { set_error("icm_gb300_check_geometry: need 1 <= k <= n"); return -1; }
        const IcmGb300Config saved = g_config;
        g_config.block_size = block_size;
        g_config.fft_min_degree = fft_min_degree;
        Plan p;
        p.coeff_only = (flags & 1) != 0 || ((flags & 2) != 0 && g_config.vjp_spectral_min_degree < 0);
        p.vjp = (flags & 2) != 0;
        std::string err;
        const std::vector<double> S(n, 1.0);   // stack values do not shape the tree
        int rc = plan_geometry(&p, n, S.data(), k, err);
        g_config = saved;
        if (rc != 0) { set_error("icm_gb300_check_geometry: " + err); return -1; }
        rc = plan_check_geometry(&p, err) == 0 ? 0 : 1;
        if (!rc) {   // the level kinds, bottom up: 0 schoolbook, 1 FFT on coefficients, 2 spectral
            err = "kinds";
            for (int l = 1; l < p.L; ++l) err += " " + std::to_string(p.lv[l].kind);
        }
        if (why && why_len > 0) {
            std::strncpy(why, err.c_str(), why_len - 1);
            why[why_len - 1] = 0;
        }
        return rc;
    });
}

int icm_gb300_set_config(const IcmGb300Config *cfg) {
    if (cfg) g_config = *cfg;
    else memset(&g_config, 0, sizeof(g_config));
    return 0;
}

int icm_gpu_equity_batched(int T, const int *n, const int *k, const double *S, const double *payout, int Q,
                           double *equity, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gpu_equity_batched", -1, [&]() -> int {
        if (T < 1 || !n || !k || !S || !payout || !equity || Q < 1) {
            set_error("icm_gpu_equity_batched invalid arguments");
            return -1;
        }
        if (!ensure_device()) return -1;
        const double t0 = now_ns();
        std::string err;
        Forest *f = forest_create(T, n, k, S, err);
        if (!f) { set_error("icm_gpu_equity_batched: " + err); return -1; }
        f->graphs = false;   // one run: capturing would not pay
        const int rc = forest_run(f, Q, payout, equity, stats, err);
        t_launches = f->launches;
        forest_destroy(f);
        if (rc != 0) { set_error("icm_gpu_equity_batched: " + err); return -1; }
        if (stats) stats->total_ns = now_ns() - t0;
        return 0;
    });
}

IcmGb300Batch *icm_gb300_batch_create(int T, const int *n, const int *k, const double *S) {
    return guarded<IcmGb300Batch *>("icm_gb300_batch_create", nullptr, [&]() -> IcmGb300Batch * {
        if (!ensure_device()) return nullptr;
        std::string err;
        Forest *f = forest_create(T, n, k, S, err);
        if (!f) { set_error("icm_gb300_batch_create: " + err); return nullptr; }
        return reinterpret_cast<IcmGb300Batch *>(f);
    });
}

int icm_gb300_batch_run(IcmGb300Batch *b, int Q, const double *payout, double *equity, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gb300_batch_run", -1, [&]() -> int {
        if (!b) { set_error("icm_gb300_batch_run: null batch"); return -1; }
        if (!ensure_device()) return -1;
        Forest *f = reinterpret_cast<Forest *>(b);
        std::string err;
        const int rc = forest_run(f, Q, payout, equity, stats, err);
        t_launches = f->launches;
        if (rc != 0) { set_error("icm_gb300_batch_run: " + err); return -1; }
        return 0;
    });
}

void icm_gb300_batch_destroy(IcmGb300Batch *b) { forest_destroy(reinterpret_cast<Forest *>(b)); }

int icm_gb300_batch_set_options(IcmGb300Batch *b, int use_graphs, int profiling) {
    if (!b) return -1;
    Forest *f = reinterpret_cast<Forest *>(b);
    f->graphs = use_graphs != 0;
    if (profiling >= 0) {
        f->prof.on = profiling != 0;
        f->kstats.clear();
    }
    return 0;
}

int icm_gb300_batch_info(const IcmGb300Batch *b, long *members, long *fallbacks, long *players, int *q_chunk,
                         double *device_ms, size_t *device_bytes) {
    if (!b) return -1;
    const Forest *f = reinterpret_cast<const Forest *>(b);
    if (members) *members = (long)f->tr.size();
    if (fallbacks) *fallbacks = (long)f->fallback.size();
    if (players) *players = f->Ntot;
    if (q_chunk) *q_chunk = f->qc;
    if (device_ms) *device_ms = f->last_device_ms;
    if (device_bytes) *device_bytes = f->arena_bytes;
    return 0;
}

int icm_gb300_batch_kernel_stats(const IcmGb300Batch *b, int i, char *name, int name_len, double *ms,
                                 long *launches, double *flops) {
    if (!b) return -1;
    const Forest *f = reinterpret_cast<const Forest *>(b);
    if (i < 0) return (int)f->kstats.size();
    if (i >= (int)f->kstats.size()) return -1;
    const auto &k = f->kstats[i];
    if (name && name_len > 0) {
        strncpy(name, k.name.c_str(), name_len - 1);
        name[name_len - 1] = 0;
    }
    if (ms) *ms = k.ms;
    if (launches) *launches = k.launches;
    if (flops) *flops = k.flops;
    return (int)f->kstats.size();
}

// ------------------------------------------------------------ VJP
IcmGb300Vjp *icm_gb300_vjp_create(int n, const double *S, int k) {
    return guarded<IcmGb300Vjp *>("icm_gb300_vjp_create", nullptr, [&]() -> IcmGb300Vjp * {
        if (!ensure_device()) return nullptr;
        std::string err;
        VjpPlan *v = vjp_plan_create(n, S, k, err);
        if (!v) { set_error("icm_gb300_vjp_create: " + err); return nullptr; }
        return reinterpret_cast<IcmGb300Vjp *>(v);
    });
}

int icm_gb300_vjp_run(IcmGb300Vjp *plan, int Q, const double *payout, const double *cot, double *grad_S,
                      double *grad_payout, int flags, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gb300_vjp_run", -1, [&]() -> int {
        if (!plan) { set_error("icm_gb300_vjp_run: null plan"); return -1; }
        if (!ensure_device()) return -1;
        VjpPlan *v = reinterpret_cast<VjpPlan *>(plan);
        std::string err;
        const int rc = vjp_plan_run(v, Q, payout, cot, grad_S, grad_payout, flags, stats, err);
        t_launches = v->p->launches;
        if (rc != 0) { set_error("icm_gb300_vjp_run: " + err); return -1; }
        return 0;
    });
}

int icm_gb300_vjp_run_dev(IcmGb300Vjp *plan, int Q, const double *d_payout, const double *d_cot,
                          double *d_grad_S, double *d_grad_payout, int flags, void *stream) {
    return guarded<int>("icm_gb300_vjp_run_dev", -1, [&]() -> int {
        const char *fn = "icm_gb300_vjp_run_dev";
        if (!plan || Q < 1) { set_error(std::string(fn) + ": invalid arguments"); return -1; }
        if (!ensure_device()) return -1;
        if (!device_pointer(d_payout, "payout", fn) || !device_pointer(d_cot, "cotangent", fn) ||
            !device_pointer(d_grad_S, "grad_S", fn) || !device_pointer(d_grad_payout, "grad_payout", fn))
            return -1;
        VjpPlan *v = reinterpret_cast<VjpPlan *>(plan);
        std::string err;
        DevIO io;
        io.st = static_cast<cudaStream_t>(stream);
        int rc = vjp_plan_enqueue(v, Q, d_payout, d_cot, flags, err, &io);
        if (rc == 0) rc = vjp_plan_finish(v, d_grad_S, d_grad_payout, nullptr, err, &io);
        t_launches = v->p->launches;
        if (rc != 0) { set_error(std::string(fn) + ": " + err); return -1; }
        return 0;
    });
}

void icm_gb300_vjp_destroy(IcmGb300Vjp *plan) { vjp_plan_destroy(reinterpret_cast<VjpPlan *>(plan)); }

double icm_gb300_vjp_device_ms(const IcmGb300Vjp *plan) {
    return plan ? reinterpret_cast<const VjpPlan *>(plan)->p->last_device_ms : 0.0;
}

int icm_gb300_equity_vjp(int n, const double *S, int Q, const double *payout, int k, const double *cot,
                         double *grad_S, double *grad_payout, int flags) {
    return guarded<int>("icm_gb300_equity_vjp", -1, [&]() -> int {
        if (n < 1 || k < 1 || k > n || Q < 1 || !S || !payout || !cot || !grad_S || !grad_payout) {
            set_error("icm_gb300_equity_vjp: invalid arguments (need 1 <= k <= n, Q >= 1)");
            return -1;
        }
        IcmGb300Vjp *v = icm_gb300_vjp_create(n, S, k);
        if (!v) return -1;
        const int rc = icm_gb300_vjp_run(v, Q, payout, cot, grad_S, grad_payout, flags, nullptr);
        icm_gb300_vjp_destroy(v);
        return rc;
    });
}

int icm_gb300_equity_vjp_batched(int T, const int *n, const int *k, const double *S, const double *payout, int Q,
                                 const double *cot, double *grad_S, double *grad_payout, int flags) {
    return guarded<int>("icm_gb300_equity_vjp_batched", -1, [&]() -> int {
        if (T < 1 || !n || !k || !S || !payout || !cot || !grad_S || !grad_payout || Q < 1) {
            set_error("icm_gb300_equity_vjp_batched: invalid arguments");
            return -1;
        }
        std::vector<long> so(T + 1, 0), po(T + 1, 0);
        for (int t = 0; t < T; ++t) {
            if (n[t] < 1 || k[t] < 1 || k[t] > n[t]) {
                set_error("icm_gb300_equity_vjp_batched: tournament " + std::to_string(t) + " needs 1 <= k <= n");
                return -1;
            }
            so[t + 1] = so[t] + n[t];
            po[t + 1] = po[t] + k[t];
        }
        if (!ensure_device()) return -1;
        std::string err;
        Forest *f = forest_create(T, n, k, S, err, /*vjp=*/true);
        if (!f) { set_error("icm_gb300_equity_vjp_batched: " + err); return -1; }
        f->graphs = false;   // one run: capturing would not pay
        const int rc = forest_vjp_run(f, Q, payout, cot, flags, grad_S, grad_payout, nullptr, err);
        t_launches = f->launches;
        forest_destroy(f);
        if (rc != 0) { set_error("icm_gb300_equity_vjp_batched: " + err); return -1; }
        return 0;
    });
}

IcmGb300Batch *icm_gb300_vjp_batch_create(int T, const int *n, const int *k, const double *S) {
    return guarded<IcmGb300Batch *>("icm_gb300_vjp_batch_create", nullptr, [&]() -> IcmGb300Batch * {
        if (!ensure_device()) return nullptr;
        std::string err;
        Forest *f = forest_create(T, n, k, S, err, /*vjp=*/true);
        if (!f) { set_error("icm_gb300_vjp_batch_create: " + err); return nullptr; }
        return reinterpret_cast<IcmGb300Batch *>(f);
    });
}

int icm_gb300_vjp_batch_run(IcmGb300Batch *b, int Q, const double *payout, const double *cot, double *grad_S,
                            double *grad_payout, int flags, IcmGpuRunStats *stats) {
    return guarded<int>("icm_gb300_vjp_batch_run", -1, [&]() -> int {
        if (!b) { set_error("icm_gb300_vjp_batch_run: null batch"); return -1; }
        if (!ensure_device()) return -1;
        Forest *f = reinterpret_cast<Forest *>(b);
        std::string err;
        const int rc = forest_vjp_run(f, Q, payout, cot, flags, grad_S, grad_payout, stats, err);
        t_launches = f->launches;
        if (rc != 0) { set_error("icm_gb300_vjp_batch_run: " + err); return -1; }
        return 0;
    });
}

// ------------------------------------------------------------ tuner, Q ladder
int icm_gb300_tuner_load(const char *path) {
    return guarded<int>("icm_gb300_tuner_load", -1, [&]() -> int {
        if (!path) { set_error("icm_gb300_tuner_load: null path"); return -1; }
        std::string err;
        const int r = tune_load(path, err);
        if (r < 0) set_error("icm_gb300_tuner_load: " + err);
        return r;
    });
}

int icm_gb300_tuner_save(const char *path) {
    return guarded<int>("icm_gb300_tuner_save", -1, [&]() -> int {
        if (!path) { set_error("icm_gb300_tuner_save: null path"); return -1; }
        std::string err;
        const int r = tune_save(path, err);
        if (r < 0) set_error("icm_gb300_tuner_save: " + err);
        return r;
    });
}

void icm_gb300_tuner_clear(void) { tune_clear(); }

int icm_gb300_tuner_lookup(int n, int k, int *block_size, int *fft_min_degree) {
    if (!block_size || !fft_min_degree || n < 1 || k < 1) return -1;
    tune_lookup(n, k, block_size, fft_min_degree);
    return (*block_size > 0) ? 1 : 0;
}

int icm_gb300_tuner_lookup_level(int n, int k, int level, int *spectral, int *cta_points) {
    if (!spectral || !cta_points || n < 1 || k < 1 || level < 0) return -1;
    *spectral = 1;
    *cta_points = 0;
    return tune_level_lookup(n, k, level, spectral, cta_points);
}

int icm_gb300_autotune(int n, const double *S, int Q, const double *payout, int k, int runs, int *block_size,
                       int *fft_min_degree, double *best_ms) {
    return guarded<int>("icm_gb300_autotune", -1, [&]() -> int {
        if (n < 1 || k < 1 || k > n || Q < 1 || !S || !payout || !block_size || !fft_min_degree || !best_ms) {
            set_error("icm_gb300_autotune: invalid arguments");
            return -1;
        }
        if (!ensure_device()) return -1;
        std::string err;
        if (tune_search(n, S, Q, payout, k, runs, block_size, fft_min_degree, best_ms, err) != 0) {
            set_error("icm_gb300_autotune: " + err);
            return -1;
        }
        return 0;
    });
}

int icm_gb300_equity_adaptive(int n, const double *S, const double *payout, int k, int Q0, double tol, int Qmax,
                              double *equity, int *Q_used, double *est_err) {
    return guarded<int>("icm_gb300_equity_adaptive", -1, [&]() -> int {
        if (n < 1 || k < 1 || k > n || Q0 < 2 || Qmax < Q0 || !(tol > 0.0) || !S || !payout || !equity) {
            set_error("icm_gb300_equity_adaptive: invalid arguments (need 1 <= k <= n, 2 <= Q0 <= Qmax, tol > 0)");
            return -1;
        }
        if (!ensure_device()) return -1;
        std::string err;
        Plan *p = plan_create(n, S, k, nullptr, err);
        if (!p) { set_error("icm_gb300_equity_adaptive: " + err); return -1; }
        std::vector<double> prev(n), cur(n);
        int Q = Q0;
        double e = INFINITY;
        int rc = plan_run(p, Q, payout, prev.data(), nullptr, err);
        long launches = p->launches;
        // double Q until two successive rules agree to tol (relative, per player,
        // against a floor of 1e-12 of the largest equity)
        while (rc == 0 && 2L * Q <= Qmax) {
            rc = plan_run(p, 2 * Q, payout, cur.data(), nullptr, err);
            launches += p->launches;
            if (rc != 0) break;
            Q *= 2;
            double mx = 0.0;
            for (int i = 0; i < n; ++i) mx = std::max(mx, std::fabs(cur[i]));
            const double floor = 1e-12 * mx;
            e = 0.0;
            for (int i = 0; i < n; ++i)
                e = std::max(e, std::fabs(cur[i] - prev[i]) / std::max(std::fabs(cur[i]), floor));
            prev.swap(cur);
            if (e <= tol) break;
        }
        plan_destroy(p);
        t_launches = launches;
        if (rc != 0) { set_error("icm_gb300_equity_adaptive: " + err); return -1; }
        memcpy(equity, prev.data(), sizeof(double) * n);
        if (Q_used) *Q_used = Q;
        if (est_err) *est_err = e;
        return 0;
    });
}

int icm_gpu_measure_fp64_gflops(double *gflops_out) {
    return guarded<int>("icm_gpu_measure_fp64_gflops", 0, [&]() -> int {
        if (!gflops_out || !ensure_device()) return 0;
        std::string err;
        if (measure_fp64_gflops(gflops_out, err) != 0) { set_error(err); return 0; }
        return 1;
    });
}

int icm_gb300_leaf_factors(int n, const double *arg, double *out) {
    return guarded<int>("icm_gb300_leaf_factors", -1, [&]() -> int {
        if (n < 0 || (n > 0 && (!arg || !out))) { set_error("icm_gb300_leaf_factors: invalid arguments"); return -1; }
        if (n == 0) return 0;
        if (!ensure_device()) return -1;
        std::string err;
        if (leaf_factors(n, arg, out, err) != 0) { set_error(err); return -1; }
        return 0;
    });
}

long icm_gpu_last_launch_count(void) { return t_launches; }

int icm_gb300_plan_set_profiling(IcmGpuPlan *plan, int enable) {
    Plan *p = reinterpret_cast<Plan *>(plan);
    if (!p) return -1;
    p->prof.on = enable != 0;
    p->kstats.clear();
    return 0;
}

int icm_gb300_plan_kernel_stats(const IcmGpuPlan *plan, int i, char *name, int name_len, double *ms,
                                long *launches, double *flops) {
    const Plan *p = reinterpret_cast<const Plan *>(plan);
    if (!p) return -1;
    const int cnt = (int)p->kstats.size();
    if (i < 0 || i >= cnt) return cnt;
    const Plan::KStat &k = p->kstats[i];
    if (name && name_len > 0) snprintf(name, (size_t)name_len, "%s", k.name.c_str());
    if (ms) *ms = k.ms;
    if (launches) *launches = k.launches;
    if (flops) *flops = k.flops;
    return cnt;
}

double icm_gb300_plan_device_ms(const IcmGpuPlan *plan) {
    const Plan *p = reinterpret_cast<const Plan *>(plan);
    return p ? p->last_device_ms : -1.0;
}

}  // extern "C"
