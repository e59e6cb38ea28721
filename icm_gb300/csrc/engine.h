// engine.h -- internal interface of the GB300 ICM engine (not installed).
//
// One plan = one tournament (or one batch of tournaments) with its tree
// geometry and device buffers.  The quadrature nodes are processed in chunks
// of `qc` nodes; every kernel of a chunk covers all nodes of the chunk
// (grid.y = node), so one launch per tree level does the work of qc trees.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/icm.h"
#include "../../include/icm_gb300.h"
#include "../../include/icm_gpu.h"
#include "kernels.h"

namespace icmg {

constexpr int kMaxLevels = 40;
constexpr int kMaxB = 32;            // largest leaf block
constexpr int kSmemFftMax = 8192;    // complex points one CTA transforms in shared memory

// Per tree level.  Level 0 = leaf blocks; level l >= 1 nodes are parents of
// level l-1 nodes.  Quantities for the *products computed at level l* (the
// FFT size etc.) are stored on level l.
struct Level {
    int nreal = 0;        // real nodes
    long deg = 0;         // players under a full node (B << l)
    int plen = 0;         // polynomial coefficients kept: min(deg+1, k)
    int glen = 0;         // g entries kept: min(deg, k)
    int pst = 0, gst = 0; // strides in doubles
    int fft = 0;          // 1: products/correlations of this parent level use FFTs
    int fftn = 0;         // real FFT size N (power of two)
    int npairs = 0;       // parents with two children (FFT levels)
    size_t P_q = 0, g_q = 0, spec_q = 0;   // per-node element counts (doubles / double2)
    double *P = nullptr, *g = nullptr;
    double2 *spec = nullptr;               // child spectra cached build -> propagate
    // Level kind (as a parent level): 0 schoolbook, 1 FFT on coefficients,
    // 2 spectral (nodes carried as spectra; spectral.cu).
    int kind = 0;
    // complex points per CTA of this level's one-CTA FFT launches (spectral
    // build/propagate/init and g-spectrum steps of single plans): items per
    // CTA = max(1, cta_pts / transform size); 0 = the default, 4096
    int cta_pts = 0;
    // spectral representation of this level's nodes: spec2 = DFT_{2 deg} (deg+1
    // bins) and end coefficients, present when the parent level is spectral;
    // G = DFT_{deg}(g) (deg/2+1 bins), present when this level is spectral
    size_t spec2_q = 0, ends_q = 0, G_q = 0;
    double2 *spec2 = nullptr, *G = nullptr;
    double *ends = nullptr;
};

// The per-node buffers of one piece of a node chunk: the plan's own pointers
// offset by the piece's first node slot (same arena), so the pieces of a
// chunk run concurrently, one stream each.
constexpr int kMaxChunkParts = 4;
struct ChunkView {
    Level lv[kMaxLevels];
    double *a = nullptr, *contrib = nullptr, *blockP = nullptr;
    double2 *fa = nullptr, *fb = nullptr, *fc = nullptr;
    cudaStream_t st = nullptr;
};

struct Plan;

// Points a plan's per-node buffers and its stream at a chunk piece's view
// while the scope lives (host-side enqueue only; a null view leaves the plan
// as it is), so that code written for the plan's own buffers enqueues that
// piece.
struct PieceScope {
    Plan *p;
    bool on;
    ChunkView saved;
    PieceScope(Plan *plan, const ChunkView *view);
    ~PieceScope();
    PieceScope(const PieceScope &) = delete;
    PieceScope &operator=(const PieceScope &) = delete;
};

struct Plan {
    int n = 0, k = 0, B = 0, nblocks = 0, L = 0;
    int fft_min_deg = 64;
    bool spectral = true;           // use spectral levels where they apply
    bool coeff_only = false;        // never use spectral levels
    bool vjp = false;               // forward tree of a single VJP plan (its adjoint reads every level)
    bool zskip = true;              // prune wholly-zero tree nodes per quadrature node
    int Lf = 0;                     // bottom schoolbook levels fused into the subtree kernels
    bool small = false;             // whole pipeline in one CTA per node (small.cu)
    bool linear = false;            // the linear engine (linear.cu)
    double *d_ck = nullptr;         // [qc][ck per node] linear-engine checkpoints
    std::vector<double> S_sorted;
    std::vector<int> perm;          // perm[i] = original index of sorted player i
    std::vector<int> inv_perm;
    double Smax = 0.0;
    Level lv[kMaxLevels];
    int qc = 1;                     // quadrature nodes per chunk
    int qmax = 0;                   // capacity of the node arrays
    IcmGpuOptions opts{};
    // device
    cudaStream_t stream = nullptr;
    // the root's payout spectrum runs on a side stream, overlapping the build
    // (one-kernel spectral roots only): fork after the uploads, join before
    // the root's propagate
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool root_forked = false;
    // node chunks split in nparts pieces, one stream each (tree path): each
    // piece's first node slot and buffers (part[0] unused: the plan's own),
    // events ordering the node sums
    int nparts = 1;
    int part_off[kMaxChunkParts] = {};
    ChunkView part[kMaxChunkParts];
    cudaEvent_t ev_split = nullptr, ev_acc[kMaxChunkParts] = {};
    char *arena = nullptr;
    size_t arena_bytes = 0;
    bool pooled = false;            // arena from the stream-ordered pool
    double *d_S = nullptr;          // sorted stacks
    int *d_perm = nullptr;
    double *d_payout = nullptr;     // g at the root: payout zero-padded to glen(root)
    double *d_a = nullptr;          // [qc][n]
    double *d_blockP = nullptr;     // [qc][nblocks][B+1]
    double *d_contrib = nullptr;    // [qc][n]
    double *d_acc = nullptr;        // [n] sorted order
    double *d_out = nullptr;        // [n] original order
    double *d_node = nullptr;       // [qmax][3]: logv, w, 1/v for the active nodes
    int *d_z = nullptr;             // [qmax] zero prefix of each active node (same allocation)
    std::vector<int> h_z;
    unsigned *d_counter = nullptr;  // finished CTAs of a small-path launch
    uint8_t *d_active = nullptr;    // [n] sorted order (subset), or null
    uint8_t *d_hot = nullptr;       // hot bitmap, all levels
    size_t hot_off[kMaxLevels] = {};
    double2 *d_fa = nullptr, *d_fb = nullptr, *d_fc = nullptr;  // FFT work buffers
    size_t fft_work = 0;            // double2 per buffer
    size_t fa_elems = 0, fb_elems = 0;   // FFT work buffers per node (double2)
    size_t tree_q_bytes = 0;        // tree buffers per node: block products, levels, work buffers
    bool subset = false;
    long launches = 0;
    // graph replay (enable_graphs)
    cudaGraphExec_t graph = nullptr;
    int graph_nq = -1;
    const double *graph_node = nullptr;   // the node buffer the graph reads
    bool graph_subset = false;            // captured with the subset masks
    long graph_launches = 0;
    bool graph_tma = false;               // the captured sequence holds TMA column passes
    double peak_bytes = 0;
    // timing: events around the kernel sequence of each run, optional
    // per-kernel events (prof.on) aggregated by kernel name
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stream-ordered runs on device buffers: the caller's stream -> the plan's
    // stream (inputs ready) and back (outputs written)
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    double last_device_ms = 0.0;
    // stage timing (opts.verbose, as the reference's instrumented path):
    // events at the stage boundaries of every chunk, 5 per chunk
    std::vector<cudaEvent_t> stage_ev;
    size_t stage_used = 0;
    double stage_ms[4] = {};        // block build, tree build, propagate, leaf extract
    Prof prof;
    struct KStat {
        std::string name;
        double ms;
        long launches;
        double flops;
    };
    std::vector<KStat> kstats;
};

// lifecycle (engine.cu)
// geometry only: validation, sort, levels, per-node element counts
int plan_geometry(Plan *p, int n, const double *S, int k, std::string &err);
// caps the player sort's threads on the calling thread while it lives (host
// code that already runs on many threads sorts on one thread each)
struct SortThreadCap {
    int prev;
    explicit SortThreadCap(int cap);
    ~SortThreadCap();
    SortThreadCap(const SortThreadCap &) = delete;
    SortThreadCap &operator=(const SortThreadCap &) = delete;
};
// device allocation of plans, batches and VJPs (stream-ordered pool or plain
// cudaMalloc), with the test hook that makes the n-th one fail
cudaError_t dev_alloc(void **ptr, size_t bytes, cudaStream_t st, bool pooled);
void set_alloc_failure(int nth);
// invariants the kernels rely on (host only): 0, or -1 with the violation
int plan_check_geometry(const Plan *p, std::string &why);
// new stacks for a plan of the same shape (n, k): sort, sorted copies on the
// host and the device; the tree geometry and buffers are kept
int plan_restack(Plan *p, const double *S, std::string &err);
// player order: stacks descending, ties by index; S_sorted (optional) gets the
// stacks in that order.  Returns the first index whose stack is not finite and
// positive, else -1 (the order is then still a permutation).
int sort_players_desc(const double *S, int n, std::vector<int> &perm, double *S_sorted = nullptr);
// p->inv_perm for the current order (built on first use after a sort)
void plan_inv_perm(Plan *p);
// tree buffers for chunks of qc nodes from `base` (nullptr: size only)
size_t plan_tree_layout(Plan *p, int qc, char *base);
// coeff_only: every FFT level on coefficients; q_bytes_scale sizes the node
// chunk for callers that add per-node buffers of their own; vjp: the forward
// tree of a single VJP plan (tree engine only, spectral levels under the VJP's
// rules, plan_geometry)
Plan *plan_create(int n, const double *S, int k, const IcmGpuOptions *opts, std::string &err,
                  bool coeff_only = false, double q_bytes_scale = 1.0, size_t budget = 0, bool vjp = false);
// launch sequence of one chunk of nq nodes (engine.cu); divide = false stops
// after the propagate pass (the tree of the chunk stays in the plan's buffers).
// view: run on a chunk piece's buffers and stream instead of the plan's own;
// the node sum waits for acc_wait and records acc_done when they are given.
void run_chunk(Plan *p, int q0, int nq, const double2 *tw, int logTW, bool first, bool divide,
               const ChunkView *view = nullptr, cudaEvent_t acc_wait = nullptr, cudaEvent_t acc_done = nullptr);
// nodes of piece i (of np) of a chunk with r nodes left for pieces i .. np-1:
// an even share within the piece's node slots, the last piece the rest
int chunk_piece_nodes(const Plan *p, int i, int np, int r);
static inline int plan_ilog2(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
void plan_destroy(Plan *p);
int plan_set_targets(Plan *p, const int *targets, int n_targets, std::string &err);
// q_begin, q_end: the rule's nodes [q_begin, q_end) only (q_end < 0: all Q)
// Device memory in and out of a run, ordered on the caller's stream `st`: the
// run starts after the work already queued on st, st's later work sees the
// outputs, and the call returns without waiting for the GPU.
struct DevIO {
    cudaStream_t st = nullptr;
};
// q_begin, q_end: the rule's nodes [q_begin, q_end) only (q_end < 0: all Q);
// dev: payout and equity are device pointers, stream-ordered on dev->st
int plan_run(Plan *p, int Q, const double *payout, double *equity, IcmGpuRunStats *stats,
             std::string &err, int q_begin = 0, int q_end = -1, const DevIO *dev = nullptr);
// event pair of stream-ordered runs, created on first use
cudaError_t plan_dev_events(Plan *p);
int select_block_size(int n, int k);
int select_fft_min(int n, int k);   // schoolbook/FFT crossover degree (config, tuner table, built-in)

// quadrature nodes (host), restating the reference's erfc-trapezoid rule
void make_nodes(int Q, double Smax, std::vector<double> &logv, std::vector<double> &w);
// number of sorted players with a leaf factor of exactly 0 at a node
int zero_prefix(const double *S_sorted, int n, double logv);

// device-wide twiddle table exp(-2 pi i t / 2^logTW); *logTW receives the
// table's size, which may exceed the request
const double2 *twiddles(int logN, cudaStream_t s, std::string &err, int *logTW);
// host image of those tables (twiddle.cpp)
size_t twiddle_bytes(int logTW);
void fill_twiddles(int logTW, std::vector<unsigned char> &out);

// probes (probes.cu)
int measure_fp64_gflops(double *out, std::string &err);
int leaf_factors(int n, const double *arg, double *out, std::string &err);
int measure_hbm_gbps(double *out, std::string &err);

// tuner table (tune.cpp)
void tune_lookup(int n, int k, int *B, int *fft_min);
int tune_cta_points(int n, int k, int level);   // the table's points per CTA at a level (0: none)
int tune_spectral_ok(int n, int k, int level);  // 0 where the table keeps a level on coefficients
int tune_level_lookup(int n, int k, int level, int *spectral, int *pts);
void tune_record_level(int n, int k, int level, int spectral, int pts, double ms);
void tune_erase_level(int n, int k, int level);
int select_cta_points(int n, int k, int level);
extern std::atomic<long> g_tune_generation;   // changes of the tuner table (tune.cpp)
// built-in choices for GB300 where the caller's table has none (0: none)
void tune_builtin(int n, int k, int *B, int *fft_min);
void tune_record(int n, int k, int B, int fft_min, double ms);
int tune_load(const char *path, std::string &err);
int tune_save(const char *path, std::string &err);
void tune_clear();
int tune_search(int n, const double *S, int Q, const double *payout, int k, int runs, int *bestB, int *best_fft,
                double *best_ms, std::string &err);

// process-wide configuration
extern IcmGb300Config g_config;
extern int g_device;

}  // namespace icmg
