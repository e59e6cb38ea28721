// kernels.h -- host-side launchers of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <vector>

namespace icmg {

struct Level;
struct Plan;

// Optional per-launch timing: when `on`, every launcher brackets its kernel
// with CUDA events on the launch stream and records the kernel's algorithmic
// FP64 flop count (the plan aggregates them by name after the run).
struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
    double flops;
};
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<ProfRec> recs;
    double scale = 1.0;   // share of the launch's nominal work not pruned (set by the caller)
    cudaEvent_t get() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(const char *name, double flops, cudaStream_t st) {
        if (!on) return;
        ProfRec r{name, get(), get(), flops * scale};
        cudaEventRecord(r.a, st);
        recs.push_back(r);
    }
    void end(cudaStream_t st) {
        if (on) cudaEventRecord(recs.back().b, st);
    }
};

// Zero prefix of a quadrature node: players are sorted by stack, descending,
// so the players whose leaf factor a = exp(S logv) is exactly 0 (S logv < -700)
// are the first zp[q0 + q] of them.  A tree node lying wholly inside that
// prefix is the monomial x^deg and nothing of it reaches an equity (those
// players' weights are 0): builds write the monomial without transforms,
// propagates skip it.  span = players under one node of the level the kernel
// decides on.  zp == nullptr: no pruning.
struct ZeroPrefix {
    const int *zp;
    int q0;
    long span;
};
__host__ __device__ __forceinline__ bool zp_cold(const ZeroPrefix &z, int q, long node) {
    return z.zp && (node + 1) * z.span <= (long)z.zp[z.q0 + q];
}

// ---- kernel argument blocks.  Each kernel body is a __device__ function of
// (args, bx, q): bx the block index within one tree level of one tournament,
// q the quadrature node within the chunk.  Single plans launch it with
// grid (nbx, nq); batches of tournaments launch one work list per level
// (batch.cu) whose blocks map to (tournament level, bx, q).
struct LeafArgs {
    int B, n, nblocks;
    const double *S, *node;
    int q0;
    double *a, *blockP, *P0;
    int pst0, plen0;
    int nbx;
    size_t aq;          // per-node stride of a (n for one tournament)
};
struct SchoolBuildArgs {
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc, nreal_c;
    double *Pp;
    size_t Pp_q;
    int pst_p, lp, nreal_p, j0;
    int nbx;
    ZeroPrefix z;
};
struct SchoolPropArgs {
    const double *gp;
    size_t gp_q;
    int gst_p, gpl;
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc;
    double *gc;
    size_t gc_q;
    int gst_c, gcl, nreal_c;
    const uint8_t *hot_c;
    int c0;
    int nbx;
    ZeroPrefix z;
};
struct DivideArgs {
    int B, n, k, nblocks;
    const double *S, *node;
    int q0;
    const double *a, *blockP, *g0;
    size_t g0_q;
    int gst0;
    const uint8_t *active;
    double *contrib;
    int nbx;
    size_t aq;          // per-node stride of a and contrib
};

struct SpecInitArgs {
    const double *P;
    size_t P_q;
    int pst, plen, nreal, logd;
    double2 *spec2;
    size_t s2_q;
    double *ends;
    size_t e_q;
    const double2 *tw;
    int logTW;
    int nbx;
    ZeroPrefix z;
    int cb;   // items per CTA (single-plan launches may lower it; work lists keep the default)
};
struct SpecBuildArgs {
    const double2 *cspec;
    size_t cs_q;
    const double *cends;
    size_t ce_q;
    int nreal_c, nreal_p, logD;
    double2 *pspec;
    size_t ps_q;
    double *pends;
    size_t pe_q;
    double *Pout;
    size_t Po_q;
    int pst_p, plen_p;
    const double2 *tw;
    int logTW;
    int nbx;
    ZeroPrefix z;
    int cb;   // parents per CTA (single-plan launches; the packed work lists have their own)
};
struct GspecArgs {
    const double *g;
    size_t g_q;
    int gst, glen, nreal, logd;
    double2 *G;
    size_t G_q;
    const uint8_t *hot;
    const double2 *tw;
    int logTW;
    int nbx;
    ZeroPrefix z;
    int cb;   // items per CTA (single-plan launches may lower it; work lists keep the default)
};
struct SpecPropArgs {
    const double2 *Gp;
    size_t Gp_q;
    const double2 *cspec;
    size_t cs_q;
    int nreal_c, npar, logD;
    double2 *Gout;
    size_t Go_q;
    double *gout;
    size_t go_q;
    int gst_c, glen_c;
    const uint8_t *hot_c;
    const double2 *tw;
    int logTW;
    int nbx;
    ZeroPrefix z;
    int cb;   // parents per CTA (single-plan launches; the packed work lists have their own)
};
// items per CTA of a single-plan launch of nitems items over nq nodes: cb,
// halved while the grid would hold fewer than two CTAs per SM (kernels.cu)
int short_grid_cb(int cb, int nitems, int nq);

struct FusedBuildArgs {
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc, npairs, logN;
    double *Pp;
    size_t Pp_q;
    int pst_p, lp;
    double2 *spec;
    const double2 *tw;
    int logTW, spectra_only;
    int nbx;
    ZeroPrefix z;
    int cb;   // pairs per CTA (single-plan launches; the packed work lists have their own)
};
struct FusedPropArgs {
    const double *gp;
    size_t gp_q;
    int gst_p, gpl, npairs, logN;
    const double2 *spec;
    double *gc;
    size_t gc_q;
    int gst_c, gcl;
    const uint8_t *hot_c;
    const double2 *tw;
    int logTW;
    int nbx;
    ZeroPrefix z;
    int cb;   // pairs per CTA (single-plan launches; the packed work lists have their own)
};

// ---- argument builders shared by the single-plan launchers and the work
// lists.  Each fills its block count per node (nbx; 0 = no work), the
// dynamic shared memory where the kernel uses some, and the algorithmic FP64
// flops per node (*fq).  Leaf and divide take the node offset at launch.
LeafArgs leaf_args(int B, int n, int nblocks, const double *S, const double *node, double *a, size_t aq,
                   double *blockP, double *P0, int pst0, int plen0, double *fq);
DivideArgs divide_args(int B, int n, int k, int nblocks, const double *S, const double *node, const double *a,
                       size_t aq, const double *blockP, const double *g0, size_t g0_q, int gst0, const uint8_t *active,
                       double *contrib, double *fq);
SchoolBuildArgs school_build_args(const Level &c, const Level &p, int j0, double *fq);
SchoolPropArgs school_prop_args(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const uint8_t *hot_c,
                                int c0, double *fq);
SpecInitArgs spec_init_args(const Level &v, const double2 *tw, int logTW, double *fq, size_t *smem);
SpecBuildArgs spec_build_args(const Level &c, const Level &p, bool write_coeffs, const double2 *tw, int logTW,
                              double *fq, size_t *smem);
GspecArgs gspec_args(const double *g, size_t g_q, int gst, int glen, int nreal, const Level &v, double2 *G, size_t G_q,
                     const uint8_t *hot, const double2 *tw, int logTW, double *fq, size_t *smem);
SpecPropArgs spec_prop_args(const double2 *Gp, size_t Gp_q, const Level &c, const Level &p, bool children_spectral,
                            const uint8_t *hot_c, const double2 *tw, int logTW, double *fq, size_t *smem);
FusedBuildArgs fused_build_args(const Level &c, const Level &p, bool spectra_only, const double2 *tw, int logTW,
                                double *fq, size_t *smem);
FusedPropArgs fused_prop_args(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p,
                              const uint8_t *hot_c, const double2 *tw, int logTW, double *fq, size_t *smem);

// ---- work lists (batch.cu drives them).  One launch runs one kind of step
// for many tournaments: grid (nctas, nq), tab[blockIdx.x] = (descriptor,
// block within the descriptor), blockIdx.y = node within the chunk.
enum class WOp : int {
    Leaf, SchoolBuild, SchoolProp, Divide, SpecInit, SpecBuild, Gspec, SpecProp, FusedBuild, FusedProp, SubBuild, SubProp,
    AdjLeafUp, AdjUpSchool, AdjUpFused, AdjDownSchool, AdjDownFused, AdjLeafDown, Small, Linear,
    AdjSpecReal, AdjSpecUp, AdjSpecDown
};
// B: leaf block size of the launch (Leaf and Divide lists are keyed by it)
void launch_worklist_basic(WOp op, int B, const void *desc, const int2 *tab, int nctas, int nq, int q0,
                           cudaStream_t st);
void launch_worklist_spec(WOp op, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                          cudaStream_t st);
// packed work lists: slots[s] = (descriptor, item); a CTA takes cb consecutive
// slots, which may belong to different tournaments (SpecBuild, SpecProp)
void launch_packed_spec(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                        cudaStream_t st);
void launch_packed_fused(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                         cudaStream_t st);
size_t spec_smem_bytes(int M);     // dynamic shared memory of the spectral kernels
size_t fused_smem_bytes(int N);    // dynamic shared memory of the fused kernels

// ---- bottom subtree (subtree.cu): leaf blocks plus the lowest Lf schoolbook
// levels in one kernel per direction, kSubBlocks leaf blocks per CTA
constexpr int kSubBlocks = 256;
constexpr int kSubMaxLevels = 8;
struct SubLevel {
    double *P;
    size_t P_q;
    int pst, plen, nreal;
    double *g;
    size_t g_q;
    int gst, glen;
    const uint8_t *hot;   // subset mask of this level, or null
    long deg;
};
struct SubArgs {
    int B, n, k, nblocks, Lf;
    const double *S, *node;
    double *a;
    size_t aq;
    double *blockP;
    SubLevel lv[kSubMaxLevels + 1];
    const uint8_t *active;
    double *contrib;
    int write_g, do_divide;
    ZeroPrefix z;   // z.q0: the chunk's first node (also the node table's offset)
    int nbx;
};
struct SubFlops {   // algorithmic FP64 flops per quadrature node
    double leaf, divide;
    double build[kSubMaxLevels + 1], prop[kSubMaxLevels + 1];   // level l products / middle products
};
SubArgs sub_args(const Plan *p, int Lf, const double *S, const double *node, double *a, size_t aq,
                 const uint8_t *active, double *contrib, bool write_g, bool do_divide, SubFlops *fl);
void launch_sub_build(const SubArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq);
void launch_sub_prop(const SubArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq);
void launch_worklist_sub(WOp op, int B, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st);
size_t sub_build_smem(int B);
size_t sub_prop_smem(int B);
void sub_set_smem_limits();

// ---- small tournaments (small.cu): the whole per-node pipeline in one CTA
constexpr size_t kOneCtaSmem = 113 * 1024;   // above this only one CTA fits on an SM
constexpr size_t kSmallMaxSmem = 200 * 1024;
constexpr int kSmallMaxN = 1536;   // the largest default limit of the small path (plan_small_ok)
constexpr int kSmallMaxLevels = 24;
struct SmallLevel {
    int nreal, pst, plen, gst, glen;
    int offP;        // shared-memory offset of the level's rows (doubles)
    int pad;
};
struct SmallArgs {
    int B, n, k, nblocks, L;
    const double *S, *node, *payout;
    const uint8_t *active;   // subset mask (sorted order), or null
    double *contrib;         // [q][aq] per-player shares
    size_t aq;
    // single solves: the last CTA sums the shares over the nodes in order
    // (null counter: the caller sums them, as forests do)
    unsigned *counter;
    double *acc, *out;
    const int *perm;
    int first, last;
    int q0;                  // the chunk's first node
    int offA, offG0, offG1;  // shared-memory offsets: leaf factors, two g buffers
    size_t smem;
    SmallLevel lv[kSmallMaxLevels];
    int nbx;
};
bool plan_small_ok(const Plan *p);
size_t small_smem_bytes(const Plan *p);
double small_flops(const Plan *p);   // algorithmic FP64 flops per node
SmallArgs small_args(const Plan *p, const double *S, const double *node, const double *payout, double *contrib,
                     size_t aq, const uint8_t *active);
void launch_small(const SmallArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq);
void launch_worklist_small(int B, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                           cudaStream_t st);
void small_set_smem_limits();
// one-shot solve of a small tournament without a plan: 1 when solved, 0 when
// the tournament is not on the small path, -1 on error (err set)
int small_solve(int n, const double *S, int Q, const double *payout, int k, double *equity, const int *targets,
                int n_targets, IcmGpuRunStats *stats, long *launches, std::string &err);
void small_context_release();

// ---- linear engine (linear.cu): one warp per (tournament, node), k <= 256
constexpr int kLinearMaxK = 256;
struct LinearArgs {
    int R, n, k;
    const double *S, *node, *payout;
    double *a;               // [q][aq] leaf factors (kept for the backward replays)
    double *contrib;         // [q][aq] per-player shares
    size_t aq;
    const uint8_t *active;   // subset mask (sorted order), or null
    double *ck;              // [q][ck_q] checkpoints of the forward sweep
    size_t ck_q;
    const int *zp;           // zero prefix per node (q0-based table), or null
    int nbx;
};
int linear_lanes(int k);   // R: coefficients per lane
bool plan_linear_auto(int n, int k);
size_t linear_ck_per_node(int n, int k);
LinearArgs linear_args(const Plan *p, const double *S, const double *node, const double *payout, double *a,
                       double *contrib, size_t aq, const uint8_t *active, double *ck, const int *zp);
double linear_flops(const Plan *p);
void launch_linear(const LinearArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq);
void launch_worklist_linear(int R, const void *desc, const int2 *tab, int nctas, int nq, int q0, cudaStream_t st);

void fft_set_smem_limits();

// one-kernel FFT levels (fused.cu), used when the level's real FFT size fits
bool fused_ok(int N);
void fused_set_smem_limits();
void launch_fused_build(const Level &c, const Level &p, int nq, bool spectra_only, const double2 *tw, int logTW,
                        cudaStream_t st, Prof *pr, const int *zp = nullptr, int zq0 = 0);
// spectral levels (spectral.cu)
constexpr int kSpecMaxD = 8192;   // largest child degree of a spectral level
void spec_set_smem_limits();
void launch_spec_init(const Level &v, int nq, const double2 *tw, int logTW, cudaStream_t st, Prof *pr,
                      const int *zp = nullptr, int zq0 = 0);
void launch_spec_build(const Level &c, const Level &p, bool write_coeffs, int nq, const double2 *tw, int logTW,
                       cudaStream_t st, Prof *pr, const int *zp = nullptr, int zq0 = 0);
void launch_gspec_init(const double *g, size_t g_q, int gst, int glen, int nreal, const Level &v, double2 *G,
                       size_t G_q, int nq, const uint8_t *hot, const double2 *tw, int logTW, cudaStream_t st,
                       Prof *pr, const int *zp = nullptr, int zq0 = 0);
void launch_spec_prop(const double2 *Gp, size_t Gp_q, const Level &c, const Level &p, bool children_spectral, int nq,
                      const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr,
                      const int *zp = nullptr, int zq0 = 0);

// spectral levels with transforms beyond one CTA (spectral_big.cu)
void launch_specbig_build(const Level &c, const Level &p, bool write_coeffs, int nq, double2 *buf, double2 *scratch,
                          const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                          const int *zp = nullptr, int zq0 = 0);
void launch_specbig_prop(const double2 *Gp, size_t Gp_q, const Level &c, int nq, const uint8_t *hot_c, double2 *buf,
                         double2 *scratch, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                         const int *zp = nullptr, int zq0 = 0);
void launch_gspecbig_init(const double *g, size_t g_q, int gst, int glen, int nreal, int logd, double2 *G, size_t G_q,
                          int nq, const uint8_t *hot, double2 *buf, double2 *scratch, const double2 *tw, int logTW,
                          cudaStream_t st, long *launches, Prof *pr, const int *zp = nullptr, int zq0 = 0);

void launch_fused_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                       const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr,
                       const int *zp = nullptr, int zq0 = 0);
// items of a batched transform that lie wholly inside a node's zero prefix
// are skipped: item i is tree node (i % per_q) of chunk node (i / per_q)
struct FftSkip {
    const int *zp = nullptr;
    int q0 = 0;
    long span = 0;
    int per_q = 1;
    long item0 = 0;
};
// shift = +1 / -1 (forward only): the transforms half-shifted by +1/2 / -1/2 bin
int fft_batched(double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw, int logTW,
                cudaStream_t st, long *launches, Prof *pr, FftSkip skip = FftSkip(), int shift = 0);
// the column pass alone of fft_batched's four-step split (data -> scratch);
// shift = +1 / -1 (forward only): the transform half-shifted by +1/2 / -1/2 bin
void launch_fft4_cols(const double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw,
                      int logTW, cudaStream_t st, long *launches, Prof *pr, FftSkip skip = FftSkip(), int shift = 0);
void specbig_set_smem_limits();
// the column pass with its tile staged by TMA (tma_cols.cu); false: not launched
bool launch_fft4_cols_tma(const double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw,
                          int logTW, int cbA, cudaStream_t st, FftSkip skip, int shift = 0);
void tma_set_smem_limits();
int tma_take_failures();
extern std::atomic<long> g_tma_launches;   // column passes launched through TMA (all plans)

void launch_leaf(int B, int n, int nblocks, const double *S, const double *node, int q0, int nq, double *a,
                 double *blockP, double *P0, int pst0, int plen0, cudaStream_t st, Prof *pr);
void launch_divide(int B, int n, int k, int nblocks, const double *S, const double *node, int q0, int nq,
                   const double *a, const double *blockP, const double *g0, size_t g0_q, int gst0,
                   const uint8_t *active, double *contrib, cudaStream_t st, Prof *pr);
void launch_school_build(const Level &c, const Level &p, int nq, int j0, cudaStream_t st, Prof *pr,
                         const int *zp = nullptr, int zq0 = 0);
void launch_school_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, int nq,
                        const uint8_t *hot_c, int c0, cudaStream_t st, Prof *pr, const int *zp = nullptr,
                        int zq0 = 0);
void launch_accumulate(int n, int nq, const double *contrib, double *acc, int first, cudaStream_t st, Prof *pr);
void launch_scatter(int n, const double *acc, const int *perm, const uint8_t *active, double *out,
                    cudaStream_t st);
void launch_fft_build(const Level &c, const Level &p, int nq, double2 *fa, double2 *fb, double2 *fc,
                      bool spectra_only, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                      const int *zp = nullptr, int zq0 = 0);
void launch_fft_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                     const uint8_t *hot_c, double2 *fa, double2 *fb, double2 *fc, const double2 *tw, int logTW,
                     cudaStream_t st, long *launches, Prof *pr, const int *zp = nullptr, int zq0 = 0);

}  // namespace icmg
