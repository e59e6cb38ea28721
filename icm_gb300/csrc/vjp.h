// vjp.h -- plans for vector-Jacobian products of the equities (vjp.cu).
// Internal to the library.
#pragma once

#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"

namespace icmg {

// ---- argument blocks of the adjoint kernels (vjp.cu); one tournament level
// each, so single plans and batch work lists run the same bodies.  zp/span:
// zero-prefix pruning of the level the kernel decides on (null: none).
struct AdjLeafUpArgs {
    int B, n, k, nblocks;
    const double *S, *node, *a;
    size_t aq;             // per-node stride of a
    const double *cot;
    double *gb0;
    size_t gb0_q;
    int gst0;
    double *blockW;        // [q][nblocks][B] full gbar of the blocks (k < B), or null
    int nbx;
};
struct AdjLeafDownArgs {
    int B, n, k;
    const double *S, *node, *a;
    size_t aq;             // per-node stride of a, contrib, partA, partB
    const double *cot, *g0;
    size_t g0_q;
    int gst0;
    const double *Pb0;
    size_t Pb0_q;
    int pst0, plen0;
    double *contrib, *partA, *partB;
    const double *blockP;  // [q][nblocks][B+1] block products from the forward leaf step
    int nblocks;
    const double *W;       // gbar of the blocks, all bs coefficients: + q Wq + b Wst
    size_t Wq;
    int Wst;
    int nbx;
};
struct AdjUpSchoolArgs {
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc, nreal_c;
    const double *gbc;
    size_t gbc_q;
    int gst_c, glen_c;
    double *gbp;
    size_t gbp_q;
    int gst_p, gpl, nreal_p, j0;
    const int *zp;
    long span;
    int nbx;
};
struct AdjDownSchoolArgs {
    const double *gp;
    size_t gp_q;
    int gst_p, gpl;
    const double *Pbp;
    size_t Pbp_q;
    int pst_p, lp;
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc;
    const double *gbc;
    size_t gbc_q;
    int gst_c, glen_c;
    double *Pbc;
    int nreal_c, c0;
    const int *zp;
    long span;
    int nbx;
};
struct AdjUpFusedArgs {
    const double *gbc;
    size_t gbc_q;
    int gst_c, glen_c, npairs, logN;
    const double2 *spec;
    double2 *gspec;
    double *gbp;
    size_t gbp_q;
    int gst_p, gpl;
    const double2 *tw;
    int logTW;
    const int *zp;
    long span;
    int nbx;
    int cb;   // pairs per CTA (single plans; the packed work lists have their own)
};
struct AdjDownFusedArgs {
    const double *gp;
    size_t gp_q;
    int gst_p, gpl;
    const double *Pbp;
    size_t Pbp_q;
    int pst_p, lp;
    const double *Pc;
    size_t Pc_q;
    int pst_c, lc, npairs, logN;
    const double2 *spec, *gspec;
    double *Pbc;
    const double2 *tw;
    int logTW;
    const int *zp;
    long span;
    int nbx;
    int cb;   // pairs per CTA (single plans; the packed work lists have their own)
};

// one tournament's adjoint buffers and the views of shared arrays it uses
struct VjpBufs {
    double *gb[kMaxLevels];      // gbar per level, shaped as g (gb[0] is the root's when L = 1)
    size_t gb_q[kMaxLevels];
    int gb_st[kMaxLevels];
    double *Pb[kMaxLevels];      // Pbar per level, shaped as P
    double2 *gspec[kMaxLevels];  // children's gbar spectra (one-kernel FFT levels)
    double *root;                // root gbar rows (L >= 2): root + q root_q, stride kst
    size_t root_q;
    int kst;
    const double *cot;           // cotangent, sorted order
    double *a;                   // leaf factors and dL/dS shares: + q aq
    size_t aq;
    double *contrib;
    const double *root_acc;      // what the payout gradient sums over nodes
    size_t root_acc_q;
    double *blockW;              // [qc][nblocks][B] full gbar of the leaf blocks when k < B
    // spectral levels (vjp_spec.cu): gbar spectra DFT_{2 deg}(gbar) (deg + 1
    // bins per node) of the nodes whose parent level is spectral; folded Pbar
    // spectra DFT_{deg}(Pbar with Pbar[deg] added to Pbar[0]) (deg/2 + 1 bins)
    // and Pbar's end coefficients (Pbar[0], Pbar[deg]) of spectral levels
    // below the root
    double2 *Gb2[kMaxLevels];
    size_t Gb2_q[kMaxLevels];
    double2 *PF[kMaxLevels];
    size_t PF_q[kMaxLevels];
    double *Pe[kMaxLevels];
    size_t Pe_q[kMaxLevels];
};

struct VjpPlan {
    Plan *p = nullptr;                   // coefficient-level plan (forward tree buffers)
    char *arena = nullptr;               // adjoint buffers
    size_t arena_bytes = 0;
    int kst = 0;                         // stride of the root's gbar (k rounded up to even)
    double *d_cot = nullptr;             // cotangent, sorted order
    double *d_gradS = nullptr;           // dL/dS, sorted order (ordered sum over nodes)
    double *d_gradP = nullptr;           // dL/dpayout
    double *d_root = nullptr;            // [qc][kst] gbar of the root
    VjpBufs bufs{};
    // per chunk piece (the plan's node slots from part_off[i]): the same
    // buffers offset by the piece's first slot; pbufs[0] = bufs
    VjpBufs pbufs[kMaxChunkParts]{};
    std::vector<double> h_cot;
    // node terms (flag 1): per-player partials [qc][n] and per-node sums
    double *d_partA = nullptr, *d_partB = nullptr, *d_nodeA = nullptr, *d_nodeB = nullptr;
    int node_cap = 0;
    // an enqueued run awaiting vjp_plan_finish
    bool pending = false, pnode = false;
    int pQ = 0, pnact = 0;
    std::vector<int> pqidx;
    std::vector<double> pw;
    double pt0 = 0.0;
};

// budget: device bytes for the plan's node chunk (0 = the engine's default)
VjpPlan *vjp_plan_create(int n, const double *S, int k, std::string &err, size_t budget = 0);
void vjp_plan_destroy(VjpPlan *v);
// enqueue a run on the plan's stream without waiting; finish waits, copies
// the gradients out and adds the node terms
// dev: payout, cot, grad_S, grad_payout are device pointers, stream-ordered on
// dev->st (the finish waits for the GPU only with node terms, whose host-side
// chain rule needs the per-node sums)
int vjp_plan_enqueue(VjpPlan *v, int Q, const double *payout, const double *cot, int flags, std::string &err,
                     const DevIO *dev = nullptr);
int vjp_plan_finish(VjpPlan *v, double *grad_S, double *grad_payout, IcmGpuRunStats *stats, std::string &err,
                    const DevIO *dev = nullptr);
// flags: 1 = add the dependence of the quadrature nodes on max S
int vjp_plan_run(VjpPlan *v, int Q, const double *payout, const double *cot, double *grad_S, double *grad_payout,
                 int flags, IcmGpuRunStats *stats, std::string &err);
double node_shift_term(int Q, double Smax, const std::vector<int> &qidx, const std::vector<double> &w,
                       const std::vector<double> &A, const std::vector<double> &Bw);
void vjp_set_smem_limits();

// adjoint steps of one tournament (vjp.cu), for single plans and work lists
size_t vjp_level_layout(const Plan *p, int qc, char *base, VjpBufs *b);
AdjLeafUpArgs adj_leaf_up_args(const Plan *p, const VjpBufs &b);
AdjLeafDownArgs adj_leaf_down_args(const Plan *p, const VjpBufs &b, double *pA, double *pB);
void adj_up_args(const Plan *p, const VjpBufs &b, int l, const double2 *tw, int logTW, AdjUpFusedArgs &F,
                 AdjUpSchoolArgs &S);
void adj_down_args(const Plan *p, const VjpBufs &b, int l, const double2 *tw, int logTW, AdjDownFusedArgs &F,
                   AdjDownSchoolArgs &S);
size_t adj_up_smem(int logN);
size_t adj_down_smem(int logN);
void launch_worklist_adj(WOp op, int key, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st);
// packed one-kernel FFT adjoint steps: slots = (descriptor, pair), cb pairs per CTA
void launch_packed_adj(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                       cudaStream_t st);
int adj_items_per_cta(int logN);
void launch_accum_strided(int n, int nq, const double *src, size_t sq, double *acc, bool first, cudaStream_t st);
// ---- argument blocks of the spectral adjoint steps (vjp_spec.cu), one
// tournament level each (single plans launch (nbx, nq) grids, batches work
// lists of (descriptor, block))
// real sequences of length 2M (node coefficients) -> DFT_{2M} bins 0..M
struct VspRealArgs {
    const double *x;   // row j at x + q x_q + j xst; xlen entries used
    size_t x_q;
    int xst, xlen, nreal, logM;
    int fold;          // add x[2M] onto x[0] (the folded spectrum of a degree-2M row)
    double2 *out;      // M + 1 bins per node
    size_t o_q;
    double *ends;      // (x[0], x[2M]) per node, or null
    size_t e_q;
    const double2 *tw;
    int logTW;
    ZeroPrefix z;      // span: the nodes' degree (wholly-zero nodes: zeros)
    int cb, nbx;       // nodes per CTA, CTAs per chunk node
};

struct VspUpArgs {
    const double2 *A;   // children's gbar spectra, D + 1 bins per node
    size_t A_q;
    const double2 *S;   // children's spec2 (forward build)
    size_t S_q;
    int nreal_c, nreal_p, logD;
    double2 *Aout;      // parents' gbar spectra (2D + 1 bins), or null: coefficients
    size_t Ao_q;
    double *gout;       // parents' gbar coefficients (glen entries, zero to gst)
    size_t go_q;
    int gst, glen;
    double2 *buf;       // multi-pass levels: nreal_p x D complex per chunk node
    const double2 *tw;
    int logTW;
    ZeroPrefix z;       // span: the parents' degree
    int cb, nbx;        // parents per CTA, CTAs per chunk node
};

struct VspDownArgs {
    const double2 *G;   // parents' g spectra, D + 1 bins (G_q = 0: one shared row, the root's)
    size_t G_q;
    const double2 *PF;  // parents' folded Pbar spectra, D + 1 bins, or null (the root: Pbar = 0)
    size_t PF_q;
    const double *Pe;   // parents' Pbar ends (Pbar[0], Pbar[2D])
    size_t Pe_q;
    const double2 *A;   // children's gbar spectra, D + 1 bins
    size_t A_q;
    const double2 *S;   // children's spec2
    size_t S_q;
    const double *E;    // children's ends (P[0], P[D])
    size_t E_q;
    int nreal_c, logD;
    double2 *PFout;     // children's folded Pbar spectra (D/2 + 1 bins) and ends, or null
    size_t PFo_q;
    double *Peout;
    size_t Peo_q;
    double *Pout;       // children's Pbar coefficients (D + 1 entries, zero to pst)
    size_t Po_q;
    int pst;
    double2 *buf;       // multi-pass levels: nreal_c x D/2 complex per chunk node
    const double2 *tw;
    int logTW;
    ZeroPrefix z;       // span: the children's degree (wholly-zero children are skipped)
    int cb, nbx;        // children per CTA, CTAs per chunk node
};


// argument blocks of level l's steps for plan p and its adjoint buffers b:
// the conversion of the children's coefficient gbar to spectra (the band's
// bottom), the upward step, the conversion of the parents' coefficient Pbar
// (the band's top), the downward step; *smem: dynamic shared memory of a CTA
VspRealArgs vsp_gbar_real_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW,
                               size_t *smem);
VspUpArgs vsp_up_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW, size_t *smem);
VspRealArgs vsp_pbar_real_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW,
                               size_t *smem);
VspDownArgs vsp_down_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW, size_t *smem);
// true: the level's steps run in one CTA (work lists hold no multi-pass levels)
bool vsp_one_cta(const Plan *p, int l);
// work lists of the spectral adjoint steps (AdjSpecReal, AdjSpecUp, AdjSpecDown)
void launch_worklist_vsp(WOp op, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st);

// adjoint steps of a spectral level l (vjp_spec.cu): upward (the children's
// gbar to the parents', converting coefficient gbar first where the level
// below is not spectral) and downward (the parents' Pbar to the children's,
// converting coefficient Pbar first where the level above is not spectral)
void adj_spec_up(Plan *p, const VjpBufs &b, int l, int nq, int q0, const double2 *tw, int logTW, long &launches);
void adj_spec_down(Plan *p, const VjpBufs &b, int l, int nq, int q0, const double2 *tw, int logTW, long &launches);
void vjp_spec_set_smem_limits();
void launch_node_reduce_members(int F, const longlong2 *mem, int nq, size_t sq, const double *pA, const double *pB,
                                double *outA, double *outB, int Qs, int q0, cudaStream_t st);

}  // namespace icmg
