// vjp.h -- plans for vector-Jacobian products of the equities (vjp.cu).
// Internal to the library.
#pragma once

#include <string>
#include <vector>

#include "engine.h"

namespace icmg {

struct VjpPlan {
    Plan *p = nullptr;                   // coefficient-level plan (forward tree buffers)
    char *arena = nullptr;               // adjoint buffers
    size_t arena_bytes = 0;
    int kst = 0;                         // stride of the root's gbar (k rounded up to even)
    double *d_cot = nullptr;             // cotangent, sorted order
    double *d_gradS = nullptr;           // dL/dS, sorted order (ordered sum over nodes)
    double *d_gradP = nullptr;           // dL/dpayout
    double *d_root = nullptr;            // [qc][kst] gbar of the root
    double *gb[kMaxLevels] = {};         // gbar per level, shaped as g
    double *Pb[kMaxLevels] = {};         // Pbar per level, shaped as P
    double2 *gspec[kMaxLevels] = {};     // children's gbar spectra (one-kernel FFT levels)
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
int vjp_plan_enqueue(VjpPlan *v, int Q, const double *payout, const double *cot, int flags, std::string &err);
int vjp_plan_finish(VjpPlan *v, double *grad_S, double *grad_payout, IcmGpuRunStats *stats, std::string &err);
// flags: 1 = add the dependence of the quadrature nodes on max S
int vjp_plan_run(VjpPlan *v, int Q, const double *payout, const double *cot, double *grad_S, double *grad_payout,
                 int flags, IcmGpuRunStats *stats, std::string &err);
double node_shift_term(int Q, double Smax, const std::vector<int> &qidx, const std::vector<double> &w,
                       const std::vector<double> &A, const std::vector<double> &Bw);
void vjp_set_smem_limits();

}  // namespace icmg
