// batch.h -- forests: many tournaments solved by shared work-list launches
// (batch.cu).  Internal to the library.
#pragma once

#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "vjp.h"

namespace icmg {

// one launch: every descriptor of one step kind and transform size
struct WStep {
    WOp op = WOp::Leaf;
    int key = 0;                      // launch variant: block size, transform size or lane width
    int one = 0;                      // 1: one node (the root's payout spectrum)
    int packed = 0;                   // 1: tab holds item slots (descriptor, item), cb per CTA
    int cb = 1;
    const char *name = "";
    size_t esz = 0;                   // bytes per descriptor
    int nd = 0;                       // descriptors
    std::vector<unsigned char> desc;  // host copies of the argument blocks
    std::vector<int2> tab;            // per CTA: (descriptor, block)
    size_t smem = 0;                  // dynamic shared memory of the launch
    double fq = 0.0;                  // algorithmic FP64 flops per node
    // per descriptor, for the profiler: member, units the kernel prunes on
    // (span players each, nreal of them; span 0 = no pruning), flops per node
    std::vector<int> dmem, dnreal;
    std::vector<long> dspan;
    std::vector<double> dfq, dfq0;   // pruned part (per unit of span) and unpruned part
    const void *d_desc = nullptr;
    const int2 *d_tab = nullptr;
};

struct Forest {
    int T = 0;                        // tournaments in the caller's batch
    std::vector<int> n, k;
    std::vector<long> ioff, ipoff;    // caller's offsets of stacks/equities and payouts
    std::vector<Plan *> tr;           // forest members: geometry, buffers in the arena
    std::vector<int> tid;             // caller's index of each member
    std::vector<long> off, poff;      // member offsets in the forest's player / payout arrays
    long Ntot = 0, Ktot = 0;
    bool compact = true;              // members are the whole batch, in order
    std::vector<int> fallback;        // caller's indices solved by single plans
    std::vector<Plan *> fb_plans;
    int qc = 1, Q = 0;
    cudaStream_t stream = nullptr;
    char *arena = nullptr;
    size_t arena_bytes = 0;
    double *d_S = nullptr, *d_payout = nullptr, *d_acc = nullptr, *d_out = nullptr;
    double *d_a = nullptr, *d_contrib = nullptr, *d_node = nullptr;
    int *d_perm = nullptr;
    const double2 *tw = nullptr;
    int logTW = 0;
    std::vector<WStep> pre, steps;    // once per run; per node chunk
    char *d_desc = nullptr;
    size_t desc_cap = 0;
    bool graphs = true;
    cudaGraphExec_t graph = nullptr;
    long launches = 0, graph_launches = 0;
    std::vector<double> h_pay, h_out;
    std::vector<int> h_z;             // [member][Q] zero prefixes (host copy)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_device_ms = 0.0;
    Prof prof;
    std::vector<Plan::KStat> kstats;
    // adjoint forests: member trees under the single VJP plan's level rules,
    // forward without the divide, then the adjoint passes as work lists;
    // d_acc sums dL/dS
    bool vjp = false;
    bool node_terms = false;          // the mode the steps were built for
    std::vector<VjpBufs> vb;          // per member adjoint buffers
    std::vector<long> roff;           // member offsets in the root gbar rows (kst each)
    long Rtot = 0;
    double *d_cot = nullptr, *d_gradP = nullptr, *d_root = nullptr;
    longlong2 *d_mem = nullptr;       // per member (offset, players)
    double *d_part = nullptr;         // node terms: partials [2][qc][Ntot], per-node sums [2][F][Q]
    size_t part_cap = 0;
    std::vector<VjpPlan *> fb_vjp;
    std::vector<double> h_cot, h_gp, h_nodeA, h_nodeB;
};

// vjp: an adjoint forest (forest_vjp_run), else a forward one (forest_run)
Forest *forest_create(int T, const int *n, const int *k, const double *S, std::string &err, bool vjp = false);
void forest_destroy(Forest *f);
int forest_run(Forest *f, int Q, const double *payout, double *equity, IcmGpuRunStats *stats, std::string &err);
// flags as vjp_plan_run; gradients in the caller's order (sum n, sum k)
int forest_vjp_run(Forest *f, int Q, const double *payout, const double *cot, int flags, double *grad_S,
                   double *grad_payout, IcmGpuRunStats *stats, std::string &err);

}  // namespace icmg
