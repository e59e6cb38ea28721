// small.cu -- the whole per-node pipeline of a small tournament in one CTA
// (the counterpart of the reference's single-kernel small-n path,
// src/gpu/gpu_kernels.cu:1547-1668, gated in src/gpu/gpu_api.cu:488-534).
//
// One CTA per quadrature node keeps everything in shared memory: the leaf
// factors and block products (one thread per block, in registers), the
// tree's levels as truncated schoolbook products, the propagate pass from
// the payout down to the blocks as middle products with the siblings, and
// the per-player division and weight.  Nothing goes to HBM but the players'
// shares.  For a single solve the last CTA of the launch to finish also sums
// the shares over the chunk's nodes in node order and scatters the equities,
// so a solve is one launch.  Small tournaments are latency-bound on the
// level-by-level path (one launch per level and direction); here the whole
// solve costs about one kernel's latency plus its FP64 work.
//
// Levels are schoolbook at every degree, so plans use this path only where
// that work is small (plan_small_ok); the arithmetic per coefficient is the
// schoolbook kernels' (same terms, same order) and the division is the
// level path's divide_dot.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "leafdiv.cuh"

namespace icmg {

constexpr int kSmallThreads = 256;

template <int B>
__device__ __forceinline__ void small_t(const SmallArgs &A, int q, int q0, int nq) {
    extern __shared__ double sm[];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = A.n, k = A.k, L = A.L;
    double *av = sm + A.offA;
    const double *nd = A.node + 3 * (q0 + q);
    const double logv = nd[0], w = nd[1], iv = nd[2];
    // leaf factors and block products (rows of B+1: the division needs all of them)
    double *P0 = sm + A.lv[0].offP;
    for (int b = tid; b < A.nblocks; b += nt) {
        const int start = b * B, bs = min(B, n - start);
        double P[B + 1];
        block_product<B>(A.S + start, bs, logv, av + start, P);
#pragma unroll
        for (int m = 0; m <= B; ++m) P0[(size_t)b * (B + 1) + m] = P[m];
    }
    __syncthreads();
    // levels 1..L-2 (the root's product is never needed)
    for (int l = 1; l <= L - 2; ++l) {
        const SmallLevel &Pl = A.lv[l], &C = A.lv[l - 1];
        const int cs = (l == 1) ? (B + 1) : C.pst;
        const double *cur = sm + C.offP;
        double *nxt = sm + Pl.offP;
        const int lc = C.plen, lp = Pl.plen;
        for (int e = tid; e < Pl.nreal * lp; e += nt) {
            const int j = e / lp, t = e - j * lp;
            const double *Lc = cur + (size_t)(2 * j) * cs;
            double v;
            if (2 * j + 1 >= C.nreal) {
                v = (t < lc) ? Lc[t] : 0.0;   // lone child copied up
            } else {
                const double *R = Lc + cs;
                const int ilo = max(0, t - (lc - 1)), ihi = min(t, lc - 1);
                double s = 0.0;
                for (int i = ilo; i <= ihi; ++i) s = fma(Lc[i], R[t - i], s);
                v = s;
            }
            nxt[(size_t)j * Pl.pst + t] = v;
        }
        __syncthreads();
    }
    // propagate: the root's g is the payout; children from parents, level by level
    double *gcur = sm + A.offG0, *gnxt = sm + A.offG1;
    for (int l = L - 1; l >= 1; --l) {
        const SmallLevel &C = A.lv[l - 1];
        const bool root = (l == L - 1);
        const double *gpb = root ? A.payout : gcur;
        const int gst_p = root ? 0 : A.lv[l].gst;
        const int gpl = root ? k : A.lv[l].glen;
        const int cs = (l == 1) ? (B + 1) : C.pst;
        const double *Pc = sm + C.offP;
        double *gout = gnxt;
        for (int e = tid; e < C.nreal * C.gst; e += nt) {
            const int c = e / C.gst, m = e - c * C.gst;
            double v = 0.0;
            if (m < C.glen) {
                const double *gp = gpb + (size_t)(c >> 1) * gst_p;
                if ((c ^ 1) >= C.nreal) {
                    v = (m < gpl) ? gp[m] : 0.0;   // lone child: the parent's g
                } else {
                    const double *Ps = Pc + (size_t)(c ^ 1) * cs;
                    const int imax = min(C.plen, gpl - m);
                    double s = 0.0;
                    for (int i = 0; i < imax; ++i) s = fma(Ps[i], gp[m + i], s);
                    v = s;
                }
            }
            gout[(size_t)c * C.gst + m] = v;
        }
        __syncthreads();
        gnxt = gcur;
        gcur = gout;
    }
    // per player: division, dot with its block's g, weight
    const double *g0 = (L == 1) ? A.payout : gcur;
    const int gst0 = (L == 1) ? 0 : A.lv[0].gst;
    for (int i = tid; i < n; i += nt) {
        double val = 0.0;
        const double a = av[i];
        if ((!A.active || A.active[i]) && w != 0.0 && a != 0.0) {
            const int b = i / B, start = b * B, bs = min(B, n - start), pk = min(bs, k);
            const double eq = divide_dot<B>(a, P0 + (size_t)b * (B + 1), bs, pk, g0 + (size_t)b * gst0);
            double pw = w * A.S[i] * a * iv;
            if (!isfinite(pw)) pw = 0.0;
            val = pw * eq;
        }
        A.contrib[(size_t)q * A.aq + i] = val;
    }
    if (!A.counter) return;
    // the last CTA to finish sums the chunk's nodes in order (k_accumulate's
    // arithmetic) and, for the last chunk, scatters to the caller's order
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (tid == 0) is_last = (atomicAdd(A.counter, 1u) == (unsigned)nq - 1) ? 1 : 0;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int i = tid; i < n; i += nt) {
        double s = A.first ? 0.0 : A.acc[i];
        for (int qq = 0; qq < nq; ++qq) s += __ldcg(A.contrib + (size_t)qq * A.aq + i);
        if (A.last)
            A.out[A.perm[i]] = (A.active && !A.active[i]) ? 0.0 : s;
        else
            A.acc[i] = s;
    }
    if (tid == 0) *A.counter = 0u;   // ready for the next launch
}

template <int B>
__global__ void __launch_bounds__(kSmallThreads) k_small(SmallArgs A, int nq) {
    small_t<B>(A, blockIdx.y, A.q0, nq);
}
template <int B>
__global__ void __launch_bounds__(kSmallThreads)
kw_small(const SmallArgs *__restrict__ D, const int2 *__restrict__ tab, int q0, int nq) {
    small_t<B>(D[tab[blockIdx.x].x], blockIdx.y, q0, nq);
}

// shared-memory layout of one node's pipeline (doubles): leaf factors,
// block products, levels 1..L-2, two g buffers
static size_t small_layout(const Plan *p, SmallArgs *A) {
    size_t off = 0;
    const int B = p->B, L = p->L;
    A->offA = (int)off;
    off += (size_t)p->n;
    A->lv[0] = SmallLevel{p->lv[0].nreal, B + 1, p->lv[0].plen, p->lv[0].gst, p->lv[0].glen, (int)off, 0};
    off += (size_t)p->nblocks * (B + 1);
    for (int l = 1; l <= L - 2; ++l) {
        const Level &v = p->lv[l];
        A->lv[l] = SmallLevel{v.nreal, v.pst, v.plen, v.gst, v.glen, (int)off, 0};
        off += (size_t)v.nreal * v.pst;
    }
    if (L >= 2) {   // the root's row sizes for its children's propagate
        const Level &v = p->lv[L - 1];
        A->lv[L - 1] = SmallLevel{v.nreal, v.pst, v.plen, v.gst, v.glen, 0, 0};
    }
    size_t gmax = 1;
    for (int l = 0; l <= L - 2; ++l) gmax = std::max(gmax, (size_t)p->lv[l].nreal * p->lv[l].gst);
    A->offG0 = (int)off;
    off += gmax;
    A->offG1 = (int)off;
    off += gmax;
    return off * sizeof(double);
}

size_t small_smem_bytes(const Plan *p) {
    SmallArgs A{};
    return small_layout(p, &A);
}

// The schoolbook work of one node grows with n and k while the level path's
// cost is mostly launch latency for small trees, so the path is taken below a
// k-dependent size, as in the reference (gpu_exec.cu:26-60).  The limits are
// the measured crossovers on GB300 (device time of one solve, Q = 256, both
// paths): k <= 16 up to n = 1536, k <= 64 up to 768, k <= 128 up to 640,
// k <= 256 up to 512, else up to 352 (n = 500, k = 200: 0.225 against
// 0.249 ms; n = 320, k = 320: 0.193 against 0.213 ms; above the limits the
// level path wins, e.g. n = 900, k = 120: 0.368 against 0.319 ms).
// g_config.small_max_n overrides them (-1 disables the path).
bool plan_small_ok(const Plan *p) {
    if (p->coeff_only || p->vjp || g_config.small_max_n < 0) return false;
    int lim;
    if (g_config.small_max_n > 0) lim = g_config.small_max_n;
    else lim = p->k <= 16 ? kSmallMaxN : p->k <= 64 ? 768 : p->k <= 128 ? 640 : p->k <= 256 ? 512 : 352;
    if (p->n > lim || p->L > kSmallMaxLevels) return false;
    return small_smem_bytes(p) <= kSmallMaxSmem;
}

// per node: leaf recurrences, every level's product terms, the middle
// products of the propagate, the divisions (one FMA = 2 flops)
double small_flops(const Plan *p) {
    const int B = p->B, n = p->n, r = n % B, L = p->L;
    double fl = (double)(n / B) * B * (3.0 * B + 1.0) + (double)r * (3.0 * r + 1.0);
    for (int l = 1; l <= L - 2; ++l) {
        const Level &c = p->lv[l - 1], &v = p->lv[l];
        double tb = 0.0;
        for (int t = 0; t < v.plen; ++t) tb += std::min(t, c.plen - 1) - std::max(0, t - (c.plen - 1)) + 1;
        fl += 2.0 * tb * std::min(v.nreal, c.nreal / 2);
    }
    for (int l = L - 1; l >= 1; --l) {
        const Level &c = p->lv[l - 1];
        const int gpl = (l == L - 1) ? p->k : p->lv[l].glen;
        double tp = 0.0;
        for (int m = 0; m < c.glen; ++m) tp += std::max(0, std::min(c.plen, gpl - m));
        fl += 2.0 * tp * 2 * (c.nreal / 2);
    }
    return fl + (double)n * (5.0 * std::min(B, p->k) + 4.0);
}

SmallArgs small_args(const Plan *p, const double *S, const double *node, const double *payout, double *contrib,
                     size_t aq, const uint8_t *active) {
    SmallArgs A{};
    A.B = p->B;
    A.n = p->n;
    A.k = p->k;
    A.nblocks = p->nblocks;
    A.L = p->L;
    A.S = S;
    A.node = node;
    A.payout = payout;
    A.active = active;
    A.contrib = contrib;
    A.aq = aq;
    A.smem = small_layout(p, &A);
    A.nbx = 1;
    return A;
}

void launch_small(const SmallArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq) {
    SmallArgs a = A;
    a.q0 = q0;
    const dim3 g(1, nq);
    pr->begin("small", fq * nq, st);
    switch (a.B) {
        case 4: k_small<4><<<g, kSmallThreads, a.smem, st>>>(a, nq); break;
        case 8: k_small<8><<<g, kSmallThreads, a.smem, st>>>(a, nq); break;
        case 16: k_small<16><<<g, kSmallThreads, a.smem, st>>>(a, nq); break;
        default: k_small<32><<<g, kSmallThreads, a.smem, st>>>(a, nq); break;
    }
    pr->end(st);
}

void launch_worklist_small(int B, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                           cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    const SmallArgs *D = (const SmallArgs *)desc;
    switch (B) {
        case 4: kw_small<4><<<g, kSmallThreads, smem, st>>>(D, tab, q0, nq); break;
        case 8: kw_small<8><<<g, kSmallThreads, smem, st>>>(D, tab, q0, nq); break;
        case 16: kw_small<16><<<g, kSmallThreads, smem, st>>>(D, tab, q0, nq); break;
        default: kw_small<32><<<g, kSmallThreads, smem, st>>>(D, tab, q0, nq); break;
    }
}

// ---- one-shot small solves without a plan (icm_equity, icm_gpu_equity):
// a per-thread context keeps a stream, a grow-only device buffer and a
// grow-only pinned staging buffer across calls, so a solve is one packed
// upload (stacks, nodes, payout, permutation, subset mask and the CTA
// counter), one launch per 256 nodes and one download; no plan, arena or
// stream is created.  The kernels and their arguments are the plan path's,
// so the equities are identical to it.
namespace {
struct SmallCtx {
    int dev = -1;
    cudaStream_t st = nullptr;
    char *d = nullptr;
    size_t dcap = 0;
    char *h = nullptr;
    size_t hcap = 0;
    void release() {
        if (st) cudaStreamSynchronize(st);
        if (d) cudaFree(d);
        if (h) cudaFreeHost(h);
        if (st) cudaStreamDestroy(st);
        *this = SmallCtx{};
    }
};
thread_local SmallCtx t_small;
size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }
}  // namespace

void small_context_release() { t_small.release(); }

int small_solve(int n, const double *S, int Q, const double *payout, int k, double *equity, const int *targets,
                int n_targets, IcmGpuRunStats *stats, long *launches, std::string &err) {
    Plan p;
    if (plan_geometry(&p, n, S, k, err) != 0) return -1;
    if (!p.small) return 0;
    std::vector<double> logv, w;
    make_nodes(Q, p.Smax, logv, w);
    int nact = 0;
    for (int q = 0; q < Q; ++q) nact += w[q] != 0.0;
    int qc = std::min(std::max(nact, 1), 256);   // node chunks as a plan would take them
    if (g_config.q_chunk > 0) qc = std::min(qc, g_config.q_chunk);
    // layout: the uploaded prefix, then the device-only arrays
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off += up256(b); return o; };
    const size_t o_S = take(8 * (size_t)n), o_node = take(24 * (size_t)std::max(nact, 1)), o_pay = take(8 * (size_t)k);
    const size_t o_perm = take(4 * (size_t)n), o_act = take(targets ? (size_t)n : 0), o_cnt = take(4);
    const size_t up = off;
    const size_t o_con = take(8 * (size_t)qc * n), o_acc = take(8 * (size_t)n), o_out = take(8 * (size_t)n);
    SmallCtx &c = t_small;
    int dev = 0;
    cudaGetDevice(&dev);
    if (c.dev != dev) {
        c.release();
        if (cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess) { err = "stream"; return -1; }
        c.dev = dev;
    }
    if (c.dcap < off) {
        if (c.d) { cudaStreamSynchronize(c.st); cudaFree(c.d); c.d = nullptr; c.dcap = 0; }
        const cudaError_t e = dev_alloc((void **)&c.d, off, c.st, false);
        if (e != cudaSuccess) { err = std::string("device allocation: ") + cudaGetErrorString(e); return -1; }
        c.dcap = off;
    }
    if (c.hcap < up) {
        if (c.h) { cudaStreamSynchronize(c.st); cudaFreeHost(c.h); c.h = nullptr; c.hcap = 0; }
        if (cudaMallocHost((void **)&c.h, up) != cudaSuccess) { err = "pinned staging buffer"; return -1; }
        c.hcap = up;
    }
    char *H = c.h;
    std::memcpy(H + o_S, p.S_sorted.data(), 8 * (size_t)n);
    double *nd = (double *)(H + o_node);
    for (int q = 0, j = 0; q < Q; ++q) {
        if (w[q] == 0.0) continue;   // the reference skips zero-weight nodes
        nd[3 * j] = logv[q];
        nd[3 * j + 1] = w[q];
        nd[3 * j + 2] = std::exp(-logv[q]);
        ++j;
    }
    std::memcpy(H + o_pay, payout, 8 * (size_t)k);
    std::memcpy(H + o_perm, p.perm.data(), 4 * (size_t)n);
    if (targets) {
        plan_inv_perm(&p);
        uint8_t *act = (uint8_t *)(H + o_act);
        std::memset(act, 0, (size_t)n);
        for (int t = 0; t < n_targets; ++t)
            if (targets[t] >= 0 && targets[t] < n) act[p.inv_perm[targets[t]]] = 1;
    }
    *(unsigned *)(H + o_cnt) = 0u;
    char *D = c.d;
    cudaError_t e = cudaMemcpyAsync(D, H, up, cudaMemcpyHostToDevice, c.st);
    if (nact == 0 && e == cudaSuccess) e = cudaMemsetAsync(D + o_out, 0, 8 * (size_t)n, c.st);
    long nl = 0;
    if (nact > 0 && e == cudaSuccess) {
        SmallArgs A = small_args(&p, (const double *)(D + o_S), (const double *)(D + o_node),
                                 (const double *)(D + o_pay), (double *)(D + o_con), (size_t)n,
                                 targets ? (const uint8_t *)(D + o_act) : nullptr);
        A.counter = (unsigned *)(D + o_cnt);
        A.acc = (double *)(D + o_acc);
        A.out = (double *)(D + o_out);
        A.perm = (const int *)(D + o_perm);
        Prof off_prof;
        for (int q0 = 0; q0 < nact; q0 += qc) {
            const int nq = std::min(qc, nact - q0);
            A.first = q0 == 0;
            A.last = q0 + nq >= nact;
            launch_small(A, nq, q0, c.st, &off_prof, 0.0);
            ++nl;
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(equity, D + o_out, 8 * (size_t)n, cudaMemcpyDeviceToHost, c.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.st);
    if (e != cudaSuccess) { err = std::string("small solve: ") + cudaGetErrorString(e); return -1; }
    if (launches) *launches = nl;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->peak_vram_bytes = off;
        stats->engine = 1;
        stats->B = p.B;
    }
    return 1;
}

template <int B>
static void small_limits_b() {
    cudaFuncSetAttribute(k_small<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallMaxSmem);
    cudaFuncSetAttribute(kw_small<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallMaxSmem);
}

void small_set_smem_limits() {
    small_limits_b<4>();
    small_limits_b<8>();
    small_limits_b<16>();
    small_limits_b<32>();
}

}  // namespace icmg
