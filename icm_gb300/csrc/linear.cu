// linear.cu -- the linear engine on the GPU: one warp per (tournament,
// quadrature node), O(n k) per node, for small k.
//
// The reference runs it on the CPU only (src/cpu/icm.c:1981-2076 and the
// node-batched src/cpu/linear_batched_impl.inc).  Per node, over the players
// in sorted order, with f_j(x) = a_j + (1 - a_j) x:
//
//   forward    g_{-1} = payout, g_j = T_{a_j} g_{j-1},
//              (T_a g)[m] = a g[m] + (1 - a) g[m+1]   (g[k] = 0)
//   backward   R = 1; for j = n-1 .. 0: inner_j = <g_{j-1}, R>, R <- R f_j mod x^k
//
// so inner_j = <payout, prod_{l != j} f_l mod x^k>, the tree engine's inner
// product, in 2-3 k FMAs per player and direction.  T_a keeps g a weighted
// average of the payouts and R's coefficients are probabilities, so both
// sweeps are stable in any order.
//
// GB300 layout: lane L of the warp holds coefficients m = L R .. L R + R - 1
// (R = ceil(k/32) rounded to 1, 2, 4 or 8, so k <= 256); the neighbour
// coefficient of T and of the product crosses lanes by one shuffle.  The
// backward sweep needs g_{j-1} in reverse order: the forward sweep stores a
// checkpoint every C = 32 / R players in global memory, and each segment is
// recomputed from its checkpoint into registers (C R doubles per lane) and
// walked backwards.  Players of the zero prefix (a = 0, S logv < -700) are
// skipped exactly: their factor is x, so the forward sweep starts from the
// payout shifted by the prefix length z and the backward sweep stops at z.
// Leaf factors are computed 32 at a time (one per lane) and kept in the
// node's row of a[] for the replays.
#include <algorithm>

#include "engine.h"
#include "kernels.h"
#include "leafdiv.cuh"

namespace icmg {

template <int R>
__device__ __forceinline__ void lin_step_T(double (&g)[R], double a, int lane) {
    const double b = 1.0 - a;
    double nxt = __shfl_down_sync(0xffffffffu, g[0], 1);
    if (lane == 31) nxt = 0.0;
#pragma unroll
    for (int r = 0; r < R - 1; ++r) g[r] = fma(a, g[r], b * g[r + 1]);
    g[R - 1] = fma(a, g[R - 1], b * nxt);
}

template <int R>
__device__ __forceinline__ void lin_step_mul(double (&P)[R], double a, int lane) {
    const double b = 1.0 - a;
    double prv = __shfl_up_sync(0xffffffffu, P[R - 1], 1);
    if (lane == 0) prv = 0.0;
#pragma unroll
    for (int r = R - 1; r >= 1; --r) P[r] = fma(a, P[r], b * P[r - 1]);
    P[0] = fma(a, P[0], b * prv);
}

template <int R>
__device__ __forceinline__ double lin_dot(const double (&g)[R], const double (&P)[R]) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r) s = fma(g[r], P[r], s);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// one warp: tournament A, node q of the chunk (q0 + q in the node table)
template <int R>
__device__ __forceinline__ void linear_t(const LinearArgs &A, int q, int q0) {
    constexpr int C = 32 / R;   // players per checkpoint segment
    const int lane = threadIdx.x & 31;
    const int n = A.n, k = A.k;
    const double *nd = A.node + 3 * (q0 + q);
    const double logv = nd[0], w = nd[1], iv = nd[2];
    double *contrib = A.contrib + (size_t)q * A.aq;
    double *arow = A.a + (size_t)q * A.aq;
    const int z = A.zp ? min(A.zp[q0 + q], n) : 0;
    for (int i = lane; i < z; i += 32) contrib[i] = 0.0;   // a = 0: no share
    if (w == 0.0 || z >= n) {   // zero-weight node (the reference skips it), or every factor 0
        for (int i = z + lane; i < n; i += 32) contrib[i] = 0.0;
        return;
    }
    double *ck = A.ck + (size_t)q * A.ck_q;   // checkpoint s: g after player z + (s+1) C - 1
    // forward sweep from the payout shifted by the zero prefix
    double g[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int m = lane * R + r;
        g[r] = (m + z < k) ? A.payout[m + z] : 0.0;
    }
    for (int j0 = z; j0 < n; j0 += 32) {
        const int i = j0 + lane;
        double al = 0.0;
        if (i < n) {
            al = leaf_factor(A.S[i] * logv);
            arow[i] = al;
        }
        const int cnt = min(32, n - j0);
        for (int t = 0; t < cnt; ++t) {
            const double a = __shfl_sync(0xffffffffu, al, t);
            lin_step_T<R>(g, a, lane);
            const int j = j0 + t;
            if ((j - z + 1) % C == 0 && j + 1 < n) {   // end of a segment that has a successor
                double *c = ck + (size_t)((j - z + 1) / C - 1) * (32 * R) + lane * R;
#pragma unroll
                for (int r = 0; r < R; ++r) c[r] = g[r];
            }
        }
    }
    __syncwarp();
    // backward sweep, segment by segment from the last
    double P[R];
#pragma unroll
    for (int r = 0; r < R; ++r) P[r] = (lane == 0 && r == 0) ? 1.0 : 0.0;
    const int nseg = (n - z + C - 1) / C;
    for (int s = nseg - 1; s >= 0; --s) {
        const int ss = z + s * C, len = min(C, n - ss);
        // g_{ss-1}: the shifted payout or the previous segment's checkpoint
        double seg[C][R];
        if (s == 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int m = lane * R + r;
                seg[0][r] = (m + z < k) ? A.payout[m + z] : 0.0;
            }
        } else {
            const double *c = ck + (size_t)(s - 1) * (32 * R) + lane * R;
#pragma unroll
            for (int r = 0; r < R; ++r) seg[0][r] = c[r];
        }
        // seg[c] = g_{ss+c-1} for c = 0 .. len-1
#pragma unroll
        for (int c = 1; c < C; ++c) {
            if (c < len) {
#pragma unroll
                for (int r = 0; r < R; ++r) seg[c][r] = seg[c - 1][r];
                lin_step_T<R>(seg[c], arow[ss + c - 1], lane);
            }
        }
#pragma unroll
        for (int c = C - 1; c >= 0; --c) {
            if (c < len) {
                const int j = ss + c;
                const double a = arow[j];
                const double eq = lin_dot<R>(seg[c], P);
                if (lane == 0) {
                    double v = 0.0;
                    if (a != 0.0 && (!A.active || A.active[j])) {
                        double pw = w * A.S[j] * a * iv;
                        if (!isfinite(pw)) pw = 0.0;
                        v = pw * eq;
                    }
                    contrib[j] = v;
                }
                lin_step_mul<R>(P, a, lane);
            }
        }
    }
}

template <int R>
__global__ void __launch_bounds__(32) k_linear(LinearArgs A, int q0) { linear_t<R>(A, blockIdx.y, q0); }
template <int R>
__global__ void __launch_bounds__(32)
kw_linear(const LinearArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    linear_t<R>(D[tab[blockIdx.x].x], blockIdx.y, q0);
}

// The linear engine's O(n k) sequential sweeps against the tree's parallel
// levels, measured on GB300 (device time per solve, Q = 256, plans resident):
// the tree is faster at every measured size, e.g. n = 300, k = 2: 0.06 against
// 0.30 ms; n = 1000, k = 8: 0.14 against 0.92 ms; n = 65536, k = 32: 4.2
// against 62.7 ms.  A warp walks its node's players one after another, and
// GB300 issues one warp-wide FP64 instruction per SMSP every 64 cycles, so
// the sweep is bound by its chain length while most SMSPs idle (Q = 256
// warps for 608 SMSPs).  So the automatic choice never takes it; callers ask
// for it with engine = 2.
bool plan_linear_auto(int n, int k) {
    (void)n;
    (void)k;
    return false;
}

int linear_lanes(int k) { return k <= 32 ? 1 : k <= 64 ? 2 : k <= 128 ? 4 : 8; }

// checkpoint doubles per node: one vector of 32 R after every C players
size_t linear_ck_per_node(int n, int k) {
    const int R = linear_lanes(k), C = 32 / R;
    return (size_t)((n + C - 1) / C) * 32 * R;
}

LinearArgs linear_args(const Plan *p, const double *S, const double *node, const double *payout, double *a,
                       double *contrib, size_t aq, const uint8_t *active, double *ck, const int *zp) {
    LinearArgs A{};
    A.R = linear_lanes(p->k);
    A.n = p->n;
    A.k = p->k;
    A.S = S;
    A.node = node;
    A.payout = payout;
    A.a = a;
    A.contrib = contrib;
    A.aq = aq;
    A.active = active;
    A.ck = ck;
    A.ck_q = linear_ck_per_node(p->n, p->k);
    A.zp = zp;
    A.nbx = 1;
    return A;
}

// per node: forward sweep and its replay (2 FMA-equivalents per coefficient
// each), backward dot and product (3 per coefficient), over the R-padded rows
double linear_flops(const Plan *p) { return 2.0 * 7.0 * 32.0 * linear_lanes(p->k) * (double)p->n; }

void launch_linear(const LinearArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq) {
    const dim3 g(1, nq);
    pr->begin("linear", fq * nq, st);
    switch (A.R) {
        case 1: k_linear<1><<<g, 32, 0, st>>>(A, q0); break;
        case 2: k_linear<2><<<g, 32, 0, st>>>(A, q0); break;
        case 4: k_linear<4><<<g, 32, 0, st>>>(A, q0); break;
        default: k_linear<8><<<g, 32, 0, st>>>(A, q0); break;
    }
    pr->end(st);
}

void launch_worklist_linear(int R, const void *desc, const int2 *tab, int nctas, int nq, int q0, cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    const LinearArgs *D = (const LinearArgs *)desc;
    switch (R) {
        case 1: kw_linear<1><<<g, 32, 0, st>>>(D, tab, q0); break;
        case 2: kw_linear<2><<<g, 32, 0, st>>>(D, tab, q0); break;
        case 4: kw_linear<4><<<g, 32, 0, st>>>(D, tab, q0); break;
        default: kw_linear<8><<<g, 32, 0, st>>>(D, tab, q0); break;
    }
}

}  // namespace icmg
