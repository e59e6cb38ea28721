// vjp.cu -- vector-Jacobian products of the equities.
//
// For the loss L = sum_i cot_i equity_i(S, payout) the engine returns
// dL/dS and dL/dpayout by reverse mode through one quadrature node at a time.
// The nodes of the erfc-trapezoid rule depend on max S; by default they are
// held fixed (the derivative of the quadrature of the exact integrand), and
// flag 1 adds their dependence (the exact derivative of the Q-node formula;
// the two differ by the derivative of the quadrature error, which is not
// small where Q does not resolve the integrand).
// Per node, with f_j(x) = a_j + (1 - a_j) x, a_j = exp(S_j logv):
//
//   forward   P_b = prod_{j in b} f_j,  P_parent = P_L P_R mod x^lp,
//             g_root = payout, g_L[m] = sum_i P_R[i] g_parent[m+i] (and R),
//             inner_i = <g_b, Q_i>, Q_i = prod_{j in b, j != i} f_j,
//             contrib_i = pw_i inner_i, pw_i = w S_i a_i / v
//   adjoint   c_i = cot_i pw_i
//             gbar_b = sum_{i in b} c_i Q_i                  (leaf, upward)
//             gbar_parent = P_R gbar_L + P_L gbar_R           (products, upward;
//             gbar_root = dL/dpayout for this node)
//             Pbar_L[i] = sum_m gbar_R[m] g_parent[m+i]       (middle products,
//                       + sum_j Pbar_parent[i+j] P_R[j]        downward; Pbar_root = 0)
//             abar_i = cot_i w S_i inner_i / v
//                    + <g_b, (1 - x) H_i>   H_i = sum_{j != i} c_j prod_{l != i, j} f_l
//                    + <Pbar_b, (1 - x) Q_i>
//             dL/dS_i += cot_i w a_i inner_i / v + abar_i logv a_i
//
// The upward pass is the transpose of the propagate pass and the downward
// pass the transpose of the build pass.  Leaf quantities come from exact
// leave-one-out recurrences over the block (no division).  The forward tree
// of a chunk of nodes is recomputed by the VJP call itself and stays in the
// plan's buffers for the adjoint passes.  Coefficient levels whose FFT fits
// one CTA use one-kernel transforms that reuse the children's spectra cached
// by the forward build, larger ones multi-pass transforms, the others
// schoolbook kernels; spectral levels (untruncated children, as in forward
// plans) keep their adjoint in the frequency domain too (vjp_spec.cu).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"
#include "vjp.h"

namespace icmg {

namespace {
constexpr int kVjpThreads = 256;
constexpr int kVjpThreadsMax = 512;   // CTAs alone on an SM (8192-point items) take twice the warps
constexpr int kVjpMaxN = 8192;

inline unsigned nblkv(long work, int threads) { return (unsigned)((work + threads - 1) / threads); }
double now_ns() {
    return (double)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
}  // namespace

// complex points per CTA of the one-kernel adjoint FFT steps (items = kVjpPts / N)
constexpr int kVjpPts = 2048;
__host__ __device__ __forceinline__ int vjp_cb(int N) { return N >= kVjpPts ? 1 : kVjpPts / N; }
static inline int vjp_cb_h(int N) { return vjp_cb(N); }
static inline int vjp_tpb(size_t smem) { return smem > kOneCtaSmem ? kVjpThreadsMax : kVjpThreads; }
// Every pair of a CTA is described by a view staged in shared memory after
// the transforms, so a CTA may hold pairs of different tournaments (packed
// work lists) and pairs under wholly-zero parents are pruned per pair.
constexpr size_t kAdjViewBytes = 80;
constexpr size_t kAdjItemBytes = kAdjViewBytes + sizeof(int);
static inline size_t vjp_up_smem(int N) {
    return (size_t)vjp_cb_h(N) * ((N + N / 2) * sizeof(double2) + kAdjItemBytes);
}
static inline size_t vjp_down_smem(int N) { return (size_t)vjp_cb_h(N) * (N * sizeof(double2) + kAdjItemBytes); }
// the same for cb pairs per CTA
static inline size_t vjp_up_smem_cb(int N, int cb) { return (size_t)cb * ((N + N / 2) * sizeof(double2) + kAdjItemBytes); }
static inline size_t vjp_down_smem_cb(int N, int cb) { return (size_t)cb * (N * sizeof(double2) + kAdjItemBytes); }

// ------------------------------------------------------------ leaf adjoints
// gbar of every leaf block: sum_i c_i Q_i by the running pair
// (prod, wsum) -> (prod f, wsum f + c prod).  One thread per (block, node).
template <int B>
__device__ __forceinline__ void adj_leaf_up_t(const AdjLeafUpArgs &A, int bx, int q, int q0) {
    const auto n = A.n;
    const auto k = A.k;
    const auto nblocks = A.nblocks;
    const auto S = A.S;
    const auto node = A.node;
    const auto a = A.a;
    const auto aq = A.aq;
    const auto cot = A.cot;
    const auto gb0 = A.gb0;
    const auto gb0_q = A.gb0_q;
    const auto gst0 = A.gst0;

    const int b = bx * blockDim.x + threadIdx.x;
    if (b >= nblocks) return;
    const double *nd = node + 3 * (q0 + q);
    const double w = nd[1], iv = nd[2];
    const int start = b * B, bs = min(B, n - start);
    double P[B + 1], W[B + 1];
#pragma unroll
    for (int m = 0; m <= B; ++m) { P[m] = 0.0; W[m] = 0.0; }
    P[0] = 1.0;
    const double *arow = a + (size_t)q * aq + start;
    for (int j = 0; j < bs; ++j) {
        const double aj = arow[j], bj = 1.0 - aj;
        double pw = w * S[start + j] * aj * iv;
        if (!isfinite(pw)) pw = 0.0;
        const double c = cot[start + j] * pw;
#pragma unroll
        for (int m = B; m >= 1; --m) W[m] = fma(aj, W[m], fma(bj, W[m - 1], c * P[m]));
        W[0] = fma(aj, W[0], c * P[0]);
#pragma unroll
        for (int m = B; m >= 1; --m) P[m] = fma(aj, P[m], bj * P[m - 1]);
        P[0] *= aj;
    }
    const int pk = min(bs, k);
    double *out = gb0 + q * gb0_q + (size_t)b * gst0;
#pragma unroll
    for (int m = 0; m <= B; ++m)
        if (m < gst0) out[m] = (m < pk) ? W[m] : 0.0;
    if (A.blockW) {   // k < B: the leaf-down divisions need W beyond the truncation
        double *wf = A.blockW + ((size_t)q * nblocks + b) * B;
#pragma unroll
        for (int m = 0; m < B; ++m) wf[m] = W[m];
    }
}

// Y = X / (a + (1 - a) x) for X of degree len (X[0..len], Y[0..len-1]):
// the forward recurrence when a > 0.5, the backward one when a > 1e-15,
// else a shift -- the rule of the forward pass's per-player division.
// Constant indices keep X and Y in registers.
template <int B>
__device__ __forceinline__ void divide_factor(double a, const double (&X)[B + 1], int len, double (&Y)[B]) {
    const double bb = 1.0 - a;
    if (a > 0.5) {
        const double ia = 1.0 / a, c = -bb * ia;
        double y = 0.0;
#pragma unroll
        for (int m = 0; m < B; ++m) {
            y = (m == 0) ? X[0] * ia : c * y + X[m] * ia;
            Y[m] = (m < len) ? y : 0.0;
        }
    } else if (a > 1e-15) {
        const double ib = 1.0 / bb, c = -a * ib;
        double y = 0.0;
#pragma unroll
        for (int m = B - 1; m >= 0; --m) {
            if (m == len - 1) y = X[m + 1] * ib;
            else if (m < len - 1) y = c * y + X[m + 1] * ib;
            Y[m] = (m < len) ? y : 0.0;
        }
    } else {
#pragma unroll
        for (int m = 0; m < B; ++m) Y[m] = (m < len) ? X[m + 1] : 0.0;
    }
}

// per player: Q_i = P_b / f_i and H_i = (gbar_b - c_i Q_i) / f_i (gbar_b =
// sum_j c_j Q_j from the upward leaf step; both quotients are exact
// polynomials), then the three terms of abar_i and the node's share of dL/dS_i
template <int B>
__device__ __forceinline__ void adj_leaf_down_t(const AdjLeafDownArgs &A, int bx, int q, int q0) {
    const int i = bx * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (i >= n) return;
    const size_t aq = A.aq;
    const double *nd = A.node + 3 * (q0 + q);
    const double logv = nd[0], w = nd[1], iv = nd[2];
    const int b = i / B, start = b * B, bs = min(B, n - start), pk = min(bs, A.k);
    const double ai = A.a[(size_t)q * aq + i];
    if (ai == 0.0) {   // leaf factor 0 (S logv < -700): no share; g of its block may be pruned
        A.contrib[(size_t)q * aq + i] = 0.0;
        if (A.partA) {
            A.partA[(size_t)q * aq + i] = 0.0;
            A.partB[(size_t)q * aq + i] = 0.0;
        }
        return;
    }
    const double Si = A.S[i], ci = A.cot[i];
    const double pw = w * Si * ai * iv;
    const bool fin = isfinite(pw);
    const double cc = fin ? ci * pw : 0.0;   // c_i as in the upward leaf step
    double X[B + 1], Q[B], H[B];
    const double *Pr = A.blockP + ((size_t)q * A.nblocks + b) * (B + 1);
#pragma unroll
    for (int m = 0; m <= B; ++m) X[m] = (m <= bs) ? Pr[m] : 0.0;
    divide_factor<B>(ai, X, bs, Q);
    const double *Wr = A.W + q * A.Wq + (size_t)b * A.Wst;
#pragma unroll
    for (int m = 0; m <= B; ++m) X[m] = (m < bs) ? fma(-cc, Q[m < B ? m : 0], Wr[m]) : 0.0;
    divide_factor<B>(ai, X, bs - 1, H);
    const double *g = A.g0 + q * A.g0_q + (size_t)b * A.gst0;
    double inner = 0.0, bterm = 0.0;
#pragma unroll
    for (int m = 0; m < B; ++m) {
        if (m < pk) {
            const double gm = g[m];
            inner = fma(gm, Q[m], inner);
            bterm = fma(gm, H[m] - (m ? H[m - 1] : 0.0), bterm);
        }
    }
    double cterm = 0.0;
    if (A.Pb0) {
        const double *pb = A.Pb0 + q * A.Pb0_q + (size_t)b * A.pst0;
#pragma unroll
        for (int m = 0; m <= B; ++m)
            if (m < A.plen0) cterm = fma(pb[m], (m < B ? Q[m < B ? m : 0] : 0.0) - (m ? Q[m - 1] : 0.0), cterm);
    }
    const double abar = (fin ? ci * w * Si * iv * inner : 0.0) + bterm + cterm;
    A.contrib[(size_t)q * aq + i] = (fin ? ci * w * ai * iv * inner : 0.0) + abar * logv * ai;
    if (A.partA) {   // dL/dlogv and w dL/dw shares of this player (a = v^S, 1/v)
        const double li = fin ? ci * pw * inner : 0.0;
        A.partA[(size_t)q * aq + i] = abar * Si * ai - li;
        A.partB[(size_t)q * aq + i] = li;
    }
}

// ------------------------------------------------------- schoolbook passes
// gbar of parents j >= j0: P_R gbar_L + P_L gbar_R, truncated to gpl; a lone
// child passes its gbar up unchanged (its g was the parent's).
__device__ __forceinline__ void adj_up_school_body(const AdjUpSchoolArgs &A, int bx, int q, int q0) {
    const auto Pc = A.Pc;
    const auto Pc_q = A.Pc_q;
    const auto pst_c = A.pst_c;
    const auto lc = A.lc;
    const auto nreal_c = A.nreal_c;
    const auto gbc = A.gbc;
    const auto gbc_q = A.gbc_q;
    const auto gst_c = A.gst_c;
    const auto glen_c = A.glen_c;
    const auto gbp = A.gbp;
    const auto gbp_q = A.gbp_q;
    const auto gst_p = A.gst_p;
    const auto gpl = A.gpl;
    const auto nreal_p = A.nreal_p;
    const auto j0 = A.j0;

    const long idx = (long)bx * blockDim.x + threadIdx.x;
    const ZeroPrefix z{A.zp, q0, A.span};
    const int j = j0 + (int)(idx / gst_p);
    const int t = (int)(idx % gst_p);
    if (j >= nreal_p) return;
    double *out = gbp + q * gbp_q + (size_t)j * gst_p;
    if (t >= gpl || zp_cold(z, q, j)) { out[t] = 0.0; return; }   // wholly-zero node: gbar = 0
    const double *gL = gbc + q * gbc_q + (size_t)(2 * j) * gst_c;
    if (2 * j + 1 >= nreal_c) { out[t] = (t < glen_c) ? gL[t] : 0.0; return; }
    const double *gR = gL + gst_c;
    const double *PL = Pc + q * Pc_q + (size_t)(2 * j) * pst_c;
    const double *PR = PL + pst_c;
    const int ilo = max(0, t - (glen_c - 1)), ihi = min(t, lc - 1);
    double s = 0.0;
    for (int i = ilo; i <= ihi; ++i) {
        s = fma(PR[i], gL[t - i], s);
        s = fma(PL[i], gR[t - i], s);
    }
    out[t] = s;
}

// Pbar of children c >= c0: sum_m gbar_sib[m] g_par[m+i] + sum_j Pbar_par[i+j] P_sib[j];
// a lone child takes the parent's Pbar (the build copied it up).
__device__ __forceinline__ void adj_down_school_body(const AdjDownSchoolArgs &A, int bx, int q, int q0) {
    const auto gp = A.gp;
    const auto gp_q = A.gp_q;
    const auto gst_p = A.gst_p;
    const auto gpl = A.gpl;
    const auto Pbp = A.Pbp;
    const auto Pbp_q = A.Pbp_q;
    const auto pst_p = A.pst_p;
    const auto lp = A.lp;
    const auto Pc = A.Pc;
    const auto Pc_q = A.Pc_q;
    const auto pst_c = A.pst_c;
    const auto lc = A.lc;
    const auto gbc = A.gbc;
    const auto gbc_q = A.gbc_q;
    const auto gst_c = A.gst_c;
    const auto glen_c = A.glen_c;
    const auto Pbc = A.Pbc;
    const auto nreal_c = A.nreal_c;
    const auto c0 = A.c0;

    const long idx = (long)bx * blockDim.x + threadIdx.x;
    const ZeroPrefix z{A.zp, q0, A.span};
    const int c = c0 + (int)(idx / pst_c);
    const int i = (int)(idx % pst_c);
    if (c >= nreal_c || zp_cold(z, q, c)) return;   // wholly zero: its Pbar meets only zero factors
    double *out = Pbc + q * Pc_q + (size_t)c * pst_c;
    if (i >= lc) { out[i] = 0.0; return; }
    const int j = c >> 1, sib = c ^ 1;
    if (sib >= nreal_c) {
        out[i] = (Pbp && i < lp) ? Pbp[q * Pbp_q + (size_t)j * pst_p + i] : 0.0;
        return;
    }
    const double *g = gp + q * gp_q + (size_t)j * gst_p;
    const double *gs = gbc + q * gbc_q + (size_t)sib * gst_c;
    double s = 0.0;
    const int mmax = min(glen_c, gpl - i);
    for (int m = 0; m < mmax; ++m) s = fma(gs[m], g[m + i], s);
    if (Pbp) {
        const double *pb = Pbp + q * Pbp_q + (size_t)j * pst_p;
        const double *Ps = Pc + q * Pc_q + (size_t)sib * pst_c;
        const int jmax = min(lc, lp - i);
        for (int jj = 0; jj < jmax; ++jj) s = fma(pb[i + jj], Ps[jj], s);
    }
    out[i] = s;
}

// ----------------------------------------------------- one-kernel FFT passes
struct AuView {          // one pair of the upward pass
    const double *gL;    // left child's gbar row (the right child's at + gst_c)
    const double2 *sL;   // children's P spectra from the build (the right child's at + h + 1)
    double2 *gsL;        // children's gbar spectra, cached for the downward pass (same layout)
    double *out;         // parent's gbar row
    int gst_c, glen_c, gst_p, gpl, cold;
};
static_assert(sizeof(AuView) <= kAdjViewBytes, "view size");
struct AdView {          // one pair of the downward pass
    const double *g;     // parent's g row (the payout at the root)
    const double *pb;    // parent's Pbar row (null at the root)
    const double *PsL;   // left child's P row (the right child's at + pst_c)
    const double2 *sL;   // children's P spectra (the right child's at + h + 1)
    const double2 *gsL;  // children's gbar spectra from the upward pass
    double *outL;        // left child's Pbar row (the right child's at + pst_c)
    int gpl, lp, lc, pst_c, cold;
};
static_assert(sizeof(AdView) <= kAdjViewBytes, "view size");

__device__ __forceinline__ void au_fill(const AdjUpFusedArgs &A, int q, int q0, int j, int h, AuView &v) {
    const size_t so = (2 * ((size_t)q * A.npairs + j)) * (size_t)(h + 1);
    v.gL = A.gbc + q * A.gbc_q + (size_t)(2 * j) * A.gst_c;
    v.sL = A.spec + so;
    v.gsL = A.gspec + so;
    v.out = A.gbp + q * A.gbp_q + (size_t)j * A.gst_p;
    v.gst_c = A.gst_c;
    v.glen_c = A.glen_c;
    v.gst_p = A.gst_p;
    v.gpl = A.gpl;
    const ZeroPrefix z{A.zp, q0, A.span};
    v.cold = zp_cold(z, q, j) ? 1 : 0;
}

__device__ __forceinline__ void ad_fill(const AdjDownFusedArgs &A, int q, int q0, int j, int h, AdView &v) {
    const size_t so = (2 * ((size_t)q * A.npairs + j)) * (size_t)(h + 1);
    v.g = A.gp + q * A.gp_q + (size_t)j * A.gst_p;
    v.pb = A.Pbp ? A.Pbp + q * A.Pbp_q + (size_t)j * A.pst_p : nullptr;
    v.PsL = A.Pc + q * A.Pc_q + (size_t)(2 * j) * A.pst_c;
    v.sL = A.spec + so;
    v.gsL = A.gspec + so;
    v.outL = A.Pbc + q * A.Pc_q + (size_t)(2 * j) * A.pst_c;
    v.gpl = A.gpl;
    v.lp = A.lp;
    v.lc = A.lc;
    v.pst_c = A.pst_c;
    const ZeroPrefix z{A.zp, q0, A.span};
    v.cold = zp_cold(z, q, j) ? 1 : 0;
}

__device__ __forceinline__ int adj_width(const AuView &v) { return v.gst_p; }
__device__ __forceinline__ int adj_width(const AdView &v) { return v.pst_c; }

// hot pairs first in idx; *w = the widest output row of the CTA's pairs
template <class View>
__device__ __forceinline__ int adj_partition(const View *V, int *idx, int cnt, int *w) {
    __shared__ int nhot_s, w_s;
    if (threadIdx.x == 0) {
        int h = 0, mw = 0;
        for (int it = 0; it < cnt; ++it)
            if (!V[it].cold) idx[h++] = it;
        int c = h;
        for (int it = 0; it < cnt; ++it) {
            if (V[it].cold) idx[c++] = it;
            mw = max(mw, adj_width(V[it]));
        }
        nhot_s = h;
        w_s = mw;
    }
    __syncthreads();
    *w = w_s;
    return nhot_s;
}

// Upward, pairs idx[0, nh): z = gbar_L + i gbar_R -> FFT N -> the children's
// gbar spectra (cached for the downward pass) -> Y = S_R G_L + S_L G_R with
// the children's P spectra S cached by the forward build -> half-size inverse
// -> gbar_parent.  N >= glen_c + lc - 1, so the products do not wrap.  Pairs
// idx[nh, cnt) sit under wholly-zero parents: their gbar is 0.
__device__ void adj_up_core(const AuView *V, const int *idx, int cnt, int nh, int wmax, int cb, int logN,
                            const double2 *__restrict__ tw, int logTW, double2 *sm) {
    const int N = 1 << logN, h = N >> 1;
    double2 *Z = sm;
    double2 *U = sm + (size_t)cb * N;
    for (int e = threadIdx.x; e < nh * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const AuView &v = V[idx[it]];
        Z[e] = (t < v.glen_c) ? make_double2(v.gL[t], v.gL[v.gst_c + t]) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, nh, tw, logTW);
    // by mirror pairs of bins (f, h - f), f <= h/2
    const double2 *tt = tw_tangent(tw, logTW);
    const int hp = (h >> 1) + 1;
    for (int e = threadIdx.x; e < nh * hp; e += blockDim.x) {
        const int it = e / hp, f = e - it * hp;
        const AuView &v = V[idx[it]];
        const double2 *z = Z + (size_t)it * N;
        const int fc = h - f;
        const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
        const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
        const double2 GLf = cscale(cadd(zf, cconj(zn)), 0.5);
        const double2 GRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
        const double2 GLc = cscale(cadd(zc, cconj(zcn)), 0.5);
        const double2 GRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
        const double2 *sL = v.sL, *sR = sL + (h + 1);
        double2 *gL = v.gsL, *gR = gL + (h + 1);
        gL[f] = GLf;
        gR[f] = GRf;
        if (fc != f) { gL[fc] = GLc; gR[fc] = GRc; }   // f = 0: bin h
        const double2 Yf = cadd(cmul(sR[f], GLf), cmul(sL[f], GRf));
        const double2 Yc = cadd(cmul(sR[fc], GLc), cmul(sL[fc], GRc));
        double2 E = cadd(Yf, cconj(Yc)), D = csub(Yf, cconj(Yc));
        if (f == 0) { E.y = 0.0; D.y = 0.0; }
        double2 Uf, Uc;   // O = D e^{+2 pi i f/N}; Uc is U[h - f]
        mirror_inv_input(E, D, tt, (long)f << (logTW - logN), logTW, Uf, Uc);
        U[(size_t)it * h + bitrev(f, logN - 1)] = Uf;
        if (f != 0 && fc != f) U[(size_t)it * h + bitrev(fc, logN - 1)] = Uc;
    }
    __syncthreads();
    smem_fft_dit<+1>(U, logN - 1, nh, tw, logTW);
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < cnt * wmax; e += blockDim.x) {
        const int it = e / wmax, t = e - it * wmax;
        const AuView &v = V[idx[it]];
        if (t >= v.gst_p) continue;
        double val = 0.0;
        if (it < nh && t < v.gpl) {
            const double2 uv = U[(size_t)it * h + (t >> 1)];
            val = ((t & 1) ? uv.y : uv.x) * inv;
        }
        v.out[t] = val;
    }
}

// Downward, pairs idx[0, nh): w = g_parent + i Pbar_parent -> FFT N -> their
// spectra G, R; Z = Y_L + i Y_R with Y_L = G conj(Gbar_R) + R conj(S_R)
// (children's gbar spectra from the upward pass, P spectra from the build),
// in place in natural order, then bit-reversed and inverted.  The only wrap
// is P_sib[lc-1] Pbar_parent[2(lc-1)] when N = 2(lc-1); it is corrected
// from the coefficients.  Children of wholly-zero parents are not needed.
__device__ void adj_down_core(const AdView *V, const int *idx, int nh, int wmax, int logN,
                              const double2 *__restrict__ tw, int logTW, double2 *sm) {
    const int N = 1 << logN, h = N >> 1;
    double2 *Z = sm;
    for (int e = threadIdx.x; e < nh * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const AdView &v = V[idx[it]];
        const double x = (t < v.gpl) ? v.g[t] : 0.0;
        const double y = (v.pb && t < v.lp) ? v.pb[t] : 0.0;
        Z[e] = make_double2(x, y);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, nh, tw, logTW);
    for (int e = threadIdx.x; e < nh * h; e += blockDim.x) {
        const int it = e / h, f = e - it * h;
        const AdView &v = V[idx[it]];
        double2 *z = Z + (size_t)it * N;
        const double2 *sL = v.sL, *sR = sL + (h + 1);
        const double2 *gL = v.gsL, *gR = gL + (h + 1);
        if (f == 0) {   // bins 0 and h: real spectra, each its own mirror
            const double2 z0 = z[0], zh = z[h];
            const double2 G0 = make_double2(z0.x, 0.0), R0 = make_double2(z0.y, 0.0);
            const double2 Gh = make_double2(zh.x, 0.0), Rh = make_double2(zh.y, 0.0);
            const double2 YL0 = cadd(cmulc(G0, gR[0]), cmulc(R0, sR[0]));
            const double2 YR0 = cadd(cmulc(G0, gL[0]), cmulc(R0, sL[0]));
            const double2 YLh = cadd(cmulc(Gh, gR[h]), cmulc(Rh, sR[h]));
            const double2 YRh = cadd(cmulc(Gh, gL[h]), cmulc(Rh, sL[h]));
            z[0] = cadd(YL0, cmul_pi(YR0));
            z[h] = cadd(YLh, cmul_pi(YRh));
        } else {
            const double2 zf = z[f], zn = z[N - f];
            const double2 G = cscale(cadd(zf, cconj(zn)), 0.5);
            const double2 R = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
            const double2 YL = cadd(cmulc(G, gR[f]), cmulc(R, sR[f]));
            const double2 YR = cadd(cmulc(G, gL[f]), cmulc(R, sL[f]));
            z[f] = cadd(YL, cmul_pi(YR));
            z[N - f] = cadd(cconj(YL), cmul_pi(cconj(YR)));
        }
    }
    __syncthreads();
    smem_bitrev_map(Z, logN, nh, [](int, int, double2 v) { return v; });
    smem_fft_dit<+1>(Z, logN, nh, tw, logTW);
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < nh * 2 * wmax; e += blockDim.x) {
        const int it = e / (2 * wmax), r = e - it * 2 * wmax;
        const int side = r / wmax, i = r - side * wmax;
        const AdView &v = V[idx[it]];
        if (i >= v.pst_c) continue;
        double val = 0.0;
        if (i < v.lc) {
            const double2 zv = Z[(size_t)it * N + i];
            val = (side ? zv.y : zv.x) * inv;
            if (v.pb && 2 * (v.lc - 1) == N && i == v.lc - 1) {
                const double *Ps = v.PsL + (size_t)(side ^ 1) * v.pst_c;
                const double top = (N < v.lp) ? v.pb[N] : 0.0;
                val = fma(Ps[v.lc - 1], top - v.pb[0], val);
            }
        }
        v.outL[(size_t)side * v.pst_c + i] = val;
    }
}

// single plans: pairs [bx cb, bx cb + cb) of one level
__device__ __forceinline__ void adj_up_fused_body(const AdjUpFusedArgs &A, int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const int N = 1 << A.logN, h = N >> 1;
    const int cb = A.cb;
    const int j0 = bx * cb;
    const int cnt = min(cb, A.npairs - j0);
    if (cnt <= 0) return;
    AuView *V = reinterpret_cast<AuView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kAdjViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) au_fill(A, q, q0, j0 + it, h, V[it]);
    __syncthreads();
    int wmax;
    const int nh = adj_partition(V, idx, cnt, &wmax);
    adj_up_core(V, idx, cnt, nh, wmax, cb, A.logN, A.tw, A.logTW, sm);
}

__device__ __forceinline__ void adj_down_fused_body(const AdjDownFusedArgs &A, int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const int N = 1 << A.logN;
    const int cb = A.cb;
    const int j0 = bx * cb;
    const int cnt = min(cb, A.npairs - j0);
    if (cnt <= 0) return;
    AdView *V = reinterpret_cast<AdView *>(sm + (size_t)cb * N);
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kAdjViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) ad_fill(A, q, q0, j0 + it, N >> 1, V[it]);
    __syncthreads();
    int wmax;
    const int nh = adj_partition(V, idx, cnt, &wmax);
    adj_down_core(V, idx, nh, wmax, A.logN, A.tw, A.logTW, sm);
}

// packed work lists: slots[s] = (descriptor, pair); one transform size per launch
__device__ __forceinline__ void adj_up_packed(const AdjUpFusedArgs *__restrict__ D, const int2 *__restrict__ slots,
                                              int nslots, int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const AdjUpFusedArgs &A0 = D[slots[0].x];
    const int N = 1 << A0.logN, h = N >> 1;
    const int cb = vjp_cb(N);
    const int s0 = bx * cb;
    const int cnt = min(cb, nslots - s0);
    if (cnt <= 0) return;
    AuView *V = reinterpret_cast<AuView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kAdjViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        au_fill(D[sl.x], q, q0, sl.y, h, V[it]);
    }
    __syncthreads();
    int wmax;
    const int nh = adj_partition(V, idx, cnt, &wmax);
    adj_up_core(V, idx, cnt, nh, wmax, cb, A0.logN, A0.tw, A0.logTW, sm);
}

__device__ __forceinline__ void adj_down_packed(const AdjDownFusedArgs *__restrict__ D, const int2 *__restrict__ slots,
                                                int nslots, int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const AdjDownFusedArgs &A0 = D[slots[0].x];
    const int N = 1 << A0.logN;
    const int cb = vjp_cb(N);
    const int s0 = bx * cb;
    const int cnt = min(cb, nslots - s0);
    if (cnt <= 0) return;
    AdView *V = reinterpret_cast<AdView *>(sm + (size_t)cb * N);
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kAdjViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        ad_fill(D[sl.x], q, q0, sl.y, N >> 1, V[it]);
    }
    __syncthreads();
    int wmax;
    const int nh = adj_partition(V, idx, cnt, &wmax);
    adj_down_core(V, idx, nh, wmax, A0.logN, A0.tw, A0.logTW, sm);
}

// ------------------------------------------ multi-pass FFT adjoint levels
// Levels whose transform exceeds one CTA (N > 8192): the one-kernel steps
// above split into a packing kernel, global batched FFTs (fft_batched:
// four-step, natural order) and pointwise kernels.  Every pair is computed,
// as the forward's multi-pass levels compute every pair (their cached
// spectra are complete).  Grids: (items of the level, nodes of the chunk).
__global__ void k_adj_up_pack(const double *__restrict__ gbc, size_t gbc_q, int gst_c, int glen_c, int npairs, int N,
                              double2 *__restrict__ z) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int j = (int)(idx / N), t = (int)(idx % N);
    if (j >= npairs) return;
    const double *gL = gbc + q * gbc_q + (size_t)(2 * j) * gst_c;
    z[((size_t)q * npairs + j) * N + t] = (t < glen_c) ? make_double2(gL[t], gL[gst_c + t]) : make_double2(0.0, 0.0);
}

// children's gbar spectra (cached for the downward pass), Y = S_R G_L + S_L G_R,
// and the half-size inverse input U[f] = E[f] + i O[f] of the real product
__global__ void k_adj_up_mid(const double2 *__restrict__ Z, const double2 *__restrict__ spec,
                             double2 *__restrict__ gspec, int npairs, int N, double2 *__restrict__ U,
                             const double2 *__restrict__ tw, int logTW, int logN) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = N >> 1;
    const int j = (int)(idx / h), f = (int)(idx % h);
    if (j >= npairs) return;
    const size_t item = (size_t)q * npairs + j;
    const double2 *z = Z + item * N;
    const int fc = h - f;
    const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
    const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
    const double2 GLf = cscale(cadd(zf, cconj(zn)), 0.5);
    const double2 GRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
    const double2 GLc = cscale(cadd(zc, cconj(zcn)), 0.5);
    const double2 GRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
    const size_t so = (2 * item) * (size_t)(h + 1);
    const double2 *sL = spec + so, *sR = sL + (h + 1);
    double2 *gL = gspec + so, *gR = gL + (h + 1);
    gL[f] = GLf;
    gR[f] = GRf;
    if (f == 0) { gL[h] = GLc; gR[h] = GRc; }
    const double2 Yf = cadd(cmul(sR[f], GLf), cmul(sL[f], GRf));
    const double2 Yc = cadd(cmul(sR[fc], GLc), cmul(sL[fc], GRc));
    double2 E = cadd(Yf, cconj(Yc)), D = csub(Yf, cconj(Yc));
    if (f == 0) { E.y = 0.0; D.y = 0.0; }
    double2 Uf, Uc;   // O = D e^{+2 pi i f/N}; Uc unused
    mirror_inv_input(E, D, tw_tangent(tw, logTW), (long)f << (logTW - logN), logTW, Uf, Uc);
    U[item * h + f] = Uf;
}

__global__ void k_adj_up_post(const double2 *__restrict__ U, int npairs, int N, double *__restrict__ gbp,
                              size_t gbp_q, int gst_p, int gpl) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int j = (int)(idx / gst_p), t = (int)(idx % gst_p);
    if (j >= npairs) return;
    double v = 0.0;
    if (t < gpl) {
        const double2 uv = U[((size_t)q * npairs + j) * (N >> 1) + (t >> 1)];
        v = ((t & 1) ? uv.y : uv.x) * (1.0 / N);
    }
    gbp[q * gbp_q + (size_t)j * gst_p + t] = v;
}

__global__ void k_adj_down_pack(const double *__restrict__ gp, size_t gp_q, int gst_p, int gpl,
                                const double *__restrict__ Pbp, size_t Pbp_q, int pst_p, int lp, int npairs, int N,
                                double2 *__restrict__ z) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int j = (int)(idx / N), t = (int)(idx % N);
    if (j >= npairs) return;
    const double x = (t < gpl) ? gp[q * gp_q + (size_t)j * gst_p + t] : 0.0;
    const double y = (Pbp && t < lp) ? Pbp[q * Pbp_q + (size_t)j * pst_p + t] : 0.0;
    z[((size_t)q * npairs + j) * N + t] = make_double2(x, y);
}

// in place: Z = Y_L + i Y_R with Y_L = G conj(Gbar_R) + R conj(S_R) (and L/R swapped)
__global__ void k_adj_down_mid(double2 *__restrict__ Z, const double2 *__restrict__ spec,
                               const double2 *__restrict__ gspec, int npairs, int N) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = N >> 1;
    const int j = (int)(idx / h), f = (int)(idx % h);
    if (j >= npairs) return;
    const size_t item = (size_t)q * npairs + j;
    double2 *z = Z + item * N;
    const size_t so = (2 * item) * (size_t)(h + 1);
    const double2 *sL = spec + so, *sR = sL + (h + 1);
    const double2 *gL = gspec + so, *gR = gL + (h + 1);
    if (f == 0) {   // bins 0 and h: real spectra, each its own mirror
        const double2 z0 = z[0], zh = z[h];
        const double2 G0 = make_double2(z0.x, 0.0), R0 = make_double2(z0.y, 0.0);
        const double2 Gh = make_double2(zh.x, 0.0), Rh = make_double2(zh.y, 0.0);
        const double2 YL0 = cadd(cmulc(G0, gR[0]), cmulc(R0, sR[0]));
        const double2 YR0 = cadd(cmulc(G0, gL[0]), cmulc(R0, sL[0]));
        const double2 YLh = cadd(cmulc(Gh, gR[h]), cmulc(Rh, sR[h]));
        const double2 YRh = cadd(cmulc(Gh, gL[h]), cmulc(Rh, sL[h]));
        z[0] = cadd(YL0, cmul_pi(YR0));
        z[h] = cadd(YLh, cmul_pi(YRh));
    } else {
        const double2 zf = z[f], zn = z[N - f];
        const double2 G = cscale(cadd(zf, cconj(zn)), 0.5);
        const double2 R = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
        const double2 YL = cadd(cmulc(G, gR[f]), cmulc(R, sR[f]));
        const double2 YR = cadd(cmulc(G, gL[f]), cmulc(R, sL[f]));
        z[f] = cadd(YL, cmul_pi(YR));
        z[N - f] = cadd(cconj(YL), cmul_pi(cconj(YR)));
    }
}

__global__ void k_adj_down_post(const double2 *__restrict__ Z, int npairs, int N, const double *__restrict__ Pbp,
                                size_t Pbp_q, int pst_p, int lp, const double *__restrict__ Pc, size_t Pc_q, int pst_c,
                                int lc, double *__restrict__ Pbc) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int c = (int)(idx / pst_c), i = (int)(idx % pst_c);
    if (c >= 2 * npairs) return;
    const int j = c >> 1, side = c & 1;
    double v = 0.0;
    if (i < lc) {
        const double2 zv = Z[((size_t)q * npairs + j) * N + i];
        v = (side ? zv.y : zv.x) * (1.0 / N);
        if (Pbp && 2 * (lc - 1) == N && i == lc - 1) {   // the one wrapped term
            const double *pb = Pbp + q * Pbp_q + (size_t)j * pst_p;
            const double *Ps = Pc + q * Pc_q + (size_t)(c ^ 1) * pst_c;
            const double top = (N < lp) ? pb[N] : 0.0;
            v = fma(Ps[lc - 1], top - pb[0], v);
        }
    }
    Pbc[q * Pc_q + (size_t)c * pst_c + i] = v;
}

// ---- kernels: single plans launch (nbx, nq) grids; work lists map blocks
// to (descriptor, block) through tab
template <int B>
__global__ void k_adj_leaf_up(AdjLeafUpArgs A, int q0) { adj_leaf_up_t<B>(A, blockIdx.x, blockIdx.y, q0); }
template <int B>
__global__ void k_adj_leaf_down(AdjLeafDownArgs A, int q0) { adj_leaf_down_t<B>(A, blockIdx.x, blockIdx.y, q0); }
__global__ void k_adj_up_school(AdjUpSchoolArgs A, int q0) { adj_up_school_body(A, blockIdx.x, blockIdx.y, q0); }
__global__ void k_adj_down_school(AdjDownSchoolArgs A, int q0) { adj_down_school_body(A, blockIdx.x, blockIdx.y, q0); }
__global__ void __launch_bounds__(kVjpThreadsMax) k_adj_up_fused(AdjUpFusedArgs A, int q0) {
    adj_up_fused_body(A, blockIdx.x, blockIdx.y, q0);
}
__global__ void __launch_bounds__(kVjpThreadsMax) k_adj_down_fused(AdjDownFusedArgs A, int q0) {
    adj_down_fused_body(A, blockIdx.x, blockIdx.y, q0);
}
template <int B>
__global__ void kw_adj_leaf_up(const AdjLeafUpArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    adj_leaf_up_t<B>(D[t.x], t.y, blockIdx.y, q0);
}
template <int B>
__global__ void kw_adj_leaf_down(const AdjLeafDownArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    adj_leaf_down_t<B>(D[t.x], t.y, blockIdx.y, q0);
}
__global__ void kw_adj_up_school(const AdjUpSchoolArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    adj_up_school_body(D[t.x], t.y, blockIdx.y, q0);
}
__global__ void kw_adj_down_school(const AdjDownSchoolArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    adj_down_school_body(D[t.x], t.y, blockIdx.y, q0);
}

__global__ void __launch_bounds__(kVjpThreadsMax)
kw_adj_up_packed(const AdjUpFusedArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    adj_up_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}
__global__ void __launch_bounds__(kVjpThreadsMax)
kw_adj_down_packed(const AdjDownFusedArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    adj_down_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}

// ordered sum over nodes with a per-node stride
__global__ void k_accum_strided(int n, int nq, const double *__restrict__ src, size_t sq, double *__restrict__ acc,
                                int first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = first ? 0.0 : acc[i];
    for (int q = 0; q < nq; ++q) s += src[(size_t)q * sq + i];
    acc[i] = s;
}

// per node: sums over players of partA and partB in a fixed order (strided
// partial sums per thread, then a fixed tree), deterministic
__global__ void k_node_reduce(int n, const double *__restrict__ partA, const double *__restrict__ partB,
                              double *__restrict__ outA, double *__restrict__ outB) {
    __shared__ double sa[256], sb[256];
    const int q = blockIdx.x;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) {
        a += partA[(size_t)q * n + i];
        b += partB[(size_t)q * n + i];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] += sa[threadIdx.x + s];
            sb[threadIdx.x] += sb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        outA[q] = sa[0];
        outB[q] = sb[0];
    }
}

// d/dSmax of L through the nodes of the erfc-trapezoid rule
// y_q = y_lo + q h, h = (y_hi - y_lo)/(Q - 1), y_hi = max(6.5, sqrt(2 (ln Smax + 25))),
// logv_q = log Phi(y_q), w_q = h phi(y_q):
//   dL = sum_q A_q dlogv_q + (B_q / w_q) dw_q,  A_q = dL/dlogv_q, B_q = w_q dL/dw_q
//   dlogv_q = phi(y_q)/Phi(y_q) dy_q,  dw_q / w_q = dh/h - y_q dy_q
// (the largest stack is the first player in sorted order; ties go to it)
double node_shift_term(int Q, double Smax, const std::vector<int> &qidx, const std::vector<double> &w,
                       const std::vector<double> &A, const std::vector<double> &Bw) {
    if (g_config.quadrature == 1) return 0.0;   // tanh-sinh nodes do not depend on the stacks
    const double y_lo = -7.7;
    const double r = std::sqrt(2.0) * std::sqrt(std::log(Smax) + 25.0);
    if (!(r > 6.5) || Q < 2) return 0.0;
    const double y_hi = r;
    const double dyhi = 1.0 / (Smax * y_hi);
    const double h = (y_hi - y_lo) / (Q - 1);
    const double dh = dyhi / (Q - 1);
    double s = 0.0;
    for (size_t j = 0; j < qidx.size(); ++j) {
        const int q = qidx[j];
        const double y = y_lo + q * h;
        const double dy = dyhi * (double)q / (Q - 1);
        const double phi = std::exp(-0.5 * y * y) / std::sqrt(2.0 * M_PI);
        const double Phi = 0.5 * std::erfc(-y / std::sqrt(2.0));
        s += A[j] * (phi / Phi) * dy + Bw[j] * (dh / h - y * dy);
    }
    (void)w;
    return s;
}

void vjp_set_smem_limits() {
    cudaFuncSetAttribute(k_adj_up_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vjp_up_smem(kVjpMaxN));
    cudaFuncSetAttribute(k_adj_down_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)vjp_down_smem(kVjpMaxN));
    cudaFuncSetAttribute(kw_adj_up_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vjp_up_smem(kVjpMaxN));
    cudaFuncSetAttribute(kw_adj_down_packed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)vjp_down_smem(kVjpMaxN));
    vjp_spec_set_smem_limits();
}

// per (member, node): k_node_reduce over one member's players of a forest
// (mem[t] = (offset, players); rows of sq players), in the same order
__global__ void k_node_reduce_members(const longlong2 *__restrict__ mem, size_t sq, const double *__restrict__ partA,
                                      const double *__restrict__ partB, double *__restrict__ outA,
                                      double *__restrict__ outB, int Qs, int q0) {
    __shared__ double sa[256], sb[256];
    const int t = blockIdx.x, q = blockIdx.y;
    const long off = (long)mem[t].x, n = (long)mem[t].y;
    const double *pa = partA + (size_t)q * sq + off, *pb = partB + (size_t)q * sq + off;
    double a = 0.0, b = 0.0;
    for (long i = threadIdx.x; i < n; i += 256) {
        a += pa[i];
        b += pb[i];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] += sa[threadIdx.x + s];
            sb[threadIdx.x] += sb[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        outA[(size_t)t * Qs + q0 + q] = sa[0];
        outB[(size_t)t * Qs + q0 + q] = sb[0];
    }
}

void launch_node_reduce_members(int F, const longlong2 *mem, int nq, size_t sq, const double *pA, const double *pB,
                                double *outA, double *outB, int Qs, int q0, cudaStream_t st) {
    if (F <= 0 || nq <= 0) return;
    k_node_reduce_members<<<dim3(F, nq), 256, 0, st>>>(mem, sq, pA, pB, outA, outB, Qs, q0);
}

// ------------------------------------------------------------ plans
static bool level_fused(const Level &v) { return v.fft && v.npairs > 0 && v.fftn <= kVjpMaxN && fused_ok(v.fftn); }
static bool level_big(const Level &v) { return v.fft && v.npairs > 0 && !level_fused(v); }

// per-level adjoint buffers of one tournament for chunks of qc nodes: gbar
// (shaped as g), Pbar (shaped as P) and the children's gbar spectra of
// one-kernel FFT levels.  Returns the bytes; with base, fills b's level views.
size_t vjp_level_layout(const Plan *p, int qc, char *base, VjpBufs *b) {
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    size_t o_gb[kMaxLevels], o_Pb[kMaxLevels], o_gsp[kMaxLevels], o_A[kMaxLevels], o_PF[kMaxLevels],
        o_Pe[kMaxLevels];
    size_t A_q[kMaxLevels], PF_q[kMaxLevels], Pe_q[kMaxLevels];
    for (int l = 0; l < p->L; ++l) {
        const Level &lv = p->lv[l];
        o_gb[l] = lv.g_q ? take(8 * (size_t)qc * lv.g_q) : 0;
        o_Pb[l] = lv.P_q ? take(8 * (size_t)qc * lv.P_q) : 0;
        o_gsp[l] = (l >= 1 && lv.fft && lv.npairs > 0) ? take(16 * (size_t)qc * lv.spec_q) : 0;
        // spectral levels: gbar spectra of nodes under a spectral parent level,
        // folded Pbar spectra and ends of spectral levels below the root
        A_q[l] = (l + 1 < p->L && p->lv[l + 1].kind == 2) ? (size_t)lv.nreal * (lv.deg + 1) : 0;
        PF_q[l] = (lv.kind == 2 && l + 1 < p->L) ? (size_t)lv.nreal * (lv.deg / 2 + 1) : 0;
        Pe_q[l] = PF_q[l] ? (size_t)lv.nreal * 2 : 0;
        o_A[l] = A_q[l] ? take(16 * (size_t)qc * A_q[l]) : 0;
        o_PF[l] = PF_q[l] ? take(16 * (size_t)qc * PF_q[l]) : 0;
        o_Pe[l] = Pe_q[l] ? take(8 * (size_t)qc * Pe_q[l]) : 0;
    }
    const size_t o_bw = (p->k < p->B) ? take(8 * (size_t)qc * p->nblocks * p->B) : 0;
    if (!base) return off;
    b->blockW = (p->k < p->B) ? (double *)(base + o_bw) : nullptr;
    for (int l = 0; l < p->L; ++l) {
        const Level &lv = p->lv[l];
        b->gb[l] = lv.g_q ? (double *)(base + o_gb[l]) : nullptr;
        b->gb_q[l] = lv.g_q;
        b->gb_st[l] = lv.gst;
        b->Pb[l] = lv.P_q ? (double *)(base + o_Pb[l]) : nullptr;
        b->gspec[l] = o_gsp[l] ? (double2 *)(base + o_gsp[l]) : nullptr;
        b->Gb2[l] = A_q[l] ? (double2 *)(base + o_A[l]) : nullptr;
        b->Gb2_q[l] = A_q[l];
        b->PF[l] = PF_q[l] ? (double2 *)(base + o_PF[l]) : nullptr;
        b->PF_q[l] = PF_q[l];
        b->Pe[l] = Pe_q[l] ? (double *)(base + o_Pe[l]) : nullptr;
        b->Pe_q[l] = Pe_q[l];
    }
    return off;
}

VjpPlan *vjp_plan_create(int n, const double *S, int k, std::string &err, size_t budget) {
    // the adjoint buffers roughly double the tree's per-node memory; spectral
    // levels as configured (vjp_spectral_min_degree < 0: all on coefficients)
    Plan *p = plan_create(n, S, k, nullptr, err, /*coeff_only=*/g_config.vjp_spectral_min_degree < 0,
                          /*q_bytes_scale=*/2.2, budget, /*vjp=*/true);
    if (!p) return nullptr;
    VjpPlan *v = new VjpPlan();
    v->p = p;
    const int qc = p->qc, L = p->L;
    v->kst = ((k + 1) & ~1);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_cot = take(8 * (size_t)n), o_gs = take(8 * (size_t)n), o_gp = take(8 * (size_t)k);
    const size_t o_root = take(8 * (size_t)qc * v->kst);
    const size_t o_lv = take(vjp_level_layout(p, qc, nullptr, nullptr));
    cudaError_t e = dev_alloc((void **)&v->arena, off, p->stream, true);
    if (e != cudaSuccess) {
        err = "VJP buffers (" + std::to_string(off) + " bytes): " + cudaGetErrorString(e);
        plan_destroy(p);
        delete v;
        return nullptr;
    }
    v->arena_bytes = off;
    char *A = v->arena;
    v->d_cot = (double *)(A + o_cot);
    v->d_gradS = (double *)(A + o_gs);
    v->d_gradP = (double *)(A + o_gp);
    v->d_root = (double *)(A + o_root);
    VjpBufs &b = v->bufs;
    b = VjpBufs{};
    vjp_level_layout(p, qc, A + o_lv, &b);
    b.root = v->d_root;
    b.root_q = (size_t)v->kst;
    b.kst = v->kst;
    b.cot = v->d_cot;
    b.a = p->d_a;
    b.aq = (size_t)n;
    b.contrib = p->d_contrib;
    // the root's gbar summed over nodes: the level-0 buffer when the tree is one block
    b.root_acc = (L == 1) ? b.gb[0] : v->d_root;
    b.root_acc_q = (L == 1) ? p->lv[0].g_q : (size_t)v->kst;
    v->pbufs[0] = b;
    for (int i = 1; i < p->nparts; ++i) {   // the pieces' views, checked against the arena
        const size_t h = (size_t)p->part_off[i];
        const size_t m = (size_t)((i + 1 < p->nparts ? p->part_off[i + 1] : qc) - p->part_off[i]);
        VjpBufs &c = v->pbufs[i];
        c = b;
        for (int l = 0; l < L; ++l) {
            if (c.gb[l]) c.gb[l] += h * b.gb_q[l];
            if (c.Pb[l]) c.Pb[l] += h * p->lv[l].P_q;
            if (c.gspec[l]) c.gspec[l] += h * p->lv[l].spec_q;
            if (c.Gb2[l]) c.Gb2[l] += h * b.Gb2_q[l];
            if (c.PF[l]) c.PF[l] += h * b.PF_q[l];
            if (c.Pe[l]) c.Pe[l] += h * b.Pe_q[l];
        }
        if (c.blockW) c.blockW += h * p->nblocks * p->B;
        c.root += h * b.root_q;
        c.a += h * b.aq;
        c.contrib += h * (size_t)n;
        c.root_acc += h * b.root_acc_q;
        const char *lo = v->arena, *hi = v->arena + off;
        auto inside = [&](const void *q, size_t bytes) {
            return !q || ((const char *)q >= lo && (const char *)q + bytes <= hi);
        };
        bool ok = inside(c.root, 8 * m * b.root_q) &&
                  inside(c.blockW, 8 * m * p->nblocks * p->B) && c.a == p->part[i].a &&
                  c.contrib == p->part[i].contrib && (L == 1 || c.root_acc == c.root);
        for (int l = 0; l < L; ++l)
            ok = ok && inside(c.gb[l], 8 * m * b.gb_q[l]) && inside(c.Pb[l], 8 * m * p->lv[l].P_q) &&
                 inside(c.gspec[l], 16 * m * p->lv[l].spec_q) && inside(c.Gb2[l], 16 * m * b.Gb2_q[l]) &&
                 inside(c.PF[l], 16 * m * b.PF_q[l]) && inside(c.Pe[l], 8 * m * b.Pe_q[l]);
        if (!ok) {
            err = "internal: a VJP chunk view leaves the VJP arena";
            vjp_plan_destroy(v);
            return nullptr;
        }
    }
    return v;
}

void vjp_plan_destroy(VjpPlan *v) {
    if (!v) return;
    if (v->arena) {
        cudaFreeAsync(v->arena, v->p->stream);
        cudaStreamSynchronize(v->p->stream);
    }
    if (v->d_partA) cudaFreeAsync(v->d_partA, v->p->stream);
    plan_destroy(v->p);
    delete v;
}

// ---- argument builders (one member level each; nbx = 0: nothing to launch)
AdjLeafUpArgs adj_leaf_up_args(const Plan *p, const VjpBufs &b) {
    AdjLeafUpArgs A{};
    A.B = p->B;
    A.n = p->n;
    A.k = p->k;
    A.nblocks = p->nblocks;
    A.S = p->d_S;
    A.node = p->d_node;
    A.a = b.a;
    A.aq = b.aq;
    A.cot = b.cot;
    A.gb0 = b.gb[0];
    A.gb0_q = b.gb_q[0];
    A.gst0 = b.gb_st[0];
    A.blockW = b.blockW;
    A.nbx = (int)nblkv(p->nblocks, 128);
    return A;
}

AdjLeafDownArgs adj_leaf_down_args(const Plan *p, const VjpBufs &b, double *pA, double *pB) {
    const int L = p->L;
    const Level *lv = p->lv;
    AdjLeafDownArgs A{};
    A.B = p->B;
    A.n = p->n;
    A.k = p->k;
    A.S = p->d_S;
    A.node = p->d_node;
    A.a = b.a;
    A.aq = b.aq;
    A.cot = b.cot;
    A.g0 = (L == 1) ? p->d_payout : lv[0].g;
    A.g0_q = (L == 1) ? 0 : lv[0].g_q;
    A.gst0 = (L == 1) ? 0 : lv[0].gst;
    A.Pb0 = (L == 1) ? nullptr : b.Pb[0];
    A.Pb0_q = lv[0].P_q;
    A.pst0 = lv[0].pst;
    A.plen0 = lv[0].plen;
    A.contrib = b.contrib;
    A.partA = pA;
    A.partB = pB;
    A.blockP = p->d_blockP;
    A.nblocks = p->nblocks;
    if (b.blockW) {   // gbar of the leaf blocks in full
        A.W = b.blockW;
        A.Wq = (size_t)p->nblocks * p->B;
        A.Wst = p->B;
    } else {          // k >= B: the level-0 gbar rows hold every coefficient
        A.W = b.gb[0];
        A.Wq = b.gb_q[0];
        A.Wst = b.gb_st[0];
    }
    A.nbx = (int)nblkv(p->n, 128);
    return A;
}

// upward step of level l (1 <= l <= L-1): the one-kernel FFT pairs and the
// schoolbook rest (all parents, or the lone one after the pairs)
void adj_up_args(const Plan *p, const VjpBufs &b, int l, const double2 *tw, int logTW, AdjUpFusedArgs &F,
                 AdjUpSchoolArgs &Sa) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    double *out = root ? b.root : b.gb[l];
    const size_t out_q = root ? b.root_q : b.gb_q[l];
    const int gst_p = root ? b.kst : b.gb_st[l];
    const int gpl = root ? p->k : pl.glen;
    const int *zp = p->zskip ? p->d_z : nullptr;
    F = AdjUpFusedArgs{};
    Sa = AdjUpSchoolArgs{};
    int j0 = 0;
    if (level_fused(pl)) {
        const int N = pl.fftn, logN = plan_ilog2(N), cb = vjp_cb_h(N);
        F = AdjUpFusedArgs{b.gb[l - 1], b.gb_q[l - 1], b.gb_st[l - 1], c.glen, pl.npairs, logN, pl.spec, b.gspec[l],
                           out, out_q, gst_p, gpl, tw, logTW, zp, pl.deg, (pl.npairs + cb - 1) / cb, cb};
        j0 = pl.npairs;
    } else if (level_big(pl)) {
        j0 = pl.npairs;   // the pairs go through the multi-pass steps (adjoint_chunk)
    }
    const long work = (long)(pl.nreal - j0) * gst_p;
    if (work > 0)
        Sa = AdjUpSchoolArgs{c.P, c.P_q, c.pst, c.plen, c.nreal, b.gb[l - 1], b.gb_q[l - 1], b.gb_st[l - 1], c.glen,
                             out, out_q, gst_p, gpl, pl.nreal, j0, zp, pl.deg, (int)nblkv(work, 256)};
}

// downward step of level l: Pbar of level l-1
void adj_down_args(const Plan *p, const VjpBufs &b, int l, const double2 *tw, int logTW, AdjDownFusedArgs &F,
                   AdjDownSchoolArgs &Sa) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    const double *gp = root ? p->d_payout : pl.g;
    const size_t gp_q = root ? 0 : pl.g_q;
    const int gst_p = root ? 0 : pl.gst;
    const int gpl = root ? p->k : pl.glen;
    const double *Pbp = root ? nullptr : b.Pb[l];
    const int *zp = p->zskip ? p->d_z : nullptr;
    F = AdjDownFusedArgs{};
    Sa = AdjDownSchoolArgs{};
    int c0 = 0;
    if (level_fused(pl)) {
        const int N = pl.fftn, logN = plan_ilog2(N), cb = vjp_cb_h(N);
        F = AdjDownFusedArgs{gp, gp_q, gst_p, gpl, Pbp, pl.P_q, pl.pst, pl.plen, c.P, c.P_q, c.pst, c.plen,
                             pl.npairs, logN, pl.spec, b.gspec[l], b.Pb[l - 1], tw, logTW, zp, pl.deg,
                             (pl.npairs + cb - 1) / cb, cb};
        c0 = 2 * pl.npairs;
    } else if (level_big(pl)) {
        c0 = 2 * pl.npairs;
    }
    const long work = (long)(c.nreal - c0) * c.pst;
    if (work > 0)
        Sa = AdjDownSchoolArgs{gp, gp_q, gst_p, gpl, Pbp, pl.P_q, pl.pst, pl.plen, c.P, c.P_q, c.pst, c.plen,
                               b.gb[l - 1], b.gb_q[l - 1], b.gb_st[l - 1], c.glen, b.Pb[l - 1], c.nreal, c0, zp,
                               c.deg, (int)nblkv(work, 256)};
}

size_t adj_up_smem(int logN) { return vjp_up_smem(1 << logN); }
size_t adj_down_smem(int logN) { return vjp_down_smem(1 << logN); }

// ---- launches: single plans
static void launch_leaf_up(const AdjLeafUpArgs &A, int nq, int q0, cudaStream_t st) {
    const dim3 g(A.nbx, nq);
    switch (A.B) {
        case 4: k_adj_leaf_up<4><<<g, 128, 0, st>>>(A, q0); break;
        case 8: k_adj_leaf_up<8><<<g, 128, 0, st>>>(A, q0); break;
        case 16: k_adj_leaf_up<16><<<g, 128, 0, st>>>(A, q0); break;
        default: k_adj_leaf_up<32><<<g, 128, 0, st>>>(A, q0); break;
    }
}
static void launch_leaf_down(const AdjLeafDownArgs &A, int nq, int q0, cudaStream_t st) {
    const dim3 g(A.nbx, nq);
    switch (A.B) {
        case 4: k_adj_leaf_down<4><<<g, 128, 0, st>>>(A, q0); break;
        case 8: k_adj_leaf_down<8><<<g, 128, 0, st>>>(A, q0); break;
        case 16: k_adj_leaf_down<16><<<g, 128, 0, st>>>(A, q0); break;
        default: k_adj_leaf_down<32><<<g, 128, 0, st>>>(A, q0); break;
    }
}

// ---- launches: work lists (batch.cu builds the descriptors and tables); the
// one-kernel FFT steps are packed (launch_packed_adj)
void launch_worklist_adj(WOp op, int key, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    switch (op) {
        case WOp::AdjLeafUp: {
            const AdjLeafUpArgs *D = (const AdjLeafUpArgs *)desc;
            switch (key) {
                case 4: kw_adj_leaf_up<4><<<g, 128, 0, st>>>(D, tab, q0); break;
                case 8: kw_adj_leaf_up<8><<<g, 128, 0, st>>>(D, tab, q0); break;
                case 16: kw_adj_leaf_up<16><<<g, 128, 0, st>>>(D, tab, q0); break;
                default: kw_adj_leaf_up<32><<<g, 128, 0, st>>>(D, tab, q0); break;
            }
            break;
        }
        case WOp::AdjLeafDown: {
            const AdjLeafDownArgs *D = (const AdjLeafDownArgs *)desc;
            switch (key) {
                case 4: kw_adj_leaf_down<4><<<g, 128, 0, st>>>(D, tab, q0); break;
                case 8: kw_adj_leaf_down<8><<<g, 128, 0, st>>>(D, tab, q0); break;
                case 16: kw_adj_leaf_down<16><<<g, 128, 0, st>>>(D, tab, q0); break;
                default: kw_adj_leaf_down<32><<<g, 128, 0, st>>>(D, tab, q0); break;
            }
            break;
        }
        case WOp::AdjUpSchool: kw_adj_up_school<<<g, 256, 0, st>>>((const AdjUpSchoolArgs *)desc, tab, q0); break;
        case WOp::AdjDownSchool:
            kw_adj_down_school<<<g, 256, 0, st>>>((const AdjDownSchoolArgs *)desc, tab, q0);
            break;
        default: break;
    }
}

void launch_packed_adj(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                       cudaStream_t st) {
    if (nslots <= 0 || nq <= 0) return;
    const dim3 g((nslots + cb - 1) / cb, nq);
    if (op == WOp::AdjUpFused)
        kw_adj_up_packed<<<g, vjp_tpb(smem), smem, st>>>((const AdjUpFusedArgs *)desc, slots, nslots, q0);
    else
        kw_adj_down_packed<<<g, vjp_tpb(smem), smem, st>>>((const AdjDownFusedArgs *)desc, slots, nslots, q0);
}

int adj_items_per_cta(int logN) { return vjp_cb_h(1 << logN); }

void launch_accum_strided(int n, int nq, const double *src, size_t sq, double *acc, bool first, cudaStream_t st) {
    k_accum_strided<<<nblkv(n, 256), 256, 0, st>>>(n, nq, src, sq, acc, first ? 1 : 0);
}

// multi-pass upward / downward steps of level l (its pairs; lone parents
// stay with the schoolbook kernels), through the plan's FFT work buffers
static void adj_up_big(Plan *p, const VjpBufs &b, int l, int nq, const double2 *tw, int logTW, long &launches) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    double *out = root ? b.root : b.gb[l];
    const size_t out_q = root ? b.root_q : b.gb_q[l];
    const int gst_p = root ? b.kst : b.gb_st[l];
    const int gpl = root ? p->k : pl.glen;
    const int N = pl.fftn, logN = plan_ilog2(N), np = pl.npairs;
    cudaStream_t st = p->stream;
    k_adj_up_pack<<<dim3(nblkv((long)np * N, 256), nq), 256, 0, st>>>(b.gb[l - 1], b.gb_q[l - 1], b.gb_st[l - 1],
                                                                      c.glen, np, N, p->d_fa);
    fft_batched(p->d_fa, p->d_fc, (long)nq * np, logN, -1, tw, logTW, st, &launches, &p->prof);
    k_adj_up_mid<<<dim3(nblkv((long)np * (N / 2), 256), nq), 256, 0, st>>>(p->d_fa, pl.spec, b.gspec[l], np, N,
                                                                          p->d_fb, tw, logTW, logN);
    fft_batched(p->d_fb, p->d_fc, (long)nq * np, logN - 1, +1, tw, logTW, st, &launches, &p->prof);
    k_adj_up_post<<<dim3(nblkv((long)np * gst_p, 256), nq), 256, 0, st>>>(p->d_fb, np, N, out, out_q, gst_p, gpl);
    launches += 3;
}

static void adj_down_big(Plan *p, const VjpBufs &b, int l, int nq, const double2 *tw, int logTW, long &launches) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    const double *gp = root ? p->d_payout : pl.g;
    const size_t gp_q = root ? 0 : pl.g_q;
    const int gst_p = root ? 0 : pl.gst;
    const int gpl = root ? p->k : pl.glen;
    const double *Pbp = root ? nullptr : b.Pb[l];
    const int N = pl.fftn, logN = plan_ilog2(N), np = pl.npairs;
    cudaStream_t st = p->stream;
    k_adj_down_pack<<<dim3(nblkv((long)np * N, 256), nq), 256, 0, st>>>(gp, gp_q, gst_p, gpl, Pbp, pl.P_q, pl.pst,
                                                                        pl.plen, np, N, p->d_fa);
    fft_batched(p->d_fa, p->d_fc, (long)nq * np, logN, -1, tw, logTW, st, &launches, &p->prof);
    k_adj_down_mid<<<dim3(nblkv((long)np * (N / 2), 256), nq), 256, 0, st>>>(p->d_fa, pl.spec, b.gspec[l], np, N);
    fft_batched(p->d_fa, p->d_fc, (long)nq * np, logN, +1, tw, logTW, st, &launches, &p->prof);
    k_adj_down_post<<<dim3(nblkv((long)2 * np * c.pst, 256), nq), 256, 0, st>>>(
        p->d_fa, np, N, Pbp, pl.P_q, pl.pst, pl.plen, c.P, c.P_q, c.pst, c.plen, b.Pb[l - 1]);
    launches += 3;
}

// adjoint passes of one chunk (the forward tree of the chunk is in place)
// (piece i: the chunk piece's node slots, on its stream; the ordered sums wait
// for acc_wait and record acc_done when given)
static void adjoint_chunk(VjpPlan *v, int q0, int nq, const double2 *tw, int logTW, bool first, bool node_terms,
                          int piece = 0, cudaEvent_t acc_wait = nullptr, cudaEvent_t acc_done = nullptr) {
    Plan *p = v->p;
    PieceScope scope(p, piece ? &p->part[piece] : nullptr);
    cudaStream_t st = p->stream;
    const int L = p->L, n = p->n, k = p->k;
    long &launches = p->launches;
    const VjpBufs b = v->pbufs[piece];
    launch_leaf_up(adj_leaf_up_args(p, b), nq, q0, st);   // for L = 1 the single block is the root
    ++launches;
    for (int l = 1; l <= L - 1; ++l) {   // upward: the root's gbar is this chunk's dL/dpayout
        if (p->lv[l].kind == 2) {
            adj_spec_up(p, b, l, nq, q0, tw, logTW, launches);
            continue;
        }
        AdjUpFusedArgs F;
        AdjUpSchoolArgs Sa;
        adj_up_args(p, b, l, tw, logTW, F, Sa);
        if (F.nbx > 0) {
            F.cb = short_grid_cb(F.cb, F.npairs, nq);
            F.nbx = (F.npairs + F.cb - 1) / F.cb;
            const size_t smu = vjp_up_smem_cb(1 << F.logN, F.cb);
            k_adj_up_fused<<<dim3(F.nbx, nq), vjp_tpb(smu), smu, st>>>(F, q0);
            ++launches;
        } else if (level_big(p->lv[l])) {
            adj_up_big(p, b, l, nq, tw, logTW, launches);
        }
        if (Sa.nbx > 0) {
            k_adj_up_school<<<dim3(Sa.nbx, nq), 256, 0, st>>>(Sa, q0);
            ++launches;
        }
    }
    for (int l = L - 1; l >= 1; --l) {   // downward: Pbar of every level below the root
        if (p->lv[l].kind == 2) {
            adj_spec_down(p, b, l, nq, q0, tw, logTW, launches);
            continue;
        }
        AdjDownFusedArgs F;
        AdjDownSchoolArgs Sa;
        adj_down_args(p, b, l, tw, logTW, F, Sa);
        if (F.nbx > 0) {
            F.cb = short_grid_cb(F.cb, F.npairs, nq);
            F.nbx = (F.npairs + F.cb - 1) / F.cb;
            const size_t smd = vjp_down_smem_cb(1 << F.logN, F.cb);
            k_adj_down_fused<<<dim3(F.nbx, nq), vjp_tpb(smd), smd, st>>>(F, q0);
            ++launches;
        } else if (level_big(p->lv[l])) {
            adj_down_big(p, b, l, nq, tw, logTW, launches);
        }
        if (Sa.nbx > 0) {
            k_adj_down_school<<<dim3(Sa.nbx, nq), 256, 0, st>>>(Sa, q0);
            ++launches;
        }
    }
    // per player: the node's share of dL/dS, then ordered sums over nodes
    const size_t poff = (size_t)p->part_off[piece] * n;
    double *pA = node_terms ? v->d_partA + poff : nullptr, *pB = node_terms ? v->d_partB + poff : nullptr;
    launch_leaf_down(adj_leaf_down_args(p, b, pA, pB), nq, q0, st);
    if (acc_wait) cudaStreamWaitEvent(st, acc_wait, 0);
    launch_accum_strided(n, nq, b.contrib, (size_t)n, v->d_gradS, first, st);
    launch_accum_strided(k, nq, b.root_acc, b.root_acc_q, v->d_gradP, first, st);
    launches += 3;
    if (node_terms) {
        k_node_reduce<<<nq, 256, 0, st>>>(n, pA, pB, v->d_nodeA + q0, v->d_nodeB + q0);
        ++launches;
    }
    if (acc_done) cudaEventRecord(acc_done, st);   // after the piece's last launch
}

// cotangent into sorted order on the device: out[i] = cot[perm[i]]
__global__ void k_gather_perm(int n, const double *__restrict__ cot, const int *__restrict__ perm,
                              double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cot[perm[i]];
}
// one entry of a device vector plus a host-computed value
__global__ void k_add_one(double *x, int i, double v) { x[i] += v; }

int vjp_plan_enqueue(VjpPlan *v, int Q, const double *payout, const double *cot, int flags, std::string &err,
                     const DevIO *dev) {
    if (!v || Q < 1 || !payout || !cot) { err = "invalid arguments"; return -1; }
    Plan *p = v->p;
    const double t0 = now_ns();
    p->launches = 0;
    const int n = p->n, k = p->k;
    const bool node_terms = (flags & 1) != 0;
    std::vector<double> logv, w;
    make_nodes(Q, p->Smax, logv, w);
    std::vector<double> node;
    std::vector<int> qidx;   // rule index of every active node
    node.reserve(3 * (size_t)Q);
    for (int q = 0; q < Q; ++q) {
        if (w[q] == 0.0) continue;
        node.push_back(logv[q]);
        node.push_back(w[q]);
        node.push_back(std::exp(-logv[q]));
        qidx.push_back(q);
    }
    const int nact = (int)(node.size() / 3);
    cudaError_t e = cudaSuccess;
    if (node_terms && (!v->d_partA || v->node_cap < nact)) {   // per-player partials and per-node sums
        if (v->d_partA) cudaFreeAsync(v->d_partA, p->stream);
        v->d_partA = nullptr;
        const size_t cap = std::max(nact, 1);
        e = dev_alloc((void **)&v->d_partA, sizeof(double) * (2 * (size_t)p->qc * n + 2 * cap), p->stream, true);
        if (e != cudaSuccess) { err = std::string("node-term buffers: ") + cudaGetErrorString(e); return -1; }
        v->d_partB = v->d_partA + (size_t)p->qc * n;
        v->d_nodeA = v->d_partB + (size_t)p->qc * n;
        v->d_nodeB = v->d_nodeA + cap;
        v->node_cap = (int)cap;
    }
    if (nact > p->qmax) {
        // stream-ordered from the pool: no device-wide synchronisation
        if (p->d_node) cudaFreeAsync(p->d_node, p->stream);
        p->d_node = nullptr;
        p->d_z = nullptr;
        const size_t nb = sizeof(double) * 3 * (size_t)std::max(nact, 1);
        e = dev_alloc((void **)&p->d_node, nb + sizeof(int) * (size_t)std::max(nact, 1), p->stream, true);
        if (e != cudaSuccess) { err = std::string("node buffer: ") + cudaGetErrorString(e); return -1; }
        p->d_z = (int *)((char *)p->d_node + nb);
        p->qmax = nact;
    }
    p->h_z.resize(nact);
    for (int j = 0; j < nact; ++j) p->h_z[j] = zero_prefix(p->S_sorted.data(), n, node[3 * j]);
    if (nact) e = cudaMemcpyAsync(p->d_z, p->h_z.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, p->stream);
    if (nact && e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_node, node.data(), sizeof(double) * node.size(), cudaMemcpyHostToDevice, p->stream);
    if (dev) {   // the caller's payout and cotangent are ready once its stream reaches this point
        if (e == cudaSuccess) e = plan_dev_events(p);
        if (e == cudaSuccess) e = cudaEventRecord(p->ev_in, dev->st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(p->stream, p->ev_in, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_payout, payout, sizeof(double) * k, cudaMemcpyDeviceToDevice, p->stream);
        if (e == cudaSuccess) {
            k_gather_perm<<<(n + 255) / 256, 256, 0, p->stream>>>(n, cot, p->d_perm, v->d_cot);
            ++p->launches;
            e = cudaGetLastError();
        }
    } else {
        v->h_cot.resize(n);
        for (int i = 0; i < n; ++i) v->h_cot[i] = cot[p->perm[i]];   // sorted order
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_payout, payout, sizeof(double) * k, cudaMemcpyHostToDevice, p->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(v->d_cot, v->h_cot.data(), sizeof(double) * n, cudaMemcpyHostToDevice, p->stream);
    }
    if (e != cudaSuccess) { err = std::string("upload: ") + cudaGetErrorString(e); return -1; }
    int logNeed = 12, logTW = 0;
    for (int l = 1; l < p->L; ++l) {
        if (p->lv[l].fft) logNeed = std::max(logNeed, plan_ilog2(p->lv[l].fftn));
        if (p->lv[l].kind == 2) logNeed = std::max(logNeed, plan_ilog2(2 * p->lv[l].deg));
    }
    const double2 *tw = twiddles(logNeed, p->stream, err, &logTW);
    if (!tw) return -1;
    if (nact == 0) {
        cudaMemsetAsync(v->d_gradS, 0, sizeof(double) * n, p->stream);
        cudaMemsetAsync(v->d_gradP, 0, sizeof(double) * k, p->stream);
    }
    if (!p->ev0) { cudaEventCreate(&p->ev0); cudaEventCreate(&p->ev1); }
    cudaEventRecord(p->ev0, p->stream);
    const int np = (p->nparts >= 2 && nact >= 2 && !p->prof.on) ? std::min(p->nparts, nact) : 1;
    if (np == 1) {
        for (int q0 = 0; q0 < nact; q0 += p->qc) {
            const int nq = std::min(p->qc, nact - q0);
            run_chunk(p, q0, nq, tw, logTW, q0 == 0, /*divide=*/false);
            adjoint_chunk(v, q0, nq, tw, logTW, q0 == 0, node_terms);
        }
    } else {
        // every chunk in up to np pieces of consecutive nodes, one stream each
        // (forward tree and adjoint passes); the sums over nodes stay in node
        // order: each piece's sums wait for the piece before
        cudaEventRecord(p->ev_split, p->stream);
        for (int i = 1; i < np; ++i) cudaStreamWaitEvent(p->part[i].st, p->ev_split, 0);
        cudaEvent_t prev = nullptr;
        for (int q0 = 0; q0 < nact; q0 += p->qc) {
            int q = q0, r = std::min(p->qc, nact - q0);
            for (int i = 0; i < np && r > 0; ++i) {
                const int m = chunk_piece_nodes(p, i, np, r);
                run_chunk(p, q, m, tw, logTW, q == 0, /*divide=*/false, i ? &p->part[i] : nullptr);
                adjoint_chunk(v, q, m, tw, logTW, q == 0, node_terms, i, prev, p->ev_acc[i]);
                prev = p->ev_acc[i];
                q += m;
                r -= m;
            }
        }
        cudaStreamWaitEvent(p->stream, prev, 0);
    }
    launch_scatter(n, v->d_gradS, p->d_perm, nullptr, p->d_out, p->stream);
    ++p->launches;
    cudaEventRecord(p->ev1, p->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("launch: ") + cudaGetErrorString(e); return -1; }
    v->pending = true;
    v->pQ = Q;
    v->pnode = node_terms;
    v->pqidx = std::move(qidx);
    v->pw = std::move(w);
    v->pnact = nact;
    v->pt0 = t0;
    return 0;
}

int vjp_plan_finish(VjpPlan *v, double *grad_S, double *grad_payout, IcmGpuRunStats *stats, std::string &err,
                    const DevIO *dev) {
    if (!v || !v->pending || !grad_S || !grad_payout) { err = "invalid arguments (no VJP enqueued)"; return -1; }
    v->pending = false;
    Plan *p = v->p;
    const int n = p->n, k = p->k, nact = v->pnact, Q = v->pQ;
    const bool node_terms = v->pnode;
    cudaError_t e = cudaSuccess;
    if (dev) {   // gradients into the caller's buffers; its stream waits for them
        e = cudaMemcpyAsync(grad_S, p->d_out, sizeof(double) * n, cudaMemcpyDeviceToDevice, p->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(grad_payout, v->d_gradP, sizeof(double) * k, cudaMemcpyDeviceToDevice, p->stream);
        if (node_terms && nact) {   // the largest stack's node term, chained on the host
            std::vector<double> hA(nact), hB(nact);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hA.data(), v->d_nodeA, sizeof(double) * nact, cudaMemcpyDeviceToHost, p->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hB.data(), v->d_nodeB, sizeof(double) * nact, cudaMemcpyDeviceToHost, p->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
            if (e == cudaSuccess) {
                k_add_one<<<1, 1, 0, p->stream>>>(grad_S, p->perm[0], node_shift_term(Q, p->Smax, v->pqidx, v->pw, hA, hB));
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(p->ev_out, p->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(dev->st, p->ev_out, 0);
        if (e != cudaSuccess) { err = std::string("execution: ") + cudaGetErrorString(e); return -1; }
        if (stats) {
            memset(stats, 0, sizeof(*stats));
            stats->total_ns = now_ns() - v->pt0;
            stats->peak_vram_bytes = p->arena_bytes + v->arena_bytes;
            stats->engine = 1;
            stats->B = p->B;
        }
        return 0;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad_S, p->d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad_payout, v->d_gradP, sizeof(double) * k, cudaMemcpyDeviceToHost, p->stream);
    std::vector<double> hA(node_terms ? nact : 0), hB(node_terms ? nact : 0);
    if (node_terms && nact && e == cudaSuccess)
        e = cudaMemcpyAsync(hA.data(), v->d_nodeA, sizeof(double) * nact, cudaMemcpyDeviceToHost, p->stream);
    if (node_terms && nact && e == cudaSuccess)
        e = cudaMemcpyAsync(hB.data(), v->d_nodeB, sizeof(double) * nact, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) { err = std::string("execution: ") + cudaGetErrorString(e); return -1; }
    if (node_terms && nact) grad_S[p->perm[0]] += node_shift_term(Q, p->Smax, v->pqidx, v->pw, hA, hB);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    p->last_device_ms = ms;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->total_ns = now_ns() - v->pt0;
        stats->peak_vram_bytes = p->arena_bytes + v->arena_bytes;
        stats->engine = 1;
        stats->B = p->B;
    }
    return 0;
}

int vjp_plan_run(VjpPlan *v, int Q, const double *payout, const double *cot, double *grad_S, double *grad_payout,
                 int flags, IcmGpuRunStats *stats, std::string &err) {
    if (!grad_S || !grad_payout) { err = "invalid arguments"; return -1; }
    if (vjp_plan_enqueue(v, Q, payout, cot, flags, err) != 0) return -1;
    return vjp_plan_finish(v, grad_S, grad_payout, stats, err);
}

}  // namespace icmg
