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
// leave-one-out recurrences over the block (no division).  Tree levels run
// on coefficients (the plan is made without spectral levels); the forward
// tree of a chunk of nodes is recomputed by the VJP call itself and stays in
// the plan's buffers for the adjoint passes.  Levels whose FFT fits one CTA
// use one-kernel transforms that reuse the children's spectra cached by the
// forward build; other levels use schoolbook kernels.
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
constexpr int kVjpMaxN = 8192;

inline unsigned nblkv(long work, int threads) { return (unsigned)((work + threads - 1) / threads); }
double now_ns() {
    return (double)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
}  // namespace

__device__ __forceinline__ int vjp_cb(int N) { return N >= 8192 ? 1 : 4096 / N; }
static inline int vjp_cb_h(int N) { return N >= 8192 ? 1 : 4096 / N; }
static inline size_t vjp_up_smem(int N) { return (size_t)vjp_cb_h(N) * (N + N / 2) * sizeof(double2); }
static inline size_t vjp_down_smem(int N) { return (size_t)vjp_cb_h(N) * N * sizeof(double2); }

// ------------------------------------------------------------ leaf adjoints
// gbar of every leaf block: sum_i c_i Q_i by the running pair
// (prod, wsum) -> (prod f, wsum f + c prod).  One thread per (block, node).
template <int B>
__global__ void k_adj_leaf_up(int n, int k, int nblocks, const double *__restrict__ S,
                              const double *__restrict__ node, int q0, const double *__restrict__ a,
                              const double *__restrict__ cot, double *__restrict__ gb0, size_t gb0_q, int gst0) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (b >= nblocks) return;
    const double *nd = node + 3 * (q0 + q);
    const double w = nd[1], iv = nd[2];
    const int start = b * B, bs = min(B, n - start);
    double P[B + 1], W[B + 1];
#pragma unroll
    for (int m = 0; m <= B; ++m) { P[m] = 0.0; W[m] = 0.0; }
    P[0] = 1.0;
    const double *arow = a + (size_t)q * n + start;
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
}

// per player: Q_i and H_i by the same recurrence over the block without i,
// then the three terms of abar_i and the node's share of dL/dS_i
template <int B>
__global__ void k_adj_leaf_down(int n, int k, const double *__restrict__ S, const double *__restrict__ node, int q0,
                                const double *__restrict__ a, const double *__restrict__ cot,
                                const double *__restrict__ g0, size_t g0_q, int gst0, const double *__restrict__ Pb0,
                                size_t Pb0_q, int pst0, int plen0, double *__restrict__ contrib,
                                double *__restrict__ partA, double *__restrict__ partB) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (i >= n) return;
    const double *nd = node + 3 * (q0 + q);
    const double logv = nd[0], w = nd[1], iv = nd[2];
    const int b = i / B, start = b * B, bs = min(B, n - start), pk = min(bs, k);
    const int me = i - start;
    const double *arow = a + (size_t)q * n + start;
    if (arow[me] == 0.0) {   // leaf factor 0 (S logv < -700): no share; g of its block may be pruned
        contrib[(size_t)q * n + i] = 0.0;
        if (partA) {
            partA[(size_t)q * n + i] = 0.0;
            partB[(size_t)q * n + i] = 0.0;
        }
        return;
    }
    double P[B], H[B];
#pragma unroll
    for (int m = 0; m < B; ++m) { P[m] = 0.0; H[m] = 0.0; }
    P[0] = 1.0;
#pragma unroll
    for (int j = 0; j < B; ++j) {
        if (j >= bs || j == me) continue;
        const double aj = arow[j], bj = 1.0 - aj;
        double pw = w * S[start + j] * aj * iv;
        if (!isfinite(pw)) pw = 0.0;
        const double c = cot[start + j] * pw;
#pragma unroll
        for (int m = B - 1; m >= 1; --m) H[m] = fma(aj, H[m], fma(bj, H[m - 1], c * P[m]));
        H[0] = fma(aj, H[0], c * P[0]);
#pragma unroll
        for (int m = B - 1; m >= 1; --m) P[m] = fma(aj, P[m], bj * P[m - 1]);
        P[0] *= aj;
    }
    const double *g = g0 + q * g0_q + (size_t)b * gst0;
    double inner = 0.0, bterm = 0.0;
#pragma unroll
    for (int m = 0; m < B; ++m) {
        if (m < pk) {
            const double gm = g[m];
            inner = fma(gm, P[m], inner);
            bterm = fma(gm, H[m] - (m ? H[m - 1] : 0.0), bterm);
        }
    }
    double cterm = 0.0;
    if (Pb0) {
        const double *pb = Pb0 + q * Pb0_q + (size_t)b * pst0;
#pragma unroll
        for (int m = 0; m <= B; ++m)
            if (m < plen0) cterm = fma(pb[m], (m < B ? P[m] : 0.0) - (m ? P[m - 1] : 0.0), cterm);
    }
    const double ai = arow[me], Si = S[i], ci = cot[i];
    const double pw = w * Si * ai * iv;
    const bool fin = isfinite(pw);
    const double abar = (fin ? ci * w * Si * iv * inner : 0.0) + bterm + cterm;
    contrib[(size_t)q * n + i] = (fin ? ci * w * ai * iv * inner : 0.0) + abar * logv * ai;
    if (partA) {   // dL/dlogv and w dL/dw shares of this player (a = v^S, 1/v)
        const double li = fin ? ci * pw * inner : 0.0;
        partA[(size_t)q * n + i] = abar * Si * ai - li;
        partB[(size_t)q * n + i] = li;
    }
}

// ------------------------------------------------------- schoolbook passes
// gbar of parents j >= j0: P_R gbar_L + P_L gbar_R, truncated to gpl; a lone
// child passes its gbar up unchanged (its g was the parent's).
__global__ void k_adj_up_school(const double *__restrict__ Pc, size_t Pc_q, int pst_c, int lc, int nreal_c,
                                const double *__restrict__ gbc, size_t gbc_q, int gst_c, int glen_c,
                                double *__restrict__ gbp, size_t gbp_q, int gst_p, int gpl, int nreal_p, int j0,
                                ZeroPrefix z) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
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
__global__ void k_adj_down_school(const double *__restrict__ gp, size_t gp_q, int gst_p, int gpl,
                                  const double *__restrict__ Pbp, size_t Pbp_q, int pst_p, int lp,
                                  const double *__restrict__ Pc, size_t Pc_q, int pst_c, int lc,
                                  const double *__restrict__ gbc, size_t gbc_q, int gst_c, int glen_c,
                                  double *__restrict__ Pbc, int nreal_c, int c0, ZeroPrefix z) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
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
// Upward, pairs [0, npairs): z = gbar_L + i gbar_R -> FFT N -> the children's
// gbar spectra (cached for the downward pass) -> Y = S_R G_L + S_L G_R with
// the children's P spectra S cached by the forward build -> half-size inverse
// -> gbar_parent.  N >= glen_c + lc - 1, so the products do not wrap.
__global__ void __launch_bounds__(kVjpThreads)
k_adj_up_fused(const double *__restrict__ gbc, size_t gbc_q, int gst_c, int glen_c, int npairs, int logN,
               const double2 *__restrict__ spec, double2 *__restrict__ gspec, double *__restrict__ gbp, size_t gbp_q,
               int gst_p, int gpl, const double2 *__restrict__ tw, int logTW, ZeroPrefix z) {
    extern __shared__ double2 sm[];
    const int N = 1 << logN, h = N >> 1;
    const int cb = vjp_cb(N);
    const int q = blockIdx.y;
    const int j0 = blockIdx.x * cb;
    const int cnt = min(cb, npairs - j0);
    if (zp_cold(z, q, j0 + cnt - 1)) {   // wholly-zero parents: gbar = 0
        for (int e = threadIdx.x; e < cnt * gst_p; e += blockDim.x)
            gbp[q * gbp_q + (size_t)(j0 + e / gst_p) * gst_p + e % gst_p] = 0.0;
        return;
    }
    double2 *Z = sm;
    double2 *U = sm + (size_t)cb * N;
    const double *base = gbc + q * gbc_q;
    for (int e = threadIdx.x; e < cnt * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const double *gL = base + (size_t)(2 * (j0 + it)) * gst_c;
        Z[e] = (t < glen_c) ? make_double2(gL[t], gL[gst_c + t]) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, cnt, tw, logTW);
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e / h, f = e - it * h;
        const double2 *z = Z + (size_t)it * N;
        const int fc = h - f;
        const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
        const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
        const double2 GLf = cscale(cadd(zf, cconj(zn)), 0.5);
        const double2 GRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
        const double2 GLc = cscale(cadd(zc, cconj(zcn)), 0.5);
        const double2 GRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
        const size_t so = (2 * ((size_t)q * npairs + j0 + it)) * (size_t)(h + 1);
        const double2 *sL = spec + so, *sR = sL + (h + 1);
        double2 *gL = gspec + so, *gR = gL + (h + 1);
        gL[f] = GLf;
        gR[f] = GRf;
        if (f == 0) { gL[h] = GLc; gR[h] = GRc; }
        const double2 Yf = cadd(cmul(sR[f], GLf), cmul(sL[f], GRf));
        const double2 Yc = cadd(cmul(sR[fc], GLc), cmul(sL[fc], GRc));
        double2 E = cadd(Yf, cconj(Yc)), D = csub(Yf, cconj(Yc));
        if (f == 0) { E.y = 0.0; D.y = 0.0; }
        const double2 O = cmulc(D, __ldg(&tw[(long)f << (logTW - logN)]));
        U[(size_t)it * h + bitrev(f, logN - 1)] = cadd(E, cmul_pi(O));
    }
    __syncthreads();
    smem_fft_dit<+1>(U, logN - 1, cnt, tw, logTW);
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < cnt * gst_p; e += blockDim.x) {
        const int it = e / gst_p, t = e - it * gst_p;
        double *out = gbp + q * gbp_q + (size_t)(j0 + it) * gst_p;
        double v = 0.0;
        if (t < gpl) {
            const double2 uv = U[(size_t)it * h + (t >> 1)];
            v = ((t & 1) ? uv.y : uv.x) * inv;
        }
        out[t] = v;
    }
}

// Downward, pairs [0, npairs): w = g_parent + i Pbar_parent -> FFT N -> their
// spectra G, R; Z = Y_L + i Y_R with Y_L = G conj(Gbar_R) + R conj(S_R)
// (children's gbar spectra from the upward pass, P spectra from the build),
// in place in natural order, then bit-reversed and inverted.  The only wrap
// is P_sib[lc-1] Pbar_parent[2(lc-1)] when N = 2(lc-1); it is corrected
// from the coefficients.
__global__ void __launch_bounds__(kVjpThreads)
k_adj_down_fused(const double *__restrict__ gp, size_t gp_q, int gst_p, int gpl, const double *__restrict__ Pbp,
                 size_t Pbp_q, int pst_p, int lp, const double *__restrict__ Pc, size_t Pc_q, int pst_c, int lc,
                 int npairs, int logN, const double2 *__restrict__ spec, const double2 *__restrict__ gspec,
                 double *__restrict__ Pbc, const double2 *__restrict__ tw, int logTW, ZeroPrefix z) {
    extern __shared__ double2 sm[];
    const int N = 1 << logN, h = N >> 1;
    const int cb = vjp_cb(N);
    const int q = blockIdx.y;
    const int j0 = blockIdx.x * cb;
    const int cnt = min(cb, npairs - j0);
    if (zp_cold(z, q, j0 + cnt - 1)) return;   // children of wholly-zero parents: not needed
    double2 *Z = sm;
    for (int e = threadIdx.x; e < cnt * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const double *g = gp + q * gp_q + (size_t)(j0 + it) * gst_p;
        double x = (t < gpl) ? g[t] : 0.0, y = 0.0;
        if (Pbp && t < lp) y = Pbp[q * Pbp_q + (size_t)(j0 + it) * pst_p + t];
        Z[e] = make_double2(x, y);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, cnt, tw, logTW);
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e / h, f = e - it * h;
        double2 *z = Z + (size_t)it * N;
        const size_t so = (2 * ((size_t)q * npairs + j0 + it)) * (size_t)(h + 1);
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
    __syncthreads();
    smem_bitrev_map(Z, logN, cnt, [](int, int, double2 v) { return v; });
    smem_fft_dit<+1>(Z, logN, cnt, tw, logTW);
    const double inv = 1.0 / N;
    const bool wrap = Pbp && 2 * (lc - 1) == N;
    for (int e = threadIdx.x; e < cnt * 2 * pst_c; e += blockDim.x) {
        const int it = e / (2 * pst_c), r = e - it * 2 * pst_c;
        const int side = r / pst_c, i = r - side * pst_c;
        const int c = 2 * (j0 + it) + side;
        double *out = Pbc + q * Pc_q + (size_t)c * pst_c;
        double v = 0.0;
        if (i < lc) {
            const double2 zv = Z[(size_t)it * N + i];
            v = (side ? zv.y : zv.x) * inv;
            if (wrap && i == lc - 1) {
                const double *pb = Pbp + q * Pbp_q + (size_t)(j0 + it) * pst_p;
                const double *Ps = Pc + q * Pc_q + (size_t)(c ^ 1) * pst_c;
                const double top = (N < lp) ? pb[N] : 0.0;
                v = fma(Ps[lc - 1], top - pb[0], v);
            }
        }
        out[i] = v;
    }
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
}

// ------------------------------------------------------------ plans
static bool level_fused(const Level &v) { return v.fft && v.npairs > 0 && v.fftn <= kVjpMaxN && fused_ok(v.fftn); }

VjpPlan *vjp_plan_create(int n, const double *S, int k, std::string &err, size_t budget) {
    // the adjoint buffers roughly double the tree's per-node memory
    Plan *p = plan_create(n, S, k, nullptr, err, /*coeff_only=*/true, /*q_bytes_scale=*/2.2, budget);
    if (!p) return nullptr;
    VjpPlan *v = new VjpPlan();
    v->p = p;
    const int qc = p->qc, L = p->L;
    v->kst = ((k + 1) & ~1);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_cot = take(8 * (size_t)n), o_gs = take(8 * (size_t)n), o_gp = take(8 * (size_t)k);
    const size_t o_root = take(8 * (size_t)qc * v->kst);
    size_t o_gb[kMaxLevels], o_Pb[kMaxLevels], o_gsp[kMaxLevels];
    for (int l = 0; l < L; ++l) {
        const Level &lv = p->lv[l];
        o_gb[l] = lv.g_q ? take(8 * (size_t)qc * lv.g_q) : 0;
        o_Pb[l] = lv.P_q ? take(8 * (size_t)qc * lv.P_q) : 0;
        o_gsp[l] = (l >= 1 && level_fused(lv)) ? take(16 * (size_t)qc * lv.spec_q) : 0;
    }
    cudaError_t e = cudaMallocAsync((void **)&v->arena, off, p->stream);
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
    for (int l = 0; l < L; ++l) {
        const Level &lv = p->lv[l];
        v->gb[l] = lv.g_q ? (double *)(A + o_gb[l]) : nullptr;
        v->Pb[l] = lv.P_q ? (double *)(A + o_Pb[l]) : nullptr;
        v->gspec[l] = o_gsp[l] ? (double2 *)(A + o_gsp[l]) : nullptr;
    }
    return v;
}

void vjp_plan_destroy(VjpPlan *v) {
    if (!v) return;
    if (v->arena) {
        cudaFreeAsync(v->arena, v->p->stream);
        cudaStreamSynchronize(v->p->stream);
    }
    if (v->d_partA) cudaFree(v->d_partA);
    plan_destroy(v->p);
    delete v;
}

// adjoint passes of one chunk (the forward tree of the chunk is in place)
static void adjoint_chunk(VjpPlan *v, int q0, int nq, const double2 *tw, int logTW, bool first, bool node_terms) {
    Plan *p = v->p;
    cudaStream_t st = p->stream;
    const int L = p->L, B = p->B, n = p->n, k = p->k;
    Level *lv = p->lv;
    long &launches = p->launches;
    const int *zp = p->zskip ? p->d_z : nullptr;   // zero-prefix pruning, as in the forward
    const dim3 gb0((unsigned)nblkv(p->nblocks, 128), nq);
    // gbar of the leaf blocks (for L = 1 the single block is the root)
    switch (B) {
        case 4: k_adj_leaf_up<4><<<gb0, 128, 0, st>>>(n, k, p->nblocks, p->d_S, p->d_node, q0, p->d_a, v->d_cot, v->gb[0], lv[0].g_q, lv[0].gst); break;
        case 8: k_adj_leaf_up<8><<<gb0, 128, 0, st>>>(n, k, p->nblocks, p->d_S, p->d_node, q0, p->d_a, v->d_cot, v->gb[0], lv[0].g_q, lv[0].gst); break;
        case 16: k_adj_leaf_up<16><<<gb0, 128, 0, st>>>(n, k, p->nblocks, p->d_S, p->d_node, q0, p->d_a, v->d_cot, v->gb[0], lv[0].g_q, lv[0].gst); break;
        default: k_adj_leaf_up<32><<<gb0, 128, 0, st>>>(n, k, p->nblocks, p->d_S, p->d_node, q0, p->d_a, v->d_cot, v->gb[0], lv[0].g_q, lv[0].gst); break;
    }
    ++launches;
    // upward: gbar of every level; the root's is this chunk's dL/dpayout
    for (int l = 1; l <= L - 1; ++l) {
        const Level &c = lv[l - 1], &pl = lv[l];
        const bool root = (l == L - 1);
        double *out = root ? v->d_root : v->gb[l];
        const size_t out_q = root ? (size_t)v->kst : pl.g_q;
        const int gst_p = root ? v->kst : pl.gst;
        const int gpl = root ? k : pl.glen;
        const ZeroPrefix zpar{zp, q0, pl.deg};
        int j0 = 0;
        if (level_fused(pl)) {
            const int N = pl.fftn, logN = plan_ilog2(N);
            const int cb = vjp_cb_h(N);
            k_adj_up_fused<<<dim3((pl.npairs + cb - 1) / cb, nq), kVjpThreads, vjp_up_smem(N), st>>>(
                v->gb[l - 1], c.g_q, c.gst, c.glen, pl.npairs, logN, pl.spec, v->gspec[l], out, out_q, gst_p, gpl, tw,
                logTW, zpar);
            ++launches;
            j0 = pl.npairs;
        }
        const long work = (long)(pl.nreal - j0) * gst_p;
        if (work > 0) {
            k_adj_up_school<<<dim3(nblkv(work, 256), nq), 256, 0, st>>>(c.P, c.P_q, c.pst, c.plen, c.nreal,
                                                                       v->gb[l - 1], c.g_q, c.gst, c.glen, out,
                                                                       out_q, gst_p, gpl, pl.nreal, j0, zpar);
            ++launches;
        }
    }
    // downward: Pbar of every level below the root
    for (int l = L - 1; l >= 1; --l) {
        const Level &c = lv[l - 1], &pl = lv[l];
        const bool root = (l == L - 1);
        const double *gp = root ? p->d_payout : pl.g;
        const size_t gp_q = root ? 0 : pl.g_q;
        const int gst_p = root ? 0 : pl.gst;
        const int gpl = root ? k : pl.glen;
        const double *Pbp = root ? nullptr : v->Pb[l];
        const ZeroPrefix zpar{zp, q0, pl.deg}, zch{zp, q0, c.deg};
        int c0 = 0;
        if (level_fused(pl)) {
            const int N = pl.fftn, logN = plan_ilog2(N);
            const int cb = vjp_cb_h(N);
            k_adj_down_fused<<<dim3((pl.npairs + cb - 1) / cb, nq), kVjpThreads, vjp_down_smem(N), st>>>(
                gp, gp_q, gst_p, gpl, Pbp, pl.P_q, pl.pst, pl.plen, c.P, c.P_q, c.pst, c.plen, pl.npairs, logN,
                pl.spec, v->gspec[l], v->Pb[l - 1], tw, logTW, zpar);
            ++launches;
            c0 = 2 * pl.npairs;
        }
        const long work = (long)(c.nreal - c0) * c.pst;
        if (work > 0) {
            k_adj_down_school<<<dim3(nblkv(work, 256), nq), 256, 0, st>>>(
                gp, gp_q, gst_p, gpl, Pbp, pl.P_q, pl.pst, pl.plen, c.P, c.P_q, c.pst, c.plen, v->gb[l - 1], c.g_q,
                c.gst, c.glen, v->Pb[l - 1], c.nreal, c0, zch);
            ++launches;
        }
    }
    // per player: the node's share of dL/dS, then ordered sums over nodes
    const double *g0 = (L == 1) ? p->d_payout : lv[0].g;
    const size_t g0_q = (L == 1) ? 0 : lv[0].g_q;
    const int gst0 = (L == 1) ? 0 : lv[0].gst;
    const double *Pb0 = (L == 1) ? nullptr : v->Pb[0];
    const dim3 gd((unsigned)nblkv(n, 128), nq);
    double *pA = node_terms ? v->d_partA : nullptr, *pB = node_terms ? v->d_partB : nullptr;
    switch (B) {
        case 4: k_adj_leaf_down<4><<<gd, 128, 0, st>>>(n, k, p->d_S, p->d_node, q0, p->d_a, v->d_cot, g0, g0_q, gst0, Pb0, lv[0].P_q, lv[0].pst, lv[0].plen, p->d_contrib, pA, pB); break;
        case 8: k_adj_leaf_down<8><<<gd, 128, 0, st>>>(n, k, p->d_S, p->d_node, q0, p->d_a, v->d_cot, g0, g0_q, gst0, Pb0, lv[0].P_q, lv[0].pst, lv[0].plen, p->d_contrib, pA, pB); break;
        case 16: k_adj_leaf_down<16><<<gd, 128, 0, st>>>(n, k, p->d_S, p->d_node, q0, p->d_a, v->d_cot, g0, g0_q, gst0, Pb0, lv[0].P_q, lv[0].pst, lv[0].plen, p->d_contrib, pA, pB); break;
        default: k_adj_leaf_down<32><<<gd, 128, 0, st>>>(n, k, p->d_S, p->d_node, q0, p->d_a, v->d_cot, g0, g0_q, gst0, Pb0, lv[0].P_q, lv[0].pst, lv[0].plen, p->d_contrib, pA, pB); break;
    }
    k_accum_strided<<<nblkv(n, 256), 256, 0, st>>>(n, nq, p->d_contrib, (size_t)n, v->d_gradS, first ? 1 : 0);
    const double *root = (L == 1) ? v->gb[0] : v->d_root;
    const size_t root_q = (L == 1) ? lv[0].g_q : (size_t)v->kst;
    k_accum_strided<<<nblkv(k, 256), 256, 0, st>>>(k, nq, root, root_q, v->d_gradP, first ? 1 : 0);
    launches += 3;
    if (node_terms) {
        k_node_reduce<<<nq, 256, 0, st>>>(n, pA, pB, v->d_nodeA + q0, v->d_nodeB + q0);
        ++launches;
    }
}

int vjp_plan_enqueue(VjpPlan *v, int Q, const double *payout, const double *cot, int flags, std::string &err) {
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
        if (v->d_partA) cudaFree(v->d_partA);
        v->d_partA = nullptr;
        const size_t cap = std::max(nact, 1);
        e = cudaMalloc(&v->d_partA, sizeof(double) * (2 * (size_t)p->qc * n + 2 * cap));
        if (e != cudaSuccess) { err = std::string("node-term buffers: ") + cudaGetErrorString(e); return -1; }
        v->d_partB = v->d_partA + (size_t)p->qc * n;
        v->d_nodeA = v->d_partB + (size_t)p->qc * n;
        v->d_nodeB = v->d_nodeA + cap;
        v->node_cap = (int)cap;
    }
    if (nact > p->qmax) {
        if (p->d_node) cudaFree(p->d_node);
        p->d_node = nullptr;
        p->d_z = nullptr;
        const size_t nb = sizeof(double) * 3 * (size_t)std::max(nact, 1);
        e = cudaMalloc(&p->d_node, nb + sizeof(int) * (size_t)std::max(nact, 1));
        if (e != cudaSuccess) { err = std::string("node buffer: ") + cudaGetErrorString(e); return -1; }
        p->d_z = (int *)((char *)p->d_node + nb);
        p->qmax = nact;
    }
    p->h_z.resize(nact);
    for (int j = 0; j < nact; ++j) p->h_z[j] = zero_prefix(p->S_sorted.data(), n, node[3 * j]);
    if (nact) e = cudaMemcpyAsync(p->d_z, p->h_z.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, p->stream);
    v->h_cot.resize(n);
    for (int i = 0; i < n; ++i) v->h_cot[i] = cot[p->perm[i]];   // sorted order
    if (nact && e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_node, node.data(), sizeof(double) * node.size(), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_payout, payout, sizeof(double) * k, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(v->d_cot, v->h_cot.data(), sizeof(double) * n, cudaMemcpyHostToDevice, p->stream);
    if (e != cudaSuccess) { err = std::string("upload: ") + cudaGetErrorString(e); return -1; }
    int logNeed = 12, logTW = 0;
    for (int l = 1; l < p->L; ++l)
        if (p->lv[l].fft) logNeed = std::max(logNeed, plan_ilog2(p->lv[l].fftn));
    const double2 *tw = twiddles(logNeed, p->stream, err, &logTW);
    if (!tw) return -1;
    if (nact == 0) {
        cudaMemsetAsync(v->d_gradS, 0, sizeof(double) * n, p->stream);
        cudaMemsetAsync(v->d_gradP, 0, sizeof(double) * k, p->stream);
    }
    if (!p->ev0) { cudaEventCreate(&p->ev0); cudaEventCreate(&p->ev1); }
    cudaEventRecord(p->ev0, p->stream);
    for (int q0 = 0; q0 < nact; q0 += p->qc) {
        const int nq = std::min(p->qc, nact - q0);
        run_chunk(p, q0, nq, tw, logTW, q0 == 0, /*divide=*/false);
        adjoint_chunk(v, q0, nq, tw, logTW, q0 == 0, node_terms);
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

int vjp_plan_finish(VjpPlan *v, double *grad_S, double *grad_payout, IcmGpuRunStats *stats, std::string &err) {
    if (!v || !v->pending || !grad_S || !grad_payout) { err = "invalid arguments (no VJP enqueued)"; return -1; }
    v->pending = false;
    Plan *p = v->p;
    const int n = p->n, k = p->k, nact = v->pnact, Q = v->pQ;
    const bool node_terms = v->pnode;
    cudaError_t e = cudaSuccess;
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
