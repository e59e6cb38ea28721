// spectral.cu -- tree levels carried in the frequency domain.
//
// A node X of degree d (d+1 coefficients) keeps spec2(X) = DFT_{2d}(x), the
// d+1 Hermitian bins of its spectrum at twice its degree, plus its end
// coefficients x_0 and x_d.  For a parent X of two children of degree D
// (d = 2D), with children spectra S_L, S_R at size 2D:
//
// build:  C = S_L S_R is X's spectrum at size 2D (x_{2D} folded onto x_0),
//         i.e. the even bins of spec2(X).  One inverse transform of size D
//         gives x (endpoints replaced by L_0 R_0 and L_D R_D); the odd bins
//         are the half-bin transform H[f] = sum_t y_t e^{-2 pi i (2f+1) t/4D}
//         of y = x with y_0 = x_0 - x_{2D}, one forward transform of size D
//         of the twisted packing (y_{2s} + i y_{2s+1}) e^{-2 pi i s/2D}.
//         Two size-D transforms per node instead of one size-2D and one
//         size-D on the coefficient path.
// propagate (the transpose): with G = DFT_{2D}(g_X), a child's correlation
//         y = IDFT_{2D}(G conj S_sib) has g_child = y[0:D).  Its even bins
//         are DFT_D(a + b), its odd bins the half-bin transform of a - b
//         (a = y[0:D), b = y[D:2D)).  One inverse half-bin transform gives
//         a - b; the child's g spectrum DFT_D(a) is (even bins + DFT_D(a-b))/2,
//         or, where the level below works on coefficients, a = (IDFT_D(even
//         bins) + (a - b))/2.  Two size-D/2 transforms per child.
//
// All transforms are decimation-in-time (bit-reversed in, natural out).  The
// twist in front of a second (forward) transform is that transform's half
// shift, folded into its twiddles (fft.cuh); other pointwise maps between two
// transforms are applied while permuting the data into bit-reversed order in
// place (smem_bitrev_map).  A missing sibling
// (ragged tree edge) is the polynomial 1: spectrum 1, ends (1, 0).
#include <algorithm>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"

namespace icmg {

constexpr int kSpecThreads = 256;
constexpr int kSpecThreadsMax = 512;   // CTAs alone on an SM (one 8192-point item) take twice the warps
static inline int spec_tpb(size_t smem) { return smem > kOneCtaSmem ? kSpecThreadsMax : kSpecThreads; }
constexpr int kSpecMaxM = kSpecMaxD;   // largest transform one CTA holds in shared memory

static inline int ilog2s(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
// complex points per CTA of the work-list launches (batches): items = kSpecPts / M
constexpr int kSpecPts = 2048;
__host__ __device__ __forceinline__ int spec_cb(int M) { return M >= kSpecPts ? 1 : kSpecPts / M; }
// items per CTA of a single plan's launch for a level with `pts` complex points
// per CTA (0: 4096); never more points than spec_cb's largest CTA (8192)
static inline int pts_cb(int pts, int M) {
    if (pts <= 0) pts = 4096;
    pts = std::min(pts, kSpecMaxM);
    return M >= pts ? 1 : pts / M;
}
static inline size_t spec_smem(int M) { return (size_t)spec_cb(M) * M * sizeof(double2); }
// build and propagate: the items' data plus one view and one index per item
constexpr size_t kViewBytes = 96;
constexpr size_t kItemBytes = kViewBytes + sizeof(int);
static inline size_t spec_smem_v(int M) { return (size_t)spec_cb(M) * (M * sizeof(double2) + kItemBytes); }
static size_t spec_smem_v_max() {   // over the transform sizes a level can use (D >= 4)
    size_t mx = 0;
    for (int M = 4; M <= kSpecMaxM; M *= 2) mx = std::max(mx, spec_smem_v(M));
    return mx;
}

__device__ __forceinline__ double2 twl(const double2 *__restrict__ tw, long idx) { return __ldg(&tw[idx]); }

// ---------------------------------------------------------------------------
// spec2 and ends of nodes given by coefficients: real FFT of size 2d through
// a complex transform of size d.  cb nodes per CTA.
__device__ void spec_init_body(const SpecInitArgs &A, int bx, int q) {
    const auto P = A.P;
    const auto P_q = A.P_q;
    const auto pst = A.pst;
    const auto plen = A.plen;
    const auto nreal = A.nreal;
    const auto logd = A.logd;
    const auto spec2 = A.spec2;
    const auto s2_q = A.s2_q;
    const auto ends = A.ends;
    const auto e_q = A.e_q;
    const auto tw = A.tw;
    const auto logTW = A.logTW;

    extern __shared__ double2 sm[];
    const int d = 1 << logd;
    const int cb = A.cb;
        const int j0 = bx * cb;
    const int cnt = min(cb, nreal - j0);
    if (cnt <= 0) return;
    if (zp_cold(A.z, q, j0 + cnt - 1)) {   // every node x^d: spec2 = (-1)^f, ends (0, 1)
        for (int e = threadIdx.x; e < cnt * (d + 1); e += blockDim.x) {
            const int it = e / (d + 1), f = e - it * (d + 1);
            spec2[q * s2_q + (size_t)(j0 + it) * (d + 1) + f] = make_double2((f & 1) ? -1.0 : 1.0, 0.0);
            if (f == 0) {
                double *en = ends + q * e_q + (size_t)(j0 + it) * 2;
                en[0] = 0.0;
                en[1] = (d < plen) ? 1.0 : 0.0;
            }
        }
        return;
    }
    for (int e = threadIdx.x; e < cnt * d; e += blockDim.x) {
        const int it = e >> logd, r = e & (d - 1);
        const int s = (int)bitrev(r, logd);
        const double *x = P + q * P_q + (size_t)(j0 + it) * pst;
        const int t0 = 2 * s, t1 = 2 * s + 1;
        sm[e] = make_double2(t0 < plen ? x[t0] : 0.0, t1 < plen ? x[t1] : 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(sm, logd, cnt, tw, logTW);
    // X[f] = (Z[f] + conj Z[d-f])/2 + e^{-2 pi i f/2d} (Z[f] - conj Z[d-f])/(2i),
    // by mirror pairs (f, d - f), f <= d/2
    const int dp = (d >> 1) + 1;
    for (int e = threadIdx.x; e < cnt * dp; e += blockDim.x) {
        const int it = e / dp, f = e - it * dp;
        const double2 *z = sm + (size_t)it * d;
        const double2 zf = z[f], zc = z[(d - f) & (d - 1)];
        const double2 Ev = cadd(zf, cconj(zc)), Od = cmul_mi(csub(zf, cconj(zc)));   // both doubled
        double2 *out = spec2 + q * s2_q + (size_t)(j0 + it) * (d + 1);
        double2 Xf, Xc;
        half_sum_tw_pair(Ev, Od, tw_tangent(tw, logTW), (long)f << (logTW - logd - 1), logTW, Xf, Xc);
        out[f] = Xf;
        if (f != 0 && 2 * f != d) out[d - f] = Xc;
        if (f == 0) {
            out[d] = cscale(csub(Ev, Od), 0.5);
            const double *x = P + q * P_q + (size_t)(j0 + it) * pst;
            double *en = ends + q * e_q + (size_t)(j0 + it) * 2;
            en[0] = x[0];
            en[1] = (d < plen) ? x[d] : 0.0;
        }
    }
}

// ---------------------------------------------------------------------------
// Build of one spectral level: nodes j of level l from children 2j, 2j+1 of
// level l-1 (degree D = 2^logD, spec2 of D+1 bins).  Writes spec2 (2D+1 bins)
// and ends of each node, and its coefficients when Pout != null.
//
// Pointwise phases work on mirror pairs of bins so shared products are
// computed once and the halves and 1/2D scalings are applied once, at the
// end: with C = S_L S_R, the inverse input for bins f and D-f is
//   U(f) = E + i O,  U(D-f) = conj(E) + i conj(O),
//   E = C[f] + conj C[D-f],  O = (C[f] - conj C[D-f]) e^{+2 pi i f/2D},
// and the odd output bins of a mirror pair (f, D-1-f) are
//   H(f) = (Ep + T) / 4D,  H(D-1-f) = conj(Ep - T) / 4D,
//   Ep = c[f] + conj c[D-1-f],  T = -i (c[f] - conj c[D-1-f]) e^{-2 pi i (2f+1)/4D}.
//
// Every item (parent) of a CTA is described by a view staged in shared memory
// (pointers for its node and quadrature node), so a CTA may hold items of
// different tournaments (packed work lists); a single plan fills the views
// from its one argument block.
struct SbView {
    const double2 *sL, *sR;   // children's spec2 (sR null: missing right child, the polynomial 1)
    const double *eL, *eR;    // children's ends (eR null: (1, 0))
    double2 *ps;              // parent spec2 (2D+1 bins) or null
    double *pe;               // parent ends or null
    double *po;               // parent coefficients or null
    int pst, plen, cold;
};
static_assert(sizeof(SbView) <= kViewBytes, "view size");

__device__ __forceinline__ void sb_fill(const SpecBuildArgs &A, int q, int q0, int j, int D, SbView &v) {
    v.sL = A.cspec + q * A.cs_q + (size_t)(2 * j) * (D + 1);
    const bool has_r = (2 * j + 1) < A.nreal_c;
    v.sR = has_r ? v.sL + (D + 1) : nullptr;
    v.eL = A.cends + q * A.ce_q + (size_t)(2 * j) * 2;
    v.eR = has_r ? v.eL + 2 : nullptr;
    v.ps = A.pspec ? A.pspec + q * A.ps_q + (size_t)j * (2 * D + 1) : nullptr;
    v.pe = A.pends ? A.pends + q * A.pe_q + (size_t)j * 2 : nullptr;
    v.po = A.Pout ? A.Pout + q * A.Po_q + (size_t)j * A.pst_p : nullptr;
    v.pst = A.pst_p;
    v.plen = A.plen_p;
    const ZeroPrefix z{A.z.zp, q0, A.z.span};
    v.cold = zp_cold(z, q, j) ? 1 : 0;
}

// the build of cnt items whose views are in V (shared memory, synchronised);
// idx from partition_items: nh items to transform first, wholly-zero ones
// after; want_spec: the items' parents keep spec2 (uniform over a launch)
__device__ void spec_build_core(const SbView *V, const int *idx, int cnt, int nh, int logD,
                                const double2 *__restrict__ tw, int logTW, double2 *sm, bool want_spec) {
    const int D = 1 << logD;
    const int hD = D >> 1;
    if (nh < cnt) {   // wholly-zero parents x^{2D}: spec2 (-1)^f, ends (0, 1), coefficients a single 1
        int maxpst = 0;
        for (int r = nh; r < cnt; ++r) maxpst = max(maxpst, V[idx[r]].pst);
        const int nb2 = 2 * D + 1;
        const int per = max(nb2, maxpst);
        for (int e = threadIdx.x; e < (cnt - nh) * per; e += blockDim.x) {
            const int r = nh + e / per, f = e % per;
            const SbView &v = V[idx[r]];
            if (v.ps && f < nb2) v.ps[f] = make_double2((f & 1) ? -1.0 : 1.0, 0.0);
            if (v.pe && f == 0) {
                v.pe[0] = 0.0;
                v.pe[1] = 1.0;
            }
            if (v.po && f < v.pst) v.po[f] = (f == 2 * D && f < v.plen) ? 1.0 : 0.0;
        }
    }
    if (nh == 0) return;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *tt = tw_tangent(tw, logTW);
    // 1. product spectrum (even bins of spec2(X)) and the inverse input, by mirror pairs
    const int np1 = hD + 1;
    for (int e = threadIdx.x; e < nh * np1; e += blockDim.x) {
        const int it = e / np1, f = e - it * np1;
        const SbView &v = V[idx[it]];
        const double2 Cf = cmul(v.sL[f], v.sR ? v.sR[f] : one);
        const double2 Cc = cmul(v.sL[D - f], v.sR ? v.sR[D - f] : one);
        if (v.ps) {
            v.ps[2 * f] = Cf;
            v.ps[2 * (D - f)] = Cc;
        }
        double2 E = cadd(Cf, cconj(Cc)), Dd = csub(Cf, cconj(Cc));
        if (f == 0) { E.y = 0.0; Dd.y = 0.0; }
        double2 Uf, Uc;   // O = Dd e^{+2 pi i f/2D}
        mirror_inv_input(E, Dd, tt, (long)f << (logTW - logD - 1), logTW, Uf, Uc);
        double2 *u = sm + (size_t)it * D;
        u[bitrev(f, logD)] = Uf;
        if (f != 0 && f != hD) u[bitrev(D - f, logD)] = Uc;
    }
    __syncthreads();
    smem_fft_dit<+1>(sm, logD, nh, tw, logTW);
    // 2. u_s = 2D (x_{2s} + i x_{2s+1}); coefficients where a coefficient level
    //    sits above (truncated at plen, zero padding to pst) and the endpoint
    //    fix; the twist e^{-2 pi i s/2D} is the forward transform's half shift
    const double one_over_2D = 1.0 / (2.0 * D);
    auto coeffs = [&](int it, int s, double2 u) -> double2 {
        const SbView &v = V[idx[it]];
        const double xtop = v.eL[1] * (v.eR ? v.eR[1] : 0.0);
        if (s == 0) {
            const double x0 = v.eL[0] * (v.eR ? v.eR[0] : 1.0);
            if (v.pe) {
                v.pe[0] = x0;
                v.pe[1] = xtop;
            }
            u.x = (x0 - xtop) * (2.0 * D);   // y_0 = x_0 - x_{2D}, in the unscaled units of u
        }
        if (v.po) {
            const int pst = v.pst, plen = v.plen;
            const double x0 = (s == 0) ? v.eL[0] * (v.eR ? v.eR[0] : 1.0) : u.x * one_over_2D;
            if (2 * s < pst) v.po[2 * s] = (2 * s < plen) ? x0 : 0.0;
            if (2 * s + 1 < pst) v.po[2 * s + 1] = (2 * s + 1 < plen) ? u.y * one_over_2D : 0.0;
            if (s == 0) {
                if (2 * D < pst) v.po[2 * D] = (2 * D < plen) ? xtop : 0.0;
                for (int t = 2 * D + 1; t < pst; ++t) v.po[t] = 0.0;
            }
        }
        return u;
    };
    if (!want_spec) {   // the level above works on coefficients: no spectrum needed
        for (int e = threadIdx.x; e < nh * D; e += blockDim.x) coeffs(e >> logD, e & (D - 1), sm[e]);
        return;
    }
    smem_bitrev_map(sm, logD, nh, coeffs);
    smem_fft_dit<-1, +1>(sm, logD, nh, tw, logTW);   // c_f = sum_s u_s e^{-2 pi i s (f + 1/2)/D}
    // 3. odd bins by mirror pairs (f, D-1-f), f < D/2
    const double kb = 1.0 / (4.0 * D);
    for (int e = threadIdx.x; e < nh * hD; e += blockDim.x) {
        const int it = e / hD, f = e - it * hD;
        const double2 *c = sm + (size_t)it * D;
        double2 Hf, Hc;   // T = -i (a - b) e^{-2 pi i (2f+1)/4D}
        mirror_out_pair(c[f], cconj(c[D - 1 - f]), kb, tt, (long)(2 * f + 1) << (logTW - logD - 2), logTW, Hf, Hc);
        double2 *ps = V[idx[it]].ps;
        ps[2 * f + 1] = Hf;
        ps[2 * (D - 1 - f) + 1] = Hc;
    }
}

template <class View>
__device__ __forceinline__ View *item_views(double2 *sm, int cb, int M) {
    return reinterpret_cast<View *>(sm + (size_t)cb * M);
}
template <class View>
__device__ __forceinline__ int *item_index(View *V, int cb) {
    return reinterpret_cast<int *>(V + cb);
}
// idx[0, nhot) = items to transform, idx[nhot, cnt) = wholly-zero items, in
// order; a CTA may hold items of different tournaments, so pruning is per
// item (one thread partitions at most a few hundred flags)
__device__ __forceinline__ bool item_skip(const SbView &v) { return v.cold; }
template <class View>
__device__ __forceinline__ int partition_items(const View *V, int *idx, int cnt) {
    __shared__ int nhot_s;
    if (threadIdx.x == 0) {
        int h = 0;
        for (int it = 0; it < cnt; ++it)
            if (!item_skip(V[it])) idx[h++] = it;
        int c = h;
        for (int it = 0; it < cnt; ++it)
            if (item_skip(V[it])) idx[c++] = it;
        nhot_s = h;
    }
    __syncthreads();
    return nhot_s;
}

__device__ void spec_build_body(const SpecBuildArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int D = 1 << A.logD;
    const int cb = A.cb;
    const int j0 = bx * cb;
    const int cnt = min(cb, A.nreal_p - j0);
    if (cnt <= 0) return;
    SbView *V = item_views<SbView>(sm, cb, D);
    int *idx = item_index(V, cb);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) sb_fill(A, q, A.z.q0, j0 + it, D, V[it]);
    __syncthreads();
    const int nh = partition_items(V, idx, cnt);
    spec_build_core(V, idx, cnt, nh, A.logD, A.tw, A.logTW, sm, A.pspec != nullptr);
}

// packed: slots[s] = (descriptor, parent); all descriptors of a launch share
// the transform size and whether parents keep spec2
__device__ void spec_build_packed(const SpecBuildArgs *__restrict__ Dsc, const int2 *__restrict__ slots, int nslots,
                                  int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const SpecBuildArgs &A0 = Dsc[slots[0].x];
    const int D = 1 << A0.logD;
    const int cb = spec_cb(D);
    const int s0 = bx * cb;
    const int cnt = min(cb, nslots - s0);
    if (cnt <= 0) return;
    SbView *V = item_views<SbView>(sm, cb, D);
    int *idx = item_index(V, cb);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        sb_fill(Dsc[sl.x], q, q0, sl.y, D, V[it]);
    }
    __syncthreads();
    const int nh = partition_items(V, idx, cnt);
    spec_build_core(V, idx, cnt, nh, A0.logD, A0.tw, A0.logTW, sm, A0.pspec != nullptr);
}

// ---------------------------------------------------------------------------
// g spectra from g coefficients: G = DFT_d(g) (bins 0..d/2), real FFT of size
// d through a complex transform of size d/2.  g_q == 0 and one node: the root.
__device__ void gspec_body(const GspecArgs &A, int bx, int q) {
    const auto g = A.g;
    const auto g_q = A.g_q;
    const auto gst = A.gst;
    const auto glen = A.glen;
    const auto nreal = A.nreal;
    const auto logd = A.logd;
    const auto G = A.G;
    const auto G_q = A.G_q;
    const auto hot = A.hot;
    const auto tw = A.tw;
    const auto logTW = A.logTW;

    extern __shared__ double2 sm[];
    const int h = 1 << (logd - 1);
    const int lh = logd - 1;
    const int cb = A.cb;
        const int j0 = bx * cb;
    const int cnt = min(cb, nreal - j0);
    if (cnt <= 0 || zp_cold(A.z, q, j0 + cnt - 1)) return;   // nothing below reads a wholly-zero node's g
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e >> lh, r = e & (h - 1);
        const int s = (int)bitrev(r, lh);
        const double *x = g + q * g_q + (size_t)(j0 + it) * gst;
        const int t0 = 2 * s, t1 = 2 * s + 1;
        sm[e] = make_double2(t0 < glen ? x[t0] : 0.0, t1 < glen ? x[t1] : 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(sm, lh, cnt, tw, logTW);
    const int hp = (h >> 1) + 1;   // mirror pairs (f, h - f), f <= h/2
    for (int e = threadIdx.x; e < cnt * hp; e += blockDim.x) {
        const int it = e / hp, f = e - it * hp;
        const int j = j0 + it;
        double2 *out = G + q * G_q + (size_t)j * (h + 1);
        if (hot && !hot[j]) {
            out[f] = out[h - f] = make_double2(0.0, 0.0);
            continue;
        }
        const double2 *z = sm + (size_t)it * h;
        const double2 zf = z[f], zc = z[(h - f) & (h - 1)];
        const double2 Ev = cadd(zf, cconj(zc)), Od = cmul_mi(csub(zf, cconj(zc)));   // both doubled
        double2 Xf, Xc;
        half_sum_tw_pair(Ev, Od, tw_tangent(tw, logTW), (long)f << (logTW - logd), logTW, Xf, Xc);
        out[f] = Xf;
        if (f != 0 && 2 * f != h) out[h - f] = Xc;
        if (f == 0) out[h] = cscale(csub(Ev, Od), 0.5);
    }
}

// ---------------------------------------------------------------------------
// Propagate of one spectral level: parent j (degree 2D, G of D+1 bins),
// children 2j, 2j+1 (degree D = 2^logD, spec2 of D+1 bins).  Each child gets
// its g spectrum (D/2+1 bins) when Gout != null, else its g coefficients.
// Work per child: a transform of size D/2 (inverse half-bin), then a second
// one (forward for the spectrum, inverse of the even bins for coefficients).
//
// With Y = G conj(S_sib) and w_f = e^{-2 pi i (2f+1)/2D}, the inverse
// half-bin input of a mirror pair (f, h-1-f), h = D/2, is (doubled)
//   C'(f) = A + i B,  C'(h-1-f) = conj A + i conj B,
//   A = Y[2f+1] + conj Y[2f'+1],  B = (Y[2f+1] - conj Y[2f'+1]) conj w_f;
// the child's spectrum bins f and h-f come from the forward transform z as
//   X(f) = E + T,  X(h-f) = conj(E - T),  E = z_f + conj z_{h-f},
//   T = -i (z_f - conj z_{h-f}) e^{-2 pi i f/D},
//   G_child[f] = Y[2f]/2 + X(f)/8h   (all scalings folded into the last step).
struct SpView;
__device__ __forceinline__ bool item_skip(const SpView &v);
struct SpView {
    const double2 *G;      // parent's g spectrum (D+1 bins)
    const double2 *S[2];   // children's spec2 (null: no such child, as a sibling the polynomial 1)
    double2 *Gout[2];      // children's g spectra (h+1 bins), or null
    double *gout[2];       // children's g coefficients, or null
    int gst, glen;
    int live[2];           // the child exists
    int zero[2];           // subset-cold child: its outputs are zero
    int cold;              // wholly-zero parent: the item is skipped
};
static_assert(sizeof(SpView) <= kViewBytes, "view size");
// per item: its view, its index in the partition and two child slots
static_assert(sizeof(SpView) + 3 * sizeof(int) <= kItemBytes, "propagate item bytes");
__device__ __forceinline__ bool item_skip(const SpView &v) {
    return v.cold || !((v.live[0] && !v.zero[0]) || (v.live[1] && !v.zero[1]));
}

__device__ __forceinline__ void sp_fill(const SpecPropArgs &A, int q, int q0, int j, int D, SpView &v) {
    const int h = D >> 1;
    v.G = A.Gp + q * A.Gp_q + (size_t)j * (D + 1);
    for (int side = 0; side < 2; ++side) {
        const int c = 2 * j + side;
        const bool live = c < A.nreal_c;
        v.live[side] = live ? 1 : 0;
        v.S[side] = live ? A.cspec + q * A.cs_q + (size_t)c * (D + 1) : nullptr;
        v.Gout[side] = (A.Gout && live) ? A.Gout + q * A.Go_q + (size_t)c * (h + 1) : nullptr;
        v.gout[side] = (A.gout && live) ? A.gout + q * A.go_q + (size_t)c * A.gst_c : nullptr;
        v.zero[side] = (live && A.hot_c && !A.hot_c[c]) ? 1 : 0;
    }
    v.gst = A.gst_c;
    v.glen = A.glen_c;
    const ZeroPrefix z{A.z.zp, q0, A.z.span};
    v.cold = zp_cold(z, q, j) ? 1 : 0;
}

// the propagate of the nh parents idx[0, nh) whose views are in V (the
// others skipped: nothing below a wholly-zero parent or a pair of
// subset-cold children is read).  Only the children that exist and are not
// subset-cold are transformed (cidx: 2 cb slots of shared memory, those
// children first as view * 2 + side, then the subset-cold ones from the
// end, whose outputs are zero; the reference CPU's single-sided correlate,
// src/cpu/icm.c:1733-1815).  want_G: children get g spectra (else
// coefficients), uniform over a launch.
__device__ void spec_prop_core(const SpView *V, const int *idx, int nh, int *cidx, int cb, int logD,
                               const double2 *__restrict__ tw, int logTW, double2 *sm, bool want_G) {
    const int D = 1 << logD;
    const int h = D >> 1, lh = logD - 1;
    if (nh == 0) return;
    __shared__ int nk_s, nz_s;
    if (threadIdx.x == 0) {
        int c = 0, z = 0;
        for (int it = 0; it < nh; ++it) {
            const SpView &v = V[idx[it]];
            for (int side = 0; side < 2; ++side) {
                if (!v.live[side]) continue;
                if (v.zero[side]) cidx[2 * cb - 1 - z++] = 2 * idx[it] + side;
                else cidx[c++] = 2 * idx[it] + side;
            }
        }
        nk_s = c;
        nz_s = z;
    }
    __syncthreads();
    const int nk = nk_s, nz = nz_s;   // children transformed, h slots each; subset-cold children
    {   // subset-cold children: zero outputs, one warp each
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int zc = warp; zc < nz; zc += nw) {
            const int c2 = cidx[2 * cb - 1 - zc];
            const SpView &v = V[c2 >> 1];
            const int side = c2 & 1;
            if (want_G)
                for (int f = lane; f <= h; f += 32) v.Gout[side][f] = make_double2(0.0, 0.0);
            else
                for (int t = lane; t < v.gst; t += 32) v.gout[side][t] = 0.0;
        }
    }
    if (nk == 0) return;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *tt = tw_tangent(tw, logTW);
    // 1. odd bins of Y -> inverse half-bin input, by mirror pairs
    const int hp = (h + 1) >> 1;   // pairs per child (h = 1: one self pair)
    for (int e = threadIdx.x; e < nk * hp; e += blockDim.x) {
        const int kk = e / hp, f = e - kk * hp;
        const int fp = h - 1 - f;
        const int c2 = cidx[kk];
        const SpView &v = V[c2 >> 1];
        const double2 *S = v.S[(c2 & 1) ^ 1];   // the sibling's spectrum
        const double2 *G = v.G;
        const double2 Y1 = cmulc(G[2 * f + 1], S ? S[2 * f + 1] : one);
        const double2 Y2 = cconj(cmulc(G[2 * fp + 1], S ? S[2 * fp + 1] : one));
        double2 Xf, Xc;   // A + i B, conj(A) + i conj(B), B = (Y1 - Y2) conj(w_f)
        mirror_inv_input(cadd(Y1, Y2), csub(Y1, Y2), tt, (long)(2 * f + 1) << (logTW - logD - 1), logTW, Xf, Xc);
        double2 *x = sm + (size_t)kk * h;
        x[bitrev(f, lh)] = Xf;
        if (fp != f) x[bitrev(fp, lh)] = Xc;
    }
    __syncthreads();
    smem_fft_dit<+1>(sm, lh, nk, tw, logTW);
    // 2. untwist (unscaled): w_s = c'_s e^{+2 pi i s/D}; in front of the
    //    forward transform it is that transform's half shift by -1/2 bin
    auto untwist = [&](int, int s, double2 v) -> double2 {
        return (s == 0) ? v : cmulc(v, twl(tw, (long)s << (logTW - logD)));
    };
    if (want_G) {
        smem_bitrev_map(sm, lh, nk, [](int, int, double2 v) { return v; });
        smem_fft_dit<-1, -1>(sm, lh, nk, tw, logTW);   // z_f = sum_s w_s e^{-2 pi i s f/h}
        // 3a. child spectra by mirror pairs (f, h-f), f <= h/2
        const double kx = 1.0 / (8.0 * h);
        const int hq = (h >> 1) + 1;
        for (int e = threadIdx.x; e < nk * hq; e += blockDim.x) {
            const int kk = e / hq, f = e - kk * hq;
            const int fp = h - f;
            const int c2 = cidx[kk];
            const SpView &v = V[c2 >> 1];
            const int side = c2 & 1;
            double2 *out = v.Gout[side];
            const double2 *G = v.G;
            const double2 *S = v.S[side ^ 1];
            const double2 *z = sm + (size_t)kk * h;
            const double2 zf = z[f & (h - 1)], zc = cconj(z[fp & (h - 1)]);
            const double2 E = cadd(zf, zc);
            double r;   // T = r u = -i (zf - zc) e^{-2 pi i f/D}
            const double2 u = tanmul_t<-1>(cmul_mi(csub(zf, zc)), tt, (long)f << (logTW - logD), logTW, &r);
            const double2 Yf = cmulc(G[2 * f], S ? S[2 * f] : one);
            const double2 Xf = make_double2(fma(r, u.x, E.x), fma(r, u.y, E.y));
            out[f] = make_double2(fma(kx, Xf.x, 0.5 * Yf.x), fma(kx, Xf.y, 0.5 * Yf.y));
            if (fp != f) {
                const double2 Yc = cmulc(G[2 * fp], S ? S[2 * fp] : one);
                const double2 Xc = make_double2(fma(-r, u.x, E.x), fma(r, u.y, -E.y));   // conj(E - T)
                out[fp] = make_double2(fma(kx, Xc.x, 0.5 * Yc.x), fma(kx, Xc.y, 0.5 * Yc.y));
            }
        }
        return;
    }
    // 3b. coefficients: (a-b) = w / 2h (C' doubled, inverse unscaled); store
    //     (a-b)/2, then add (a+b)/2 from the inverse of the even bins
    const double ka = 1.0 / (4.0 * h);
    for (int e = threadIdx.x; e < nk * h; e += blockDim.x) {
        const int kk = e >> lh, s = e & (h - 1);
        const int c2 = cidx[kk];
        const SpView &v = V[c2 >> 1];
        double *out = v.gout[c2 & 1];
        const double2 w = untwist(kk, s, sm[e]);
        if (2 * s < v.glen) out[2 * s] = ka * w.x;
        if (2 * s + 1 < v.glen) out[2 * s + 1] = ka * w.y;
    }
    __syncthreads();
    // U[f] = E + i O of the even-bin spectrum Ye (bins 0..h of a real size-D spectrum)
    for (int e = threadIdx.x; e < nk * h; e += blockDim.x) {
        const int kk = e >> lh, f = e & (h - 1);
        const int c2 = cidx[kk];
        const SpView &v = V[c2 >> 1];
        const double2 *S = v.S[(c2 & 1) ^ 1];
        const double2 *G = v.G;
        const double2 Cf = cmulc(G[2 * f], S ? S[2 * f] : one);
        const double2 Cc = cmulc(G[2 * (h - f)], S ? S[2 * (h - f)] : one);
        double2 E = cadd(Cf, cconj(Cc)), Dd = csub(Cf, cconj(Cc));
        if (f == 0) { E.y = 0.0; Dd.y = 0.0; }
        double2 Uf, Uc;   // O = Dd e^{+2 pi i f/D}; Uc unused
        mirror_inv_input(E, Dd, tt, (long)f << (logTW - logD), logTW, Uf, Uc);
        sm[(size_t)kk * h + bitrev(f, lh)] = Uf;
    }
    __syncthreads();
    smem_fft_dit<+1>(sm, lh, nk, tw, logTW);
    const double inv_D = 1.0 / D;
    for (int e = threadIdx.x; e < nk * h; e += blockDim.x) {
        const int kk = e >> lh, s = e & (h - 1);
        const int c2 = cidx[kk];
        const SpView &v = V[c2 >> 1];
        double *out = v.gout[c2 & 1];
        const int gst = v.gst, glen = v.glen;
        const double2 w = sm[e];
        if (2 * s < gst) out[2 * s] = (2 * s >= glen) ? 0.0 : out[2 * s] + 0.5 * w.x * inv_D;
        if (2 * s + 1 < gst) out[2 * s + 1] = (2 * s + 1 >= glen) ? 0.0 : out[2 * s + 1] + 0.5 * w.y * inv_D;
    }
}

__device__ void spec_prop_body(const SpecPropArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int D = 1 << A.logD;
    const int cbp = A.cb;   // parents per CTA; 2 children each
    const int j0 = bx * cbp;
    const int cnt = min(cbp, A.npar - j0);
    if (cnt <= 0) return;
    SpView *V = item_views<SpView>(sm, cbp, D);
    int *idx = item_index(V, cbp);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) sp_fill(A, q, A.z.q0, j0 + it, D, V[it]);
    __syncthreads();
    const int nh = partition_items(V, idx, cnt);
    spec_prop_core(V, idx, nh, idx + cbp, cbp, A.logD, A.tw, A.logTW, sm, A.Gout != nullptr);
}

// packed: slots[s] = (descriptor, parent); all descriptors of a launch share
// the transform size and whether children get g spectra
__device__ void spec_prop_packed(const SpecPropArgs *__restrict__ Dsc, const int2 *__restrict__ slots, int nslots,
                                 int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const SpecPropArgs &A0 = Dsc[slots[0].x];
    const int D = 1 << A0.logD;
    const int cbp = spec_cb(D);
    const int s0 = bx * cbp;
    const int cnt = min(cbp, nslots - s0);
    if (cnt <= 0) return;
    SpView *V = item_views<SpView>(sm, cbp, D);
    int *idx = item_index(V, cbp);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        sp_fill(Dsc[sl.x], q, q0, sl.y, D, V[it]);
    }
    __syncthreads();
    const int nh = partition_items(V, idx, cnt);
    spec_prop_core(V, idx, nh, idx + cbp, cbp, A0.logD, A0.tw, A0.logTW, sm, A0.Gout != nullptr);
}

__global__ void __launch_bounds__(kSpecThreadsMax) k_spec_init(SpecInitArgs A) { spec_init_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kSpecThreadsMax) k_spec_build(SpecBuildArgs A) { spec_build_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kSpecThreadsMax) k_gspec_init(GspecArgs A) { gspec_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kSpecThreadsMax) k_spec_prop(SpecPropArgs A) { spec_prop_body(A, blockIdx.x, blockIdx.y); }

size_t spec_smem_bytes(int M) { return spec_smem(M); }
void spec_wl_set_smem_limits();

// ---------------------------------------------------------------------------
void spec_set_smem_limits() {
    const int mx = (int)spec_smem(kSpecMaxM), mv = (int)spec_smem_v_max();
    cudaFuncSetAttribute(k_spec_init, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_spec_build, cudaFuncAttributeMaxDynamicSharedMemorySize, mv);
    cudaFuncSetAttribute(k_gspec_init, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_spec_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, mv);
    spec_wl_set_smem_limits();
}

SpecInitArgs spec_init_args(const Level &v, const double2 *tw, int logTW, double *fq, size_t *smem) {
    const int logd = ilog2s(v.deg), d = 1 << logd;
    const int cb = spec_cb(d);
    if (fq) *fq = (5.0 * d * logd + 20.0 * d) * v.nreal;
    if (smem) *smem = spec_smem(d);
    return SpecInitArgs{v.P, v.P_q, v.pst, v.plen, v.nreal, logd, v.spec2, v.spec2_q, v.ends, v.ends_q, tw, logTW,
                        (v.nreal + cb - 1) / cb, ZeroPrefix{nullptr, 0, v.deg}, cb};
}

SpecBuildArgs spec_build_args(const Level &c, const Level &p, bool write_coeffs, const double2 *tw, int logTW,
                              double *fq, size_t *smem) {
    const int logD = ilog2s(c.deg), D = 1 << logD;
    const int cb = spec_cb(D);
    if (fq) *fq = (10.0 * D * logD + 60.0 * D) * p.nreal;
    if (smem) *smem = spec_smem_v(D);
    return SpecBuildArgs{c.spec2, c.spec2_q, c.ends, c.ends_q, c.nreal, p.nreal, logD, p.spec2, p.spec2_q,
                         p.spec2 ? p.ends : nullptr, p.ends_q, write_coeffs ? p.P : nullptr, p.P_q, p.pst, p.plen, tw,
                         logTW, (p.nreal + cb - 1) / cb, ZeroPrefix{nullptr, 0, p.deg}, cb};
}

GspecArgs gspec_args(const double *g, size_t g_q, int gst, int glen, int nreal, const Level &v, double2 *G, size_t G_q,
                     const uint8_t *hot, const double2 *tw, int logTW, double *fq, size_t *smem) {
    const int logd = ilog2s(v.deg), h = 1 << (logd - 1);
    const int cb = spec_cb(h);
    if (fq) *fq = (5.0 * h * (logd - 1) + 20.0 * h) * nreal;
    if (smem) *smem = spec_smem(h);
    return GspecArgs{g, g_q, gst, glen, nreal, logd, G, G_q, hot, tw, logTW, (nreal + cb - 1) / cb,
                     ZeroPrefix{nullptr, 0, v.deg}, cb};
}

SpecPropArgs spec_prop_args(const double2 *Gp, size_t Gp_q, const Level &c, const Level &p, bool children_spectral,
                            const uint8_t *hot_c, const double2 *tw, int logTW, double *fq, size_t *smem) {
    const int logD = ilog2s(c.deg), D = 1 << logD;
    const int cbp = spec_cb(D);
    if (fq) *fq = (2.0 * 2 * 5.0 * (D / 2) * (logD - 1) + 60.0 * D) * p.nreal;
    if (smem) *smem = spec_smem_v(D);
    return SpecPropArgs{Gp, Gp_q, c.spec2, c.spec2_q, c.nreal, p.nreal, logD, children_spectral ? c.G : nullptr,
                        c.G_q, c.g, c.g_q, c.gst, c.glen, hot_c, tw, logTW, (p.nreal + cbp - 1) / cbp,
                        ZeroPrefix{nullptr, 0, p.deg}, cbp};
}

void launch_spec_init(const Level &v, int nq, const double2 *tw, int logTW, cudaStream_t st, Prof *pr, const int *zp,
                      int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    SpecInitArgs A = spec_init_args(v, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(pts_cb(v.cta_pts, 1 << A.logd), A.nreal, nq);
    A.nbx = (A.nreal + A.cb - 1) / A.cb;
    sm = (size_t)A.cb * (1 << A.logd) * sizeof(double2);
    pr->begin("spec_init", fq * nq, st);
    k_spec_init<<<dim3(A.nbx, nq), spec_tpb(sm), sm, st>>>(A);
    pr->end(st);
}

void launch_spec_build(const Level &c, const Level &p, bool write_coeffs, int nq, const double2 *tw, int logTW,
                       cudaStream_t st, Prof *pr, const int *zp, int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    SpecBuildArgs A = spec_build_args(c, p, write_coeffs, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(pts_cb(p.cta_pts, 1 << A.logD), p.nreal, nq);
    A.nbx = (p.nreal + A.cb - 1) / A.cb;
    sm = (size_t)A.cb * ((size_t)(1 << A.logD) * sizeof(double2) + kItemBytes);
    pr->begin("spec_build", fq * nq, st);
    k_spec_build<<<dim3(A.nbx, nq), spec_tpb(sm), sm, st>>>(A);
    pr->end(st);
}

void launch_gspec_init(const double *g, size_t g_q, int gst, int glen, int nreal, const Level &v, double2 *G,
                       size_t G_q, int nq, const uint8_t *hot, const double2 *tw, int logTW, cudaStream_t st,
                       Prof *pr, const int *zp, int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    GspecArgs A = gspec_args(g, g_q, gst, glen, nreal, v, G, G_q, hot, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(pts_cb(v.cta_pts, 1 << (A.logd - 1)), A.nreal, nq);
    A.nbx = (A.nreal + A.cb - 1) / A.cb;
    sm = (size_t)A.cb * (1 << (A.logd - 1)) * sizeof(double2);
    pr->begin("gspec_init", fq * nq, st);
    k_gspec_init<<<dim3(A.nbx, nq), spec_tpb(sm), sm, st>>>(A);
    pr->end(st);
}

void launch_spec_prop(const double2 *Gp, size_t Gp_q, const Level &c, const Level &p, bool children_spectral, int nq,
                      const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr, const int *zp,
                      int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    SpecPropArgs A = spec_prop_args(Gp, Gp_q, c, p, children_spectral, hot_c, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(pts_cb(p.cta_pts, 1 << A.logD), p.nreal, nq);
    A.nbx = (p.nreal + A.cb - 1) / A.cb;
    sm = (size_t)A.cb * ((size_t)(1 << A.logD) * sizeof(double2) + kItemBytes);
    pr->begin("spec_prop", fq * nq, st);
    k_spec_prop<<<dim3(A.nbx, nq), spec_tpb(sm), sm, st>>>(A);
    pr->end(st);
}

// ---------------------------------------------------------------- work lists
__global__ void __launch_bounds__(kSpecThreadsMax)
kw_spec_init(const SpecInitArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    SpecInitArgs A = D[t.x];
    A.z.q0 = q0;
    spec_init_body(A, t.y, blockIdx.y);
}
__global__ void __launch_bounds__(kSpecThreadsMax)
kw_gspec(const GspecArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    GspecArgs A = D[t.x];
    A.z.q0 = q0;
    gspec_body(A, t.y, blockIdx.y);
}
__global__ void __launch_bounds__(kSpecThreadsMax)
kw_spec_build_packed(const SpecBuildArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    spec_build_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}
__global__ void __launch_bounds__(kSpecThreadsMax)
kw_spec_prop_packed(const SpecPropArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    spec_prop_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}

void spec_wl_set_smem_limits() {
    const int mx = (int)spec_smem(kSpecMaxM), mv = (int)spec_smem_v_max();
    cudaFuncSetAttribute(kw_spec_init, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_gspec, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_spec_build_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, mv);
    cudaFuncSetAttribute(kw_spec_prop_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, mv);
}

// packed launch: nslots items, cb items per CTA
void launch_packed_spec(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                        cudaStream_t st) {
    if (nslots <= 0 || nq <= 0) return;
    const dim3 g((nslots + cb - 1) / cb, nq);
    if (op == WOp::SpecBuild)
        kw_spec_build_packed<<<g, spec_tpb(smem), smem, st>>>((const SpecBuildArgs *)desc, slots, nslots, q0);
    else
        kw_spec_prop_packed<<<g, spec_tpb(smem), smem, st>>>((const SpecPropArgs *)desc, slots, nslots, q0);
}

void launch_worklist_spec(WOp op, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                          cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    switch (op) {
        case WOp::SpecInit: kw_spec_init<<<g, spec_tpb(smem), smem, st>>>((const SpecInitArgs *)desc, tab, q0); break;
        case WOp::Gspec: kw_gspec<<<g, spec_tpb(smem), smem, st>>>((const GspecArgs *)desc, tab, q0); break;
        default: break;
    }
}

}  // namespace icmg
