// spectral_big.cu -- spectral tree levels whose transforms exceed one CTA's
// shared memory (child degree D > kSpecMaxD).  Same arithmetic as
// spectral.cu (see the formulas there), with the transforms split in the
// four-step way (a column pass and a row pass through global memory) and the
// pointwise phases carried inside those passes' loads and stores.  These are
// the top levels of a large tree (two at n = 65536, six at n = 2^20).
#include <algorithm>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"

namespace icmg {

static inline int ilog2b(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
static inline unsigned nb(long work, int threads) { return (unsigned)((work + threads - 1) / threads); }
// tree node `node` of chunk node q lies wholly inside the zero prefix
__device__ __forceinline__ bool zcold(const int *__restrict__ zp, int zq0, long span, int q, long node) {
    return zp && (node + 1) * span <= (long)zp[zq0 + q];
}

// ---- g spectra from coefficients: pack, transform, post
__global__ void k_sb_gpack(const double *__restrict__ g, size_t g_q, int gst, int glen, int nreal, int logd,
                           double2 *__restrict__ buf, const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = 1 << (logd - 1);
    const int j = (int)(idx >> (logd - 1)), s = (int)(idx & (h - 1));
    if (j >= nreal || zcold(zp, zq0, 1L << logd, q, j)) return;
    const double *x = g + q * g_q + (size_t)j * gst;
    const int t0 = 2 * s, t1 = 2 * s + 1;
    buf[((size_t)q * nreal + j) * h + s] = make_double2(t0 < glen ? x[t0] : 0.0, t1 < glen ? x[t1] : 0.0);
}

__global__ void k_sb_gpost(int nreal, int logd, const double2 *__restrict__ buf, double2 *__restrict__ G, size_t G_q,
                           const uint8_t *__restrict__ hot, const double2 *__restrict__ tw, int logTW,
                           const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = 1 << (logd - 1);
    const int j = (int)(idx >> (logd - 1)), f = (int)(idx & (h - 1));
    if (j >= nreal || zcold(zp, zq0, 1L << logd, q, j)) return;
    double2 *out = G + q * G_q + (size_t)j * (h + 1);
    if (hot && !hot[j]) {
        out[f] = make_double2(0.0, 0.0);
        if (f == 0) out[h] = make_double2(0.0, 0.0);
        return;
    }
    const double2 *z = buf + ((size_t)q * nreal + j) * h;
    const double2 zf = z[f], zc = z[(h - f) & (h - 1)];
    const double2 Ev = cadd(zf, cconj(zc)), Od = cmul_mi(csub(zf, cconj(zc)));   // both doubled
    out[f] = half_sum_tw(Ev, Od, tw_tangent(tw, logTW), (long)f << (logTW - logd), logTW);
    if (f == 0) out[h] = cscale(csub(Ev, Od), 0.5);
}

// ============================================================================
// Multi-pass levels with the pointwise steps inside the transform passes.
//
// A four-step transform of M = M1 M2 points (as fft_batched: a column pass,
// FFTs of size M1 down the columns n2 of x[M2 n1 + n2] with the twiddles
// w^(n2 k1), into scratch[n2 M1 + k1]; then a row pass, FFTs of size M2 along
// the rows k1, giving X[k1 + M1 k2]) carries the level's pointwise steps in
// its loads and stores, so no pointwise kernel makes a pass of its own:
//
//   build (transform size D):  column pass loading the product spectrum's
//     inverse input U from the children's spectra (mirror bins f, D - f),
//     row pass storing the coefficients / ends and the sequence, a column pass
//     half-shifted by +1/2 bin (the twist, folded into its twiddles), and a
//     row pass storing the parent's odd bins (mirror bins f, D - 1 - f);
//   propagate (size h = D/2, per child): column pass loading the inverse
//     half-bin input from the parent's g spectrum and the sibling's spectrum
//     (mirror bins f, h - 1 - f), row pass storing the sequence, a column pass
//     half-shifted by -1/2 bin (the untwist), and a row pass storing the
//     child's g spectrum (mirror bins f, h - f); children with h <= kSmemFftMax
//     run all of it in one CTA.
//
// A mirror pair's two bins lie in two columns (rows) that map onto each other,
// so a CTA holds whole mirror-paired columns (rows): slot 0 = {0, M/2} (each
// its own mirror) and slot p = {p, M - p} for the f <-> M - f pairings, or
// {p, M - 1 - p} for f <-> M - 1 - f.  Every bin goes through the same
// operations as in separate pointwise kernels, so results are bit for bit
// those of the unfused sequence.

struct SbfArgs {
    // build
    const double2 *cspec;
    size_t cs_q;
    const double *cends;
    size_t ce_q;
    int nreal_c, nreal_p;
    double2 *pspec;
    size_t ps_q;
    double *pends;
    size_t pe_q;
    double *Pout;
    size_t Po_q;
    int pst_p, plen_p;
    // propagate
    const double2 *Gp;
    size_t Gp_q;
    double2 *Gout;
    size_t Go_q;
    const uint8_t *hot_c;
    // transform
    int logD;            // the children's degree D
    int logM1, logM2;    // four-step split (build: D points, propagate: D/2)
    int cb;              // columns / rows per CTA (even)
    double2 *buf, *scratch;
    const double2 *tw;
    int logTW;
    const int *zp;
    int zq0;
};

__device__ __forceinline__ int slot_mirror(int slot, int m, int M) {   // slots {0, M/2}, {p, M - p}
    return slot == 0 ? (m ? (M >> 1) : 0) : (m ? M - slot : slot);
}
__device__ __forceinline__ int slot_rev(int slot, int m, int M) {      // slots {p, M - 1 - p}
    return m ? M - 1 - slot : slot;
}
// work item e of a CTA holding hc line slots from slot s0, for the
// {0, M/2} / {p, M - p} pairing of M lines of L points each (L even): the two
// (local line, point) positions of a mirror pair, c1 == -1 when the bin is its
// own mirror.  Line 0 pairs point r with (L - r) mod L, line M/2 point r with
// L - 1 - r, and line p with line M - p point r with L - 1 - r.  Slot 0 (in
// the CTA with s0 == 0) takes items 0..L; the other slots come slot-fastest,
// so that neighbouring threads touch neighbouring lines (neighbouring bins
// in global memory).
__device__ __forceinline__ void mirror_item(int e, int s0, int hc, int logL, int &c0, int &r0, int &c1, int &r1) {
    const int L = 1 << logL;
    int sl, ee, nsl;
    if (s0 == 0) {
        if (e <= L) {
            if (e <= (L >> 1)) {
                c0 = 0;
                r0 = e;
                c1 = (e == 0 || e == (L >> 1)) ? -1 : 0;
                r1 = L - e;
            } else {
                c0 = 1;
                r0 = e - (L >> 1) - 1;
                c1 = 1;
                r1 = L - 1 - r0;
            }
            return;
        }
        ee = e - (L + 1);
        nsl = hc - 1;
        sl = 1 + ee % nsl;
    } else {
        ee = e;
        nsl = hc;
        sl = ee % nsl;
    }
    c0 = 2 * sl;
    r0 = ee / nsl;
    c1 = c0 + 1;
    r1 = L - 1 - r0;
}

// ---- build, pass 1: columns of U (+1 transform)
__global__ void __launch_bounds__(256) k_sbf_build_cols(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int j = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, D = 1 << logD;
    const int logM1 = A.logM1, M1 = 1 << logM1, M2 = 1 << A.logM2, cb = A.cb;
    const int s0 = blockIdx.x * (cb >> 1);
    const bool cold = zcold(A.zp, A.zq0, 2L * D, q, j);
    double2 *ps = A.pspec ? A.pspec + q * A.ps_q + (size_t)j * (2 * D + 1) : nullptr;
    if (cold && !ps) return;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *sL = A.cspec + q * A.cs_q + (size_t)(2 * j) * (D + 1);
    const bool has_r = (2 * j + 1) < A.nreal_c;
    const double2 *sR = sL + (D + 1);
    const int nitems = (cb >> 1) * M1 + (s0 == 0 ? 1 : 0);
    for (int e = threadIdx.x; e < nitems; e += blockDim.x) {
        int c0, r0, c1, r1;
        mirror_item(e, s0, cb >> 1, logM1, c0, r0, c1, r1);
        const int fa = r0 * M2 + slot_mirror(s0 + (c0 >> 1), c0 & 1, M2);
        const int g = min(fa, D - fa);   // the pair's bin in [0, D/2]
        if (cold) {   // x^{2D}: even bins of spec2 are 1
            ps[2 * g] = one;
            ps[2 * (D - g)] = one;
            continue;
        }
        const double2 Cf = cmul(sL[g], has_r ? sR[g] : one);
        const double2 Cc = cmul(sL[D - g], has_r ? sR[D - g] : one);
        if (ps) {
            ps[2 * g] = Cf;
            ps[2 * (D - g)] = Cc;
        }
        double2 E = cadd(Cf, cconj(Cc)), Dd = csub(Cf, cconj(Cc));
        if (g == 0) { E.y = 0.0; Dd.y = 0.0; }
        double2 ug, um;   // U[g], U[D - g]
        mirror_inv_input(E, Dd, tw_tangent(A.tw, A.logTW), (long)g << (A.logTW - logD - 1), A.logTW, ug, um);
        const int pa = c0 * M1 + (int)bitrev(r0, logM1);
        if (fa == g) {
            sx[pa] = ug;
            if (c1 >= 0) sx[c1 * M1 + (int)bitrev(r1, logM1)] = um;
        } else {   // fa = D - g; its mirror holds g
            sx[pa] = um;
            sx[c1 * M1 + (int)bitrev(r1, logM1)] = ug;
        }
    }
    if (cold) return;
    __syncthreads();
    smem_fft_dit<+1>(sx, logM1, cb, A.tw, A.logTW);
    double2 *dst = A.scratch + ((size_t)q * A.nreal_p + j) * D;
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int c = e >> logM1, k1 = e & (M1 - 1);
        const int n2 = slot_mirror(s0 + (c >> 1), c & 1, M2);
        const int t = (n2 * k1) & (D - 1);
        double2 v = sx[e];
        if (t) v = twmul<+1>(v, __ldg(&A.tw[(long)t << (A.logTW - logD)]));
        dst[(long)n2 * M1 + k1] = v;
    }
}

// ---- build, pass 2: rows of the inverse; coefficients, ends, endpoint fix
__global__ void __launch_bounds__(256) k_sbf_build_rows1(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int j = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, D = 1 << logD;
    const int M1 = 1 << A.logM1, logM2 = A.logM2, M2 = 1 << logM2, cb = A.cb;
    const int k10 = blockIdx.x * cb;
    const int pst_p = A.pst_p, plen_p = A.plen_p;
    double *out = A.Pout ? A.Pout + q * A.Po_q + (size_t)j * pst_p : nullptr;
    double *en = A.pends ? A.pends + q * A.pe_q + (size_t)j * 2 : nullptr;
    if (zcold(A.zp, A.zq0, 2L * D, q, j)) {   // x^{2D}: coefficients and ends
        for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
            const int s = (e / cb) * M1 + k10 + (e % cb);
            if (out) {
                if (2 * s < pst_p) out[2 * s] = 0.0;
                if (2 * s + 1 < pst_p) out[2 * s + 1] = 0.0;
                if (s == 0) {
                    if (2 * D < pst_p) out[2 * D] = (2 * D < plen_p) ? 1.0 : 0.0;
                    for (int t = 2 * D + 1; t < pst_p; ++t) out[t] = 0.0;
                }
            }
            if (s == 0 && en) {
                en[0] = 0.0;
                en[1] = 1.0;
            }
        }
        return;
    }
    const size_t item = (size_t)q * A.nreal_p + j;
    const double2 *src = A.scratch + item * D;
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int c = e % cb, s = e / cb;
        sx[c * M2 + s] = src[(long)bitrev(s, logM2) * M1 + k10 + c];
    }
    __syncthreads();
    smem_fft_dit<+1>(sx, logM2, cb, A.tw, A.logTW);
    double2 *up = A.buf + item * D;
    const double *eL = A.cends + q * A.ce_q + (size_t)(2 * j) * 2;
    const bool has_r = (2 * j + 1) < A.nreal_c;
    const double xtop = eL[1] * (has_r ? eL[3] : 0.0);
    const double inv2D = 1.0 / (2.0 * D);
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int c = e % cb, k2 = e / cb;
        const int s = k2 * M1 + k10 + c;
        double2 u = sx[c * M2 + k2];
        if (out) {   // truncated at plen_p; the row's padding up to pst_p is zero
            const double x0 = (s == 0) ? eL[0] * (has_r ? eL[2] : 1.0) : u.x * inv2D;
            if (2 * s < pst_p) out[2 * s] = (2 * s < plen_p) ? x0 : 0.0;
            if (2 * s + 1 < pst_p) out[2 * s + 1] = (2 * s + 1 < plen_p) ? u.y * inv2D : 0.0;
            if (s == 0) {
                if (2 * D < pst_p) out[2 * D] = (2 * D < plen_p) ? xtop : 0.0;
                for (int t = 2 * D + 1; t < pst_p; ++t) out[t] = 0.0;
            }
        }
        if (s == 0) {
            const double x0 = eL[0] * (has_r ? eL[2] : 1.0);
            if (en) {
                en[0] = x0;
                en[1] = xtop;
            }
            u.x = (x0 - xtop) * (2.0 * D);
            if (A.pspec) up[0] = u;
        } else if (A.pspec) {
            up[s] = u;   // the twist e^{-2 pi i s/2D} is the next column pass's half shift
        }
    }
}

// ---- build, pass 4: rows of the forward transform; odd bins (pairs f, D-1-f)
__global__ void __launch_bounds__(256) k_sbf_build_rows2(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int j = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, D = 1 << logD, hD = D >> 1;
    const int M1 = 1 << A.logM1, logM2 = A.logM2, M2 = 1 << logM2, cb = A.cb, hc = cb >> 1;
    const int p0 = blockIdx.x * hc;   // first row pair {p, M1 - 1 - p}
    double2 *ps = A.pspec + q * A.ps_q + (size_t)j * (2 * D + 1);
    if (zcold(A.zp, A.zq0, 2L * D, q, j)) {   // x^{2D}: odd bins of spec2 are -1
        for (int e = threadIdx.x; e < hc * M2; e += blockDim.x) {
            const int fa = p0 + e % hc + M1 * (e / hc);
            const int f = fa < hD ? fa : D - 1 - fa;
            ps[2 * f + 1] = make_double2(-1.0, 0.0);
            ps[2 * (D - 1 - f) + 1] = make_double2(-1.0, 0.0);
        }
        return;
    }
    const double2 *src = A.scratch + ((size_t)q * A.nreal_p + j) * D;
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int c = e % cb, s = e / cb;
        sx[c * M2 + s] = src[(long)bitrev(s, logM2) * M1 + slot_rev(p0 + (c >> 1), c & 1, M1)];
    }
    __syncthreads();
    smem_fft_dit<-1>(sx, logM2, cb, A.tw, A.logTW);
    const double kb = 1.0 / (4.0 * D);
    for (int e = threadIdx.x; e < hc * M2; e += blockDim.x) {
        const int cp = e % hc, k2 = e / hc;
        const int fa = p0 + cp + M1 * k2;
        const double2 za = sx[(2 * cp) * M2 + k2];                // bin fa
        const double2 zb = sx[(2 * cp + 1) * M2 + (M2 - 1 - k2)];   // bin D - 1 - fa
        int f;
        double2 a, b;
        if (fa < hD) { f = fa; a = za; b = cconj(zb); }
        else { f = D - 1 - fa; a = zb; b = cconj(za); }
        double2 Hf, Hc;
        mirror_out_pair(a, b, kb, tw_tangent(A.tw, A.logTW), (long)(2 * f + 1) << (A.logTW - logD - 2), A.logTW, Hf,
                        Hc);
        ps[2 * f + 1] = Hf;
        ps[2 * (D - 1 - f) + 1] = Hc;
    }
}

// ---- propagate: the inverse half-bin input of child c at bins f, h-1-f
// (mirror pair), from the parent's g spectrum and the sibling's spectrum
__device__ __forceinline__ void sbf_prop_input(const SbfArgs &A, int q, int c, int f, double2 &xf, double2 &xfp) {
    const int D = 1 << A.logD, h = D >> 1, fp = h - 1 - f;
    const int j = c >> 1, sib = c ^ 1;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *G = A.Gp + q * A.Gp_q + (size_t)j * (D + 1);
    const bool has_sib = sib < A.nreal_c;
    const double2 *S = A.cspec + q * A.cs_q + (size_t)sib * (D + 1);
    const double2 Y1 = cmulc(G[2 * f + 1], has_sib ? S[2 * f + 1] : one);
    const double2 Y2 = cconj(cmulc(G[2 * fp + 1], has_sib ? S[2 * fp + 1] : one));
    mirror_inv_input(cadd(Y1, Y2), csub(Y1, Y2), tw_tangent(A.tw, A.logTW), (long)(2 * f + 1) << (A.logTW - A.logD - 1),
                     A.logTW, xf, xfp);
}

// ---- propagate: child c's g spectrum bins f and h-f (f <= h/2) from the
// forward transform values z_f, z_{(h-f) mod h}
__device__ __forceinline__ void sbf_prop_output(const SbfArgs &A, int q, int c, int f, double2 zf0, double2 zc0,
                                                double2 *out) {
    const int D = 1 << A.logD, h = D >> 1, fp = h - f;
    const int j = c >> 1, sib = c ^ 1;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *G = A.Gp + q * A.Gp_q + (size_t)j * (D + 1);
    const bool has_sib = sib < A.nreal_c;
    const double2 *S = A.cspec + q * A.cs_q + (size_t)sib * (D + 1);
    const double2 zf = zf0, zc = cconj(zc0);
    const double2 E = cadd(zf, zc);
    double r;   // T = r u = -i (zf - zc) e^{-2 pi i f/D}
    const double2 u =
        tanmul_t<-1>(cmul_mi(csub(zf, zc)), tw_tangent(A.tw, A.logTW), (long)f << (A.logTW - A.logD), A.logTW, &r);
    const double kx = 1.0 / (8.0 * h);
    const double2 Yf = cmulc(G[2 * f], has_sib ? S[2 * f] : one);
    const double2 Xf = make_double2(fma(r, u.x, E.x), fma(r, u.y, E.y));
    out[f] = make_double2(fma(kx, Xf.x, 0.5 * Yf.x), fma(kx, Xf.y, 0.5 * Yf.y));
    if (fp != f) {
        const double2 Yc = cmulc(G[2 * fp], has_sib ? S[2 * fp] : one);
        const double2 Xc = make_double2(fma(-r, u.x, E.x), fma(r, u.y, -E.y));   // conj(E - T)
        out[fp] = make_double2(fma(kx, Xc.x, 0.5 * Yc.x), fma(kx, Xc.y, 0.5 * Yc.y));
    }
}

// ---- propagate, children with h <= kSmemFftMax: the whole child in one CTA
__global__ void __launch_bounds__(512) k_sbf_prop_one(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int c = blockIdx.x, q = blockIdx.y;
    const int logD = A.logD, D = 1 << logD, h = D >> 1, lh = logD - 1;
    if (zcold(A.zp, A.zq0, D, q, c)) return;   // wholly zero: never read
    double2 *out = A.Gout + q * A.Go_q + (size_t)c * (h + 1);
    if (A.hot_c && !A.hot_c[c]) {               // subset-cold child: zero g spectrum
        for (int f = threadIdx.x; f <= h; f += blockDim.x) out[f] = make_double2(0.0, 0.0);
        return;
    }
    for (int f = threadIdx.x; f < (h >> 1); f += blockDim.x) {
        double2 xf, xfp;
        sbf_prop_input(A, q, c, f, xf, xfp);
        sx[bitrev(f, lh)] = xf;
        sx[bitrev(h - 1 - f, lh)] = xfp;
    }
    __syncthreads();
    smem_fft_dit<+1>(sx, lh, 1, A.tw, A.logTW);
    // the untwist e^{+2 pi i s/D} is the forward transform's half shift by -1/2 bin
    smem_bitrev_map(sx, lh, 1, [](int, int, double2 v) { return v; });
    smem_fft_dit<-1, -1>(sx, lh, 1, A.tw, A.logTW);
    for (int f = threadIdx.x; f <= (h >> 1); f += blockDim.x)
        sbf_prop_output(A, q, c, f, sx[f & (h - 1)], sx[(h - f) & (h - 1)], out);
}

// ---- propagate (h > kSmemFftMax), pass 1: columns of the inverse half-bin input
__global__ void __launch_bounds__(256) k_sbf_prop_cols(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int c = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, D = 1 << logD, h = D >> 1, logh = logD - 1;
    const int logM1 = A.logM1, M1 = 1 << logM1, M2 = 1 << A.logM2, cb = A.cb, hc = cb >> 1;
    if (zcold(A.zp, A.zq0, D, q, c) || (A.hot_c && !A.hot_c[c])) return;
    const int p0 = blockIdx.x * hc;   // first column pair {p, M2 - 1 - p}
    for (int e = threadIdx.x; e < hc * M1; e += blockDim.x) {
        const int cp = e % hc, r = e / hc;   // neighbouring threads: neighbouring columns
        const int fa = r * M2 + p0 + cp;   // its mirror h - 1 - fa: column M2 - 1 - p, row M1 - 1 - r
        const int f = (r < (M1 >> 1)) ? fa : h - 1 - fa;
        double2 xf, xfp;
        sbf_prop_input(A, q, c, f, xf, xfp);
        const int pa = (2 * cp) * M1 + (int)bitrev(r, logM1);
        const int pb = (2 * cp + 1) * M1 + (int)bitrev(M1 - 1 - r, logM1);
        if (f == fa) { sx[pa] = xf; sx[pb] = xfp; }
        else { sx[pa] = xfp; sx[pb] = xf; }
    }
    __syncthreads();
    smem_fft_dit<+1>(sx, logM1, cb, A.tw, A.logTW);
    double2 *dst = A.scratch + ((size_t)q * A.nreal_c + c) * h;
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int cc = e >> logM1, k1 = e & (M1 - 1);
        const int n2 = slot_rev(p0 + (cc >> 1), cc & 1, M2);
        const int t = (n2 * k1) & (h - 1);
        double2 v = sx[e];
        if (t) v = twmul<+1>(v, __ldg(&A.tw[(long)t << (A.logTW - logh)]));
        dst[(long)n2 * M1 + k1] = v;
    }
}

// ---- propagate, pass 2: rows into buf (the untwist e^{+2 pi i s/D} is the
// next column pass's half shift by -1/2 bin)
__global__ void __launch_bounds__(256) k_sbf_prop_rows1(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int c = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, h = 1 << (logD - 1);
    const int M1 = 1 << A.logM1, logM2 = A.logM2, M2 = 1 << logM2, cb = A.cb;
    if (zcold(A.zp, A.zq0, 1L << logD, q, c) || (A.hot_c && !A.hot_c[c])) return;
    const int k10 = blockIdx.x * cb;
    const size_t item = (size_t)q * A.nreal_c + c;
    const double2 *src = A.scratch + item * h;
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int cc = e % cb, s = e / cb;
        sx[cc * M2 + s] = src[(long)bitrev(s, logM2) * M1 + k10 + cc];
    }
    __syncthreads();
    smem_fft_dit<+1>(sx, logM2, cb, A.tw, A.logTW);
    double2 *x = A.buf + item * h;
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int cc = e % cb, k2 = e / cb;
        x[k2 * M1 + k10 + cc] = sx[cc * M2 + k2];
    }
}

// ---- propagate, pass 4: rows of the forward transform; child g spectrum (pairs f, h-f)
__global__ void __launch_bounds__(256) k_sbf_prop_rows2(SbfArgs A) {
    extern __shared__ double2 sx[];
    const int c = blockIdx.y, q = blockIdx.z;
    const int logD = A.logD, h = 1 << (logD - 1);
    const int logM1 = A.logM1, M1 = 1 << logM1, logM2 = A.logM2, M2 = 1 << logM2, cb = A.cb;
    if (zcold(A.zp, A.zq0, 1L << logD, q, c)) return;
    const int s0 = blockIdx.x * (cb >> 1);   // first row slot: {0, M1/2}, {p, M1 - p}
    const int nitems = (cb >> 1) * M2 + (s0 == 0 ? 1 : 0);
    double2 *out = A.Gout + q * A.Go_q + (size_t)c * (h + 1);
    if (A.hot_c && !A.hot_c[c]) {   // subset-cold child: zero g spectrum over this CTA's bins
        for (int e = threadIdx.x; e < nitems; e += blockDim.x) {
            int c0, r0, c1, r1;
            mirror_item(e, s0, cb >> 1, logM2, c0, r0, c1, r1);
            const int fa = slot_mirror(s0 + (c0 >> 1), c0 & 1, M1) + M1 * r0;
            const int f = min(fa, h - fa);
            out[f] = make_double2(0.0, 0.0);
            out[h - f] = make_double2(0.0, 0.0);
        }
        return;
    }
    const double2 *src = A.scratch + ((size_t)q * A.nreal_c + c) * h;
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int cc = e % cb, s = e / cb;
        sx[cc * M2 + s] = src[(long)bitrev(s, logM2) * M1 + slot_mirror(s0 + (cc >> 1), cc & 1, M1)];
    }
    __syncthreads();
    smem_fft_dit<-1>(sx, logM2, cb, A.tw, A.logTW);
    for (int e = threadIdx.x; e < nitems; e += blockDim.x) {
        // rows: slot 0 row 0 pairs k2 with (M2 - k2) mod M2 (bin 0 with bin h),
        // slot 0 row M1/2 pairs k2 with M2 - 1 - k2, row p with row M1 - p
        int c0, r0, c1, r1;
        mirror_item(e, s0, cb >> 1, logM2, c0, r0, c1, r1);
        const int fa = slot_mirror(s0 + (c0 >> 1), c0 & 1, M1) + M1 * r0;
        const double2 za = sx[c0 * M2 + r0];
        const double2 zb = (c1 >= 0) ? sx[c1 * M2 + (r1 & (M2 - 1))] : za;   // bin (h - fa) mod h
        if (fa <= h - fa) sbf_prop_output(A, q, c, fa, za, zb, out);
        else sbf_prop_output(A, q, c, h - fa, zb, za, out);
    }
}

// ------------------------------------------------------------ launchers
// four-step split of 2^logM points and its columns / rows per CTA: 4096
// points' worth, fewer on short grids, at least 2 where lines go in mirror pairs
static void sbf_split(int logM, long items, int &logM1, int &logM2, int &cbA, int &cbB, bool pairsA, bool pairsB) {
    logM1 = (logM + 1) / 2;
    logM2 = logM - logM1;
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    const int it = (int)std::min<long>(items, 1L << 30);
    cbA = short_grid_cb(std::max(1, std::min(M2, 4096 / M1)), M2, it);
    cbB = short_grid_cb(std::max(1, std::min(M1, 4096 / M2)), M1, it);
    if (pairsA) cbA = std::max(cbA, 2);
    if (pairsB) cbB = std::max(cbB, 2);
}

void launch_specbig_build(const Level &c, const Level &p, bool write_coeffs, int nq, double2 *buf, double2 *scratch,
                          const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr, const int *zp,
                          int zq0) {
    const int logD = ilog2b(c.deg), D = 1 << logD;
    const long items = (long)nq * p.nreal;
    const double pts = (double)items * D;
    SbfArgs A{};
    A.cspec = c.spec2;
    A.cs_q = c.spec2_q;
    A.cends = c.ends;
    A.ce_q = c.ends_q;
    A.nreal_c = c.nreal;
    A.nreal_p = p.nreal;
    A.pspec = p.spec2;
    A.ps_q = p.spec2_q;
    A.pends = p.spec2 ? p.ends : nullptr;
    A.pe_q = p.ends_q;
    A.Pout = write_coeffs ? p.P : nullptr;
    A.Po_q = p.P_q;
    A.pst_p = p.pst;
    A.plen_p = p.plen;
    A.logD = logD;
    A.buf = buf;
    A.scratch = scratch;
    A.tw = tw;
    A.logTW = logTW;
    A.zp = zp;
    A.zq0 = zq0;
    int cbA, cbB;
    sbf_split(logD, items, A.logM1, A.logM2, cbA, cbB, true, true);
    const int M1 = 1 << A.logM1, M2 = 1 << A.logM2;
    const int cbR = short_grid_cb(std::max(1, std::min(M1, 4096 / M2)), M1, (int)std::min<long>(items, 1L << 30));
    A.cb = cbA;
    pr->begin("specbig_build", pts * 10.0 + (5.0 * A.logM1 + 6.0) * pts, st);
    k_sbf_build_cols<<<dim3(M2 / cbA, p.nreal, nq), 256, (size_t)cbA * M1 * sizeof(double2), st>>>(A);
    pr->end(st);
    A.cb = cbR;
    pr->begin("specbig_build", 5.0 * A.logM2 * pts + pts * 4.0, st);
    k_sbf_build_rows1<<<dim3(M1 / cbR, p.nreal, nq), 256, (size_t)cbR * M2 * sizeof(double2), st>>>(A);
    pr->end(st);
    *launches += 2;
    if (!p.spec2) return;
    FftSkip sk;
    sk.zp = zp;
    sk.q0 = zq0;
    sk.span = p.deg;
    sk.per_q = p.nreal;
    launch_fft4_cols(buf, scratch, items, logD, -1, tw, logTW, st, launches, pr, sk, +1);   // half-shifted
    A.cb = cbB;
    pr->begin("specbig_build", 5.0 * A.logM2 * pts + pts * 8.0, st);
    k_sbf_build_rows2<<<dim3(M1 / cbB, p.nreal, nq), 256, (size_t)cbB * M2 * sizeof(double2), st>>>(A);
    pr->end(st);
    *launches += 1;
}

void launch_specbig_prop(const double2 *Gp, size_t Gp_q, const Level &c, int nq, const uint8_t *hot_c, double2 *buf,
                         double2 *scratch, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                         const int *zp, int zq0) {
    const int logD = ilog2b(c.deg), D = 1 << logD, h = D / 2, logh = logD - 1;
    const long items = (long)nq * c.nreal;
    const double pts = (double)items * h;
    SbfArgs A{};
    A.cspec = c.spec2;
    A.cs_q = c.spec2_q;
    A.nreal_c = c.nreal;
    A.Gp = Gp;
    A.Gp_q = Gp_q;
    A.Gout = c.G;
    A.Go_q = c.G_q;
    A.hot_c = hot_c;
    A.logD = logD;
    A.buf = buf;
    A.scratch = scratch;
    A.tw = tw;
    A.logTW = logTW;
    A.zp = zp;
    A.zq0 = zq0;
    if (h <= kSmemFftMax) {   // one CTA per child
        const size_t smem = (size_t)h * sizeof(double2);
        pr->begin("specbig_prop", pts * 28.0 + 10.0 * logh * pts, st);
        k_sbf_prop_one<<<dim3(c.nreal, nq), smem > kOneCtaSmem ? 512 : 256, smem, st>>>(A);
        pr->end(st);
        *launches += 1;
        return;
    }
    int cbA, cbB;
    sbf_split(logh, items, A.logM1, A.logM2, cbA, cbB, true, true);
    const int M1 = 1 << A.logM1, M2 = 1 << A.logM2;
    const int cbR = short_grid_cb(std::max(1, std::min(M1, 4096 / M2)), M1, (int)std::min<long>(items, 1L << 30));
    A.cb = cbA;
    pr->begin("specbig_prop", pts * 10.0 + (5.0 * A.logM1 + 6.0) * pts, st);
    k_sbf_prop_cols<<<dim3(M2 / cbA, c.nreal, nq), 256, (size_t)cbA * M1 * sizeof(double2), st>>>(A);
    pr->end(st);
    A.cb = cbR;
    pr->begin("specbig_prop", 5.0 * A.logM2 * pts + pts * 4.0, st);
    k_sbf_prop_rows1<<<dim3(M1 / cbR, c.nreal, nq), 256, (size_t)cbR * M2 * sizeof(double2), st>>>(A);
    pr->end(st);
    FftSkip sk;
    sk.zp = zp;
    sk.q0 = zq0;
    sk.span = c.deg;
    sk.per_q = c.nreal;
    launch_fft4_cols(buf, scratch, items, logh, -1, tw, logTW, st, launches, pr, sk, -1);   // half-shifted
    A.cb = cbB;
    pr->begin("specbig_prop", 5.0 * A.logM2 * pts + pts * 14.0, st);
    k_sbf_prop_rows2<<<dim3(M1 / cbB, c.nreal, nq), 256, (size_t)cbB * M2 * sizeof(double2), st>>>(A);
    pr->end(st);
    *launches += 3;
}

void specbig_set_smem_limits() {
    const int four = 4096 * (int)sizeof(double2), one = kSmemFftMax * (int)sizeof(double2);
    cudaFuncSetAttribute(k_sbf_build_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_build_rows1, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_build_rows2, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_prop_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_prop_rows1, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_prop_rows2, cudaFuncAttributeMaxDynamicSharedMemorySize, four);
    cudaFuncSetAttribute(k_sbf_prop_one, cudaFuncAttributeMaxDynamicSharedMemorySize, one);
}

void launch_gspecbig_init(const double *g, size_t g_q, int gst, int glen, int nreal, int logd, double2 *G, size_t G_q,
                          int nq, const uint8_t *hot, double2 *buf, double2 *scratch, const double2 *tw, int logTW,
                          cudaStream_t st, long *launches, Prof *pr, const int *zp, int zq0) {
    const int h = 1 << (logd - 1);
    const long items = (long)nq * nreal;
    FftSkip sk;
    sk.zp = zp;
    sk.q0 = zq0;
    sk.span = 1L << logd;
    sk.per_q = nreal;
    pr->begin("gspec_init", 0.0, st);
    k_sb_gpack<<<dim3(nb((long)nreal * h, 256), nq), 256, 0, st>>>(g, g_q, gst, glen, nreal, logd, buf, zp, zq0);
    pr->end(st);
    fft_batched(buf, scratch, items, logd - 1, -1, tw, logTW, st, launches, pr, sk);
    pr->begin("gspec_init", (double)items * h * 20.0, st);
    k_sb_gpost<<<dim3(nb((long)nreal * h, 256), nq), 256, 0, st>>>(nreal, logd, buf, G, G_q, hot, tw, logTW, zp, zq0);
    pr->end(st);
    *launches += 2;
}

}  // namespace icmg
