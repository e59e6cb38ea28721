// spectral_big.cu -- spectral tree levels whose transforms exceed one CTA's
// shared memory (child degree D > kSpecMaxD).  Same arithmetic as
// spectral.cu (see the formulas there), with the pointwise phases as
// separate kernels over global buffers and the transforms done by the
// batched four-step FFT (fft_batched).  These are the top one or two levels
// of a large tree: few nodes per quadrature node, so the extra passes over
// memory are small next to the FP64 work.
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
__device__ __forceinline__ double2 twb(const double2 *__restrict__ tw, long idx) { return __ldg(&tw[idx]); }
// tree node `node` of chunk node q lies wholly inside the zero prefix
__device__ __forceinline__ bool zcold(const int *__restrict__ zp, int zq0, long span, int q, long node) {
    return zp && (node + 1) * span <= (long)zp[zq0 + q];
}

// ---- build: 1. even bins of spec2(X) and the inverse input U (mirror pairs)
__global__ void k_sb_build1(const double2 *__restrict__ cspec, size_t cs_q, int nreal_c, int nreal_p, int logD,
                            double2 *__restrict__ pspec, size_t ps_q, double2 *__restrict__ buf,
                            const double2 *__restrict__ tw, int logTW, const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << logD, hD = D >> 1, np1 = hD + 1;
    const int j = (int)(idx / np1), f = (int)(idx % np1);
    if (j >= nreal_p) return;
    if (zcold(zp, zq0, 2L * D, q, j)) {   // x^{2D}: even bins of spec2 are 1
        if (pspec) {
            double2 *ps = pspec + q * ps_q + (size_t)j * (2 * D + 1);
            ps[2 * f] = make_double2(1.0, 0.0);
            ps[2 * (D - f)] = make_double2(1.0, 0.0);
        }
        return;
    }
    const double2 one = make_double2(1.0, 0.0);
    const double2 *sL = cspec + q * cs_q + (size_t)(2 * j) * (D + 1);
    const bool has_r = (2 * j + 1) < nreal_c;
    const double2 *sR = sL + (D + 1);
    const double2 Cf = cmul(sL[f], has_r ? sR[f] : one);
    const double2 Cc = cmul(sL[D - f], has_r ? sR[D - f] : one);
    if (pspec) {
        double2 *ps = pspec + q * ps_q + (size_t)j * (2 * D + 1);
        ps[2 * f] = Cf;
        ps[2 * (D - f)] = Cc;
    }
    double2 E = cadd(Cf, cconj(Cc)), Dd = csub(Cf, cconj(Cc));
    if (f == 0) { E.y = 0.0; Dd.y = 0.0; }
    const double2 O = (f == 0) ? Dd : cmulc(Dd, twb(tw, (long)f << (logTW - logD - 1)));
    double2 *u = buf + ((size_t)q * nreal_p + j) * D;
    u[f] = cadd(E, cmul_pi(O));
    if (f != 0 && f != hD) u[D - f] = cadd(cconj(E), cmul_pi(cconj(O)));
}

// ---- build: 2. coefficients / ends / endpoint fix / twist, in place
__global__ void k_sb_build2(const double *__restrict__ cends, size_t ce_q, int nreal_c, int nreal_p, int logD,
                            double *__restrict__ pends, size_t pe_q, double *__restrict__ Pout, size_t Po_q,
                            int pst_p, int plen_p, double2 *__restrict__ buf, const double2 *__restrict__ tw,
                            int logTW, const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << logD;
    const int j = (int)(idx >> logD), s = (int)(idx & (D - 1));
    if (j >= nreal_p) return;
    if (zcold(zp, zq0, 2L * D, q, j)) {   // x^{2D}: coefficients and ends
        if (Pout) {
            double *out = Pout + q * Po_q + (size_t)j * pst_p;
            if (2 * s < pst_p) out[2 * s] = 0.0;
            if (2 * s + 1 < pst_p) out[2 * s + 1] = 0.0;
            if (s == 0) {
                if (2 * D < pst_p) out[2 * D] = (2 * D < plen_p) ? 1.0 : 0.0;
                for (int t = 2 * D + 1; t < pst_p; ++t) out[t] = 0.0;
            }
        }
        if (s == 0 && pends) {
            double *en = pends + q * pe_q + (size_t)j * 2;
            en[0] = 0.0;
            en[1] = 1.0;
        }
        return;
    }
    double2 *up = buf + ((size_t)q * nreal_p + j) * D + s;
    double2 u = *up;
    const double *eL = cends + q * ce_q + (size_t)(2 * j) * 2;
    const bool has_r = (2 * j + 1) < nreal_c;
    const double xtop = eL[1] * (has_r ? eL[3] : 0.0);
    const double inv2D = 1.0 / (2.0 * D);
    if (Pout) {   // truncated at plen_p; the row's padding up to pst_p is zero
        double *out = Pout + q * Po_q + (size_t)j * pst_p;
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
        if (pends) {
            double *en = pends + q * pe_q + (size_t)j * 2;
            en[0] = x0;
            en[1] = xtop;
        }
        u.x = (x0 - xtop) * (2.0 * D);
        *up = u;
    } else {
        *up = cmul(u, twb(tw, (long)s << (logTW - logD - 1)));
    }
}

// ---- build: 3. odd bins from the forward transform (mirror pairs f, D-1-f)
__global__ void k_sb_build3(int nreal_p, int logD, double2 *__restrict__ pspec, size_t ps_q,
                            const double2 *__restrict__ buf, const double2 *__restrict__ tw, int logTW,
                            const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << logD, hD = D >> 1;
    const int j = (int)(idx / hD), f = (int)(idx % hD);
    if (j >= nreal_p) return;
    if (zcold(zp, zq0, 2L * D, q, j)) {   // x^{2D}: odd bins of spec2 are -1
        double2 *ps = pspec + q * ps_q + (size_t)j * (2 * D + 1);
        ps[2 * f + 1] = make_double2(-1.0, 0.0);
        ps[2 * (D - 1 - f) + 1] = make_double2(-1.0, 0.0);
        return;
    }
    const double2 *c = buf + ((size_t)q * nreal_p + j) * D;
    const double2 a = c[f], b = cconj(c[D - 1 - f]);
    const double2 Ep = cadd(a, b);
    const double2 T = cmul(cmul_mi(csub(a, b)), twb(tw, (long)(2 * f + 1) << (logTW - logD - 2)));
    const double kb = 1.0 / (4.0 * D);
    double2 *ps = pspec + q * ps_q + (size_t)j * (2 * D + 1);
    ps[2 * f + 1] = cscale(cadd(Ep, T), kb);
    ps[2 * (D - 1 - f) + 1] = cscale(cconj(csub(Ep, T)), kb);
}

// ---- propagate (children get g spectra): 1. inverse half-bin input per child
__global__ void k_sb_prop1(const double2 *__restrict__ Gp, size_t Gp_q, const double2 *__restrict__ cspec,
                           size_t cs_q, int nreal_c, int logD, double2 *__restrict__ buf,
                           const uint8_t *__restrict__ hot_c, const double2 *__restrict__ tw, int logTW,
                           const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << logD, h = D >> 1, hp = (h + 1) >> 1;
    const int c = (int)(idx / hp), f = (int)(idx % hp);
    if (c >= nreal_c || (hot_c && !hot_c[c])) return;   // cold: output zeroed in pass 3
    if (zcold(zp, zq0, D, q, c)) return;                 // wholly zero: never read
    const int fp = h - 1 - f;
    const int j = c >> 1, sib = c ^ 1;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *G = Gp + q * Gp_q + (size_t)j * (D + 1);
    const bool has_sib = sib < nreal_c;
    const double2 *S = cspec + q * cs_q + (size_t)sib * (D + 1);
    const double2 Y1 = cmulc(G[2 * f + 1], has_sib ? S[2 * f + 1] : one);
    const double2 Y2 = cconj(cmulc(G[2 * fp + 1], has_sib ? S[2 * fp + 1] : one));
    const double2 A = cadd(Y1, Y2);
    const double2 B = cmulc(csub(Y1, Y2), twb(tw, (long)(2 * f + 1) << (logTW - logD - 1)));
    double2 *x = buf + ((size_t)q * nreal_c + c) * h;
    x[f] = cadd(A, cmul_pi(B));
    if (fp != f) x[fp] = cadd(cconj(A), cmul_pi(cconj(B)));
}

// ---- propagate: 2. untwist in place (unscaled)
__global__ void k_sb_prop2(int nreal_c, int logD, double2 *__restrict__ buf, const double2 *__restrict__ tw,
                           int logTW, const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = 1 << (logD - 1);
    const int c = (int)(idx >> (logD - 1)), s = (int)(idx & (h - 1));
    if (c >= nreal_c || s == 0 || zcold(zp, zq0, 1L << logD, q, c)) return;
    double2 *x = buf + ((size_t)q * nreal_c + c) * h + s;
    *x = cmulc(*x, twb(tw, (long)s << (logTW - logD)));
}

// ---- propagate: 3. child g spectra (mirror pairs f, h-f)
__global__ void k_sb_prop3(const double2 *__restrict__ Gp, size_t Gp_q, const double2 *__restrict__ cspec,
                           size_t cs_q, int nreal_c, int logD, const double2 *__restrict__ buf,
                           double2 *__restrict__ Gout, size_t Go_q, const uint8_t *__restrict__ hot_c,
                           const double2 *__restrict__ tw, int logTW, const int *__restrict__ zp, int zq0) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << logD, h = D >> 1, hq = (h >> 1) + 1;
    const int c = (int)(idx / hq), f = (int)(idx % hq);
    if (c >= nreal_c || zcold(zp, zq0, D, q, c)) return;
    const int fp = h - f;
    double2 *out = Gout + q * Go_q + (size_t)c * (h + 1);
    if (hot_c && !hot_c[c]) {
        out[f] = make_double2(0.0, 0.0);
        out[fp] = make_double2(0.0, 0.0);
        return;
    }
    const int j = c >> 1, sib = c ^ 1;
    const double2 one = make_double2(1.0, 0.0);
    const double2 *G = Gp + q * Gp_q + (size_t)j * (D + 1);
    const bool has_sib = sib < nreal_c;
    const double2 *S = cspec + q * cs_q + (size_t)sib * (D + 1);
    const double2 *z = buf + ((size_t)q * nreal_c + c) * h;
    const double2 zf = z[f & (h - 1)], zc = cconj(z[fp & (h - 1)]);
    const double2 E = cadd(zf, zc);
    const double2 T = (f == 0) ? cmul_mi(csub(zf, zc)) : cmul(cmul_mi(csub(zf, zc)), twb(tw, (long)f << (logTW - logD)));
    const double kx = 1.0 / (8.0 * h);
    const double2 Yf = cmulc(G[2 * f], has_sib ? S[2 * f] : one);
    const double2 Xf = cadd(E, T);
    out[f] = make_double2(fma(kx, Xf.x, 0.5 * Yf.x), fma(kx, Xf.y, 0.5 * Yf.y));
    if (fp != f) {
        const double2 Yc = cmulc(G[2 * fp], has_sib ? S[2 * fp] : one);
        const double2 Xc = cconj(csub(E, T));
        out[fp] = make_double2(fma(kx, Xc.x, 0.5 * Yc.x), fma(kx, Xc.y, 0.5 * Yc.y));
    }
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
    const double2 Ev = cscale(cadd(zf, cconj(zc)), 0.5);
    const double2 Od = cscale(cmul_mi(csub(zf, cconj(zc))), 0.5);
    out[f] = cadd(Ev, cmul(Od, twb(tw, (long)f << (logTW - logd))));
    if (f == 0) out[h] = csub(Ev, Od);
}

// ------------------------------------------------------------ launchers
void launch_specbig_build(const Level &c, const Level &p, bool write_coeffs, int nq, double2 *buf, double2 *scratch,
                          const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr, const int *zp,
                          int zq0) {
    const int logD = ilog2b(c.deg), D = 1 << logD;
    const long items = (long)nq * p.nreal;
    const double pts = (double)items * D;
    FftSkip sk;
    sk.zp = zp;
    sk.q0 = zq0;
    sk.span = p.deg;
    sk.per_q = p.nreal;
    pr->begin("specbig_build", pts * 10.0, st);
    k_sb_build1<<<dim3(nb((long)p.nreal * (D / 2 + 1), 256), nq), 256, 0, st>>>(
        c.spec2, c.spec2_q, c.nreal, p.nreal, logD, p.spec2, p.spec2_q, buf, tw, logTW, zp, zq0);
    pr->end(st);
    fft_batched(buf, scratch, items, logD, +1, tw, logTW, st, launches, pr, sk);
    pr->begin("specbig_build", pts * 4.0, st);
    k_sb_build2<<<dim3(nb((long)p.nreal * D, 256), nq), 256, 0, st>>>(
        c.ends, c.ends_q, c.nreal, p.nreal, logD, p.spec2 ? p.ends : nullptr, p.ends_q, write_coeffs ? p.P : nullptr,
        p.P_q, p.pst, p.plen, buf, tw, logTW, zp, zq0);
    pr->end(st);
    *launches += 2;
    if (!p.spec2) return;
    fft_batched(buf, scratch, items, logD, -1, tw, logTW, st, launches, pr, sk);
    pr->begin("specbig_build", pts * 8.0, st);
    k_sb_build3<<<dim3(nb((long)p.nreal * (D / 2), 256), nq), 256, 0, st>>>(p.nreal, logD, p.spec2, p.spec2_q, buf,
                                                                          tw, logTW, zp, zq0);
    pr->end(st);
    *launches += 1;
}

void launch_specbig_prop(const double2 *Gp, size_t Gp_q, const Level &c, int nq, const uint8_t *hot_c, double2 *buf,
                         double2 *scratch, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                         const int *zp, int zq0) {
    const int logD = ilog2b(c.deg), D = 1 << logD, h = D / 2;
    const long items = (long)nq * c.nreal;
    const double pts = (double)items * h;
    FftSkip sk;
    sk.zp = zp;
    sk.q0 = zq0;
    sk.span = c.deg;
    sk.per_q = c.nreal;
    pr->begin("specbig_prop", pts * 10.0, st);
    k_sb_prop1<<<dim3(nb((long)c.nreal * ((h + 1) / 2), 256), nq), 256, 0, st>>>(
        Gp, Gp_q, c.spec2, c.spec2_q, c.nreal, logD, buf, hot_c, tw, logTW, zp, zq0);
    pr->end(st);
    fft_batched(buf, scratch, items, logD - 1, +1, tw, logTW, st, launches, pr, sk);
    pr->begin("specbig_prop", pts * 4.0, st);
    k_sb_prop2<<<dim3(nb((long)c.nreal * h, 256), nq), 256, 0, st>>>(c.nreal, logD, buf, tw, logTW, zp, zq0);
    pr->end(st);
    fft_batched(buf, scratch, items, logD - 1, -1, tw, logTW, st, launches, pr, sk);
    pr->begin("specbig_prop", pts * 14.0, st);
    k_sb_prop3<<<dim3(nb((long)c.nreal * (h / 2 + 1), 256), nq), 256, 0, st>>>(
        Gp, Gp_q, c.spec2, c.spec2_q, c.nreal, logD, buf, c.G, c.G_q, hot_c, tw, logTW, zp, zq0);
    pr->end(st);
    *launches += 3;
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
