// vjp_spec.cu -- adjoint passes of spectral tree levels (single VJP plans).
//
// A spectral level keeps, per node X of degree d, spec2(X) = DFT_{2d}(x) and
// the end coefficients (x_0, x_d) (spectral.cu); its g is kept as
// G = DFT_d(g).  For a parent X of degree 2D with children of degree D:
//
// upward (transpose of the propagate g_c[m] = sum_j g_X[m+j] P_sib[j]):
//   gbar_X = gbar_L P_R + gbar_R P_L has 2D coefficients (gbar_c has D), so
//   with the children's gbar spectra A_c = DFT_{2D}(gbar_c),
//   C = A_L S_R + A_R S_L is DFT_{2D}(gbar_X) exactly.  One inverse transform
//   of size D gives gbar_X (a real sequence of 2D through its even/odd
//   packing).  Where the level above is spectral too, the parent's own
//   A = DFT_{4D}(gbar_X) has C as its even bins and the half-bin transform of
//   gbar_X as its odd bins (a second transform of size D of the twisted
//   packing), as in the forward build, without the build's folded top
//   coefficient (gbar_X has none).
// downward (transpose of the build and of the propagate's sibling factor):
//   Pbar_L[i] = sum_m gbar_R[m] g_X[m+i] + sum_j Pbar_X[i+j] P_R[j], i <= D.
//   With G = DFT_{2D}(g_X) from the forward and PF = DFT_{2D}(Pbar_X folded,
//   Pbar_X[2D] added to Pbar_X[0]), y = IDFT_{2D}(G conj A_R + PF conj S_R)
//   equals Pbar_L[i] for 0 < i < D; at i = 0 and i = D the fold adds
//   Pbar_X[2D] P_R[0] and Pbar_X[0] P_R[D], taken off with the carried ends
//   of Pbar_X and the forward's ends of P_R.  Where the level below is
//   spectral, the child's PF = DFT_D(Pbar_L folded) is
//   (even bins of y's spectrum + DFT_D(a - b))/2 + delta with a = y[0:D),
//   b = y[D:2D): a - b from the odd bins by one inverse half-bin transform
//   (as in the forward propagate), delta = Pbar_L[0] + Pbar_L[D] - y[0],
//   y[0] = a[0] the mean of DFT_D(a) and y[D] = a[0] - (a - b)[0].  Where the
//   level below works on coefficients, Pbar_L[0..D] comes from one real
//   inverse of size 2D.
// A missing sibling is the polynomial 1 (spectrum 1, ends (1, 0)) with gbar
// 0.  Wholly-zero parents pass gbar 0 up; wholly-zero children are skipped
// on the way down (nothing reads their Pbar: their players' leaf factors are
// 0).  Children of degree up to kSpecMaxD (upward) or 2 kSpecMaxD (downward)
// run each step in one CTA; larger levels split the transforms in the
// four-step way through global memory (fft_batched) with pointwise kernels
// between them.
#include <algorithm>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"
#include "vjp.h"

namespace icmg {

namespace {
constexpr int kVspThreads = 256;
constexpr int kVspThreadsMax = 512;   // CTAs alone on an SM take twice the warps
constexpr int kVspPts = 4096;         // complex points per CTA of the one-CTA steps
constexpr int kVspMaxItems = 256;     // items per CTA (views staged in shared memory)
inline int vsp_tpb(size_t smem) { return smem > kOneCtaSmem ? kVspThreadsMax : kVspThreads; }
inline int ilog2v(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
inline unsigned nbv(long work, int threads) { return (unsigned)((work + threads - 1) / threads); }
inline int vsp_cb(int pts) { return std::min(kVspMaxItems, pts >= kVspPts ? 1 : kVspPts / pts); }
}  // namespace

// idx[0, nh) = items to compute, idx[nh, cnt) = wholly-zero ones, in order
__device__ __forceinline__ int vsp_partition(int *idx, int cnt, const ZeroPrefix &z, int q, int node0) {
    __shared__ int nh_s;
    if (threadIdx.x == 0) {
        int h = 0;
        for (int it = 0; it < cnt; ++it)
            if (!zp_cold(z, q, node0 + it)) idx[h++] = it;
        int c = h;
        for (int it = 0; it < cnt; ++it)
            if (zp_cold(z, q, node0 + it)) idx[c++] = it;
        nh_s = h;
    }
    __syncthreads();
    return nh_s;
}

// one child of the downward step: the operands of Z = G conj(A_sib) + PF conj(S_sib)
struct DnView {
    const double2 *G, *PF, *As, *Ss;   // null As: no sibling gbar; null Ss: sibling 1; null PF: Pbar_X = 0
    double pb0, pbt, ps0, psd;         // parent's Pbar ends, sibling's P ends
    double amb0, delta;                // (a - b)[0], the fold correction
    double2 pfh;                       // bin D/2 of the child's folded spectrum
    int c;
};

__device__ __forceinline__ DnView dn_view(const VspDownArgs &A, int q, int c) {
    const int D = 1 << A.logD;
    const int j = c >> 1, sib = c ^ 1;
    DnView v;
    v.c = c;
    v.G = A.G + q * A.G_q + (size_t)j * (D + 1);
    v.PF = A.PF ? A.PF + q * A.PF_q + (size_t)j * (D + 1) : nullptr;
    v.pb0 = A.PF ? A.Pe[q * A.Pe_q + (size_t)j * 2] : 0.0;
    v.pbt = A.PF ? A.Pe[q * A.Pe_q + (size_t)j * 2 + 1] : 0.0;
    const bool has_s = sib < A.nreal_c;
    v.As = has_s ? A.A + q * A.A_q + (size_t)sib * (D + 1) : nullptr;
    v.Ss = has_s ? A.S + q * A.S_q + (size_t)sib * (D + 1) : nullptr;
    v.ps0 = has_s ? A.E[q * A.E_q + (size_t)sib * 2] : 1.0;
    v.psd = has_s ? A.E[q * A.E_q + (size_t)sib * 2 + 1] : 0.0;
    v.amb0 = v.delta = 0.0;
    v.pfh = make_double2(0.0, 0.0);
    return v;
}

__device__ __forceinline__ double2 dn_z(const DnView &v, int F) {
    double2 z = v.As ? cmulc(v.G[F], v.As[F]) : make_double2(0.0, 0.0);
    if (v.PF) z = cadd(z, v.Ss ? cmulc(v.PF[F], v.Ss[F]) : v.PF[F]);
    return z;
}

// upward product C[f] and C[D - f] of parent j
__device__ __forceinline__ void up_pair(const VspUpArgs &A, int q, int j, int f, double2 &Cf, double2 &Cc) {
    const int D = 1 << A.logD;
    const double2 *aL = A.A + q * A.A_q + (size_t)(2 * j) * (D + 1);
    if (2 * j + 1 < A.nreal_c) {
        const double2 *aR = aL + (D + 1);
        const double2 *sL = A.S + q * A.S_q + (size_t)(2 * j) * (D + 1), *sR = sL + (D + 1);
        Cf = cadd(cmul(aL[f], sR[f]), cmul(aR[f], sL[f]));
        Cc = cadd(cmul(aL[D - f], sR[D - f]), cmul(aR[D - f], sL[D - f]));
    } else {   // lone child: the sibling is 1 with gbar 0
        Cf = aL[f];
        Cc = aL[D - f];
    }
}

// inverse input of a real sequence's spectrum C by mirror pairs (f, D - f):
// U(f) = E + i O, U(D - f) = conj(E) + i conj(O), E = C[f] + conj C[D-f],
// O = (C[f] - conj C[D-f]) e^{+2 pi i f/2D}; the unscaled inverse of size D
// is then 2D (x_{2s} + i x_{2s+1})
__device__ __forceinline__ void inv_input(double2 Cf, double2 Cc, int f, const double2 *__restrict__ tw, int logTW,
                                          int logD, double2 &Uf, double2 &Uc) {
    double2 E = cadd(Cf, cconj(Cc)), Dd = csub(Cf, cconj(Cc));
    if (f == 0) { E.y = 0.0; Dd.y = 0.0; }
    mirror_inv_input(E, Dd, tw_tangent(tw, logTW), (long)f << (logTW - logD - 1), logTW, Uf, Uc);
}

// odd bins of DFT_{4D} from the forward transform c of the twisted packing, mirror pair (f, D-1-f)
__device__ __forceinline__ void odd_bins(double2 a, double2 bc, int f, const double2 *__restrict__ tw, int logTW,
                                         int logD, double2 &Hf, double2 &Hc) {
    const double kb = 1.0 / (4.0 * (1 << logD));
    mirror_out_pair(a, cconj(bc), kb, tw_tangent(tw, logTW), (long)(2 * f + 1) << (logTW - logD - 2), logTW, Hf, Hc);
}

// ------------------------------------------------------------ one-CTA kernels
__device__ void vsp_real_body(const VspRealArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int M = 1 << A.logM;
    const int j0 = bx * A.cb;
    const int cnt = min(A.cb, A.nreal - j0);
    if (cnt <= 0) return;
    int *idx = reinterpret_cast<int *>(sm + (size_t)A.cb * M);
    const int nh = vsp_partition(idx, cnt, A.z, q, j0);
    for (int e = threadIdx.x; e < (cnt - nh) * (M + 1); e += blockDim.x) {   // wholly-zero nodes
        const int j = j0 + idx[nh + e / (M + 1)], f = e % (M + 1);
        A.out[q * A.o_q + (size_t)j * (M + 1) + f] = make_double2(0.0, 0.0);
        if (A.ends && f < 2) A.ends[q * A.e_q + (size_t)j * 2 + f] = 0.0;
    }
    if (nh == 0) return;
    for (int e = threadIdx.x; e < nh * M; e += blockDim.x) {
        const int it = e >> A.logM, r = e & (M - 1);
        const int s = (int)bitrev(r, A.logM);
        const double *x = A.x + q * A.x_q + (size_t)(j0 + idx[it]) * A.xst;
        const int t0 = 2 * s, t1 = 2 * s + 1;
        double v0 = t0 < A.xlen ? x[t0] : 0.0;
        if (s == 0 && A.fold && 2 * M < A.xlen) v0 += x[2 * M];
        sm[e] = make_double2(v0, t1 < A.xlen ? x[t1] : 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(sm, A.logM, nh, A.tw, A.logTW);
    // X[f] = (Z[f] + conj Z[M-f])/2 + e^{-2 pi i f/2M} (Z[f] - conj Z[M-f])/(2i),
    // by mirror pairs (f, M - f), f <= M/2
    const int mp = (M >> 1) + 1;
    for (int e = threadIdx.x; e < nh * mp; e += blockDim.x) {
        const int it = e / mp, f = e - it * mp;
        const int j = j0 + idx[it];
        const double2 *zz = sm + (size_t)it * M;
        const double2 zf = zz[f], zc = zz[(M - f) & (M - 1)];
        const double2 Ev = cadd(zf, cconj(zc)), Od = cmul_mi(csub(zf, cconj(zc)));   // both doubled
        double2 *out = A.out + q * A.o_q + (size_t)j * (M + 1);
        double2 Xf, Xc;
        half_sum_tw_pair(Ev, Od, tw_tangent(A.tw, A.logTW), (long)f << (A.logTW - A.logM - 1), A.logTW, Xf, Xc);
        out[f] = Xf;
        if (f != 0 && 2 * f != M) out[M - f] = Xc;
        if (f == 0) {
            out[M] = cscale(csub(Ev, Od), 0.5);
            if (A.ends) {
                const double *x = A.x + q * A.x_q + (size_t)j * A.xst;
                double *en = A.ends + q * A.e_q + (size_t)j * 2;
                en[0] = A.xlen > 0 ? x[0] : 0.0;
                en[1] = 2 * M < A.xlen ? x[2 * M] : 0.0;
            }
        }
    }
}

__device__ void vsp_up_body(const VspUpArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int D = 1 << A.logD, hD = D >> 1;
    const int j0 = bx * A.cb;
    const int cnt = min(A.cb, A.nreal_p - j0);
    if (cnt <= 0) return;
    int *idx = reinterpret_cast<int *>(sm + (size_t)A.cb * D);
    const int nh = vsp_partition(idx, cnt, A.z, q, j0);
    const int wz = A.Aout ? 2 * D + 1 : A.gst;
    for (int e = threadIdx.x; e < (cnt - nh) * wz; e += blockDim.x) {   // wholly-zero parents: gbar 0
        const int j = j0 + idx[nh + e / wz], t = e % wz;
        if (A.Aout) A.Aout[q * A.Ao_q + (size_t)j * (2 * D + 1) + t] = make_double2(0.0, 0.0);
        else A.gout[q * A.go_q + (size_t)j * A.gst + t] = 0.0;
    }
    if (nh == 0) return;
    // 1. C (the even bins of the parent's spectrum) and the inverse input
    const int np1 = hD + 1;
    for (int e = threadIdx.x; e < nh * np1; e += blockDim.x) {
        const int it = e / np1, f = e - it * np1;
        const int j = j0 + idx[it];
        double2 Cf, Cc, Uf, Uc;
        up_pair(A, q, j, f, Cf, Cc);
        if (A.Aout) {
            double2 *ao = A.Aout + q * A.Ao_q + (size_t)j * (2 * D + 1);
            ao[2 * f] = Cf;
            ao[2 * (D - f)] = Cc;
        }
        inv_input(Cf, Cc, f, A.tw, A.logTW, A.logD, Uf, Uc);
        double2 *u = sm + (size_t)it * D;
        u[bitrev(f, A.logD)] = Uf;
        if (f != 0 && f != hD) u[bitrev(D - f, A.logD)] = Uc;
    }
    __syncthreads();
    smem_fft_dit<+1>(sm, A.logD, nh, A.tw, A.logTW);
    const double inv2D = 1.0 / (2.0 * D);
    if (!A.Aout) {   // 2. coefficients, truncated at glen, zero to gst
        const int W = max(D, (A.gst + 1) / 2);
        for (int e = threadIdx.x; e < nh * W; e += blockDim.x) {
            const int it = e / W, s = e - it * W;
            double *go = A.gout + q * A.go_q + (size_t)(j0 + idx[it]) * A.gst;
            const double2 u = (s < D) ? sm[(size_t)it * D + s] : make_double2(0.0, 0.0);
            const int t0 = 2 * s, t1 = 2 * s + 1;
            if (t0 < A.gst) go[t0] = t0 < A.glen ? u.x * inv2D : 0.0;
            if (t1 < A.gst) go[t1] = t1 < A.glen ? u.y * inv2D : 0.0;
        }
        return;
    }
    // 3. odd bins: twisted packing (y_{2s} + i y_{2s+1}) e^{-2 pi i s/2D}, forward
    //    transform; the twist is the transform's half shift by +1/2 bin
    const double2 *tw = A.tw;
    const int logTW = A.logTW, logD = A.logD;
    smem_bitrev_map(sm, logD, nh, [](int, int, double2 v) { return v; });
    smem_fft_dit<-1, +1>(sm, logD, nh, tw, logTW);
    for (int e = threadIdx.x; e < nh * hD; e += blockDim.x) {
        const int it = e / hD, f = e - it * hD;
        const double2 *c = sm + (size_t)it * D;
        double2 Hf, Hc;
        odd_bins(c[f], c[D - 1 - f], f, tw, logTW, logD, Hf, Hc);
        double2 *ao = A.Aout + q * A.Ao_q + (size_t)(j0 + idx[it]) * (2 * D + 1);
        ao[2 * f + 1] = Hf;
        ao[2 * (D - 1 - f) + 1] = Hc;
    }
}

__device__ void vsp_down_body(const VspDownArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int D = 1 << A.logD, h = D >> 1, lh = A.logD - 1;
    const bool spec = A.PFout != nullptr;
    const int per = spec ? h : D;   // complex points per child
    const int c0 = bx * A.cb;
    const int cnt = min(A.cb, A.nreal_c - c0);
    if (cnt <= 0) return;
    DnView *V = reinterpret_cast<DnView *>(sm + (size_t)A.cb * per);
    int *idx = reinterpret_cast<int *>(V + A.cb);
    const int nh = vsp_partition(idx, cnt, A.z, q, c0);
    if (nh == 0) return;
    for (int it = threadIdx.x; it < nh; it += blockDim.x) V[it] = dn_view(A, q, c0 + idx[it]);
    __syncthreads();
    const double2 *tw = A.tw;
    const int logTW = A.logTW, logD = A.logD;
    if (!spec) {   // coefficients Pbar_c[0..D] from the real inverse of size 2D
        for (int e = threadIdx.x; e < nh * (h + 1); e += blockDim.x) {
            const int it = e / (h + 1), f = e - it * (h + 1);
            const DnView &v = V[it];
            double2 Uf, Uc;
            inv_input(dn_z(v, f), dn_z(v, D - f), f, tw, logTW, logD, Uf, Uc);
            double2 *u = sm + (size_t)it * D;
            u[bitrev(f, logD)] = Uf;
            if (f != 0 && f != h) u[bitrev(D - f, logD)] = Uc;
        }
        __syncthreads();
        smem_fft_dit<+1>(sm, logD, nh, tw, logTW);
        const double inv2D = 1.0 / (2.0 * D);
        const int W = max(h + 1, (A.pst + 1) / 2);   // entry pairs (2s, 2s + 1)
        for (int e = threadIdx.x; e < nh * W; e += blockDim.x) {
            const int it = e / W, s = e - it * W;
            const DnView &v = V[it];
            double *po = A.Pout + q * A.Po_q + (size_t)v.c * A.pst;
            double y0 = 0.0, y1 = 0.0;
            if (s <= h) {   // y_{2s}, y_{2s+1}; entry D = y_D, above D zero
                const double2 u = sm[(size_t)it * D + s];
                y0 = u.x * inv2D;
                y1 = (2 * s + 1 < D) ? u.y * inv2D : 0.0;
                if (s == 0) y0 -= v.pbt * v.ps0;
                if (2 * s == D) y0 -= v.pb0 * v.psd;
            }
            if (2 * s < A.pst) po[2 * s] = y0;
            if (2 * s + 1 < A.pst) po[2 * s + 1] = y1;
        }
        return;
    }
    // 1. odd bins of Z -> inverse half-bin input by mirror pairs (f, h-1-f)
    const int hp = (h + 1) >> 1;
    for (int e = threadIdx.x; e < nh * hp; e += blockDim.x) {
        const int it = e / hp, f = e - it * hp;
        const int fp = h - 1 - f;
        const DnView &v = V[it];
        const double2 Y1 = dn_z(v, 2 * f + 1);
        const double2 Y2 = cconj(dn_z(v, 2 * fp + 1));
        double2 Xf, Xc;   // A + i B, conj(A) + i conj(B), B = (Y1 - Y2) conj(w_f)
        mirror_inv_input(cadd(Y1, Y2), csub(Y1, Y2), tw_tangent(tw, logTW), (long)(2 * f + 1) << (logTW - logD - 1),
                         logTW, Xf, Xc);
        double2 *x = sm + (size_t)it * h;
        x[bitrev(f, lh)] = Xf;
        if (fp != f) x[bitrev(fp, lh)] = Xc;
    }
    __syncthreads();
    smem_fft_dit<+1>(sm, lh, nh, tw, logTW);
    // 2. untwist w_s = c'_s e^{+2 pi i s/D} (the forward transform's half shift
    //    by -1/2 bin), into bit-reversed order; (a - b)[0] = w_0.x / D
    const double invD = 1.0 / D;
    smem_bitrev_map(sm, lh, nh, [V, invD](int it, int s, double2 v) -> double2 {
        if (s == 0) V[it].amb0 = v.x * invD;
        return v;
    });
    smem_fft_dit<-1, -1>(sm, lh, nh, tw, logTW);
    // 3. DFT_D(a) = Z_even/2 + DFT_D(a - b)/2 by mirror pairs (f, h - f), in
    //    place (bin h beside the view)
    const double kx = 1.0 / (8.0 * h);
    const int hq = (h >> 1) + 1;
    for (int e = threadIdx.x; e < nh * hq; e += blockDim.x) {
        const int it = e / hq, f = e - it * hq;
        const int fp = h - f;
        DnView &v = V[it];
        double2 *zz = sm + (size_t)it * h;
        const double2 zf = zz[f & (h - 1)], zc = cconj(zz[fp & (h - 1)]);
        const double2 E = cadd(zf, zc);
        double r;   // T = r u = -i (zf - zc) e^{-2 pi i f/D}
        const double2 u =
            tanmul_t<-1>(cmul_mi(csub(zf, zc)), tw_tangent(tw, logTW), (long)f << (logTW - logD), logTW, &r);
        const double2 Yf = dn_z(v, 2 * f);
        const double2 Xf = make_double2(fma(r, u.x, E.x), fma(r, u.y, E.y));
        const double2 of = make_double2(fma(kx, Xf.x, 0.5 * Yf.x), fma(kx, Xf.y, 0.5 * Yf.y));
        if (fp != f) {
            const double2 Yc = dn_z(v, 2 * fp);
            const double2 Xc = make_double2(fma(-r, u.x, E.x), fma(r, u.y, -E.y));   // conj(E - T)
            const double2 oc = make_double2(fma(kx, Xc.x, 0.5 * Yc.x), fma(kx, Xc.y, 0.5 * Yc.y));
            if (fp == h) v.pfh = oc;
            else zz[fp] = oc;
        }
        zz[f] = of;
    }
    __syncthreads();
    // 4. a[0] = mean of DFT_D(a) (bins 0 and h once, 1..h-1 twice), one warp
    //    per child in a fixed order; the ends and the fold correction
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int it = warp; it < nh; it += nw) {
        const double2 *zz = sm + (size_t)it * h;
        double s = 0.0;
        for (int f = 1 + lane; f < h; f += 32) s += zz[f].x;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            DnView &v = V[it];
            const double a0 = (zz[0].x + v.pfh.x + 2.0 * s) * invD;
            const double yD = a0 - v.amb0;
            const double e0 = a0 - v.pbt * v.ps0;
            const double eD = yD - v.pb0 * v.psd;
            v.delta = e0 + eD - a0;
            double *pe = A.Peout + q * A.Peo_q + (size_t)v.c * 2;
            pe[0] = e0;
            pe[1] = eD;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nh * (h + 1); e += blockDim.x) {
        const int it = e / (h + 1), f = e - it * (h + 1);
        const DnView &v = V[it];
        const double2 val = (f < h) ? sm[(size_t)it * h + f] : v.pfh;
        A.PFout[q * A.PFo_q + (size_t)v.c * (h + 1) + f] = make_double2(val.x + v.delta, val.y);
    }
}

// single plans: grid (nbx, nq); work lists: CTA i runs block tab[i].y of
// descriptor tab[i].x (members of a batch, one level each)
__global__ void __launch_bounds__(kVspThreadsMax) k_vsp_real(VspRealArgs A) { vsp_real_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kVspThreadsMax) k_vsp_up(VspUpArgs A) { vsp_up_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kVspThreadsMax) k_vsp_down(VspDownArgs A) { vsp_down_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kVspThreadsMax)
kw_vsp_real(const VspRealArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    VspRealArgs A = D[t.x];
    A.z.q0 = q0;
    vsp_real_body(A, t.y, blockIdx.y);
}
__global__ void __launch_bounds__(kVspThreadsMax)
kw_vsp_up(const VspUpArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    VspUpArgs A = D[t.x];
    A.z.q0 = q0;
    vsp_up_body(A, t.y, blockIdx.y);
}
__global__ void __launch_bounds__(kVspThreadsMax)
kw_vsp_down(const VspDownArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    VspDownArgs A = D[t.x];
    A.z.q0 = q0;
    vsp_down_body(A, t.y, blockIdx.y);
}

// ------------------------------------------------------------ multi-pass kernels
// upward, children of degree D > kSpecMaxD: items = parents, buf rows of D points
__global__ void k_vsb_up_in(VspUpArgs A) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD, hD = D >> 1;
    const int j = (int)(e / (hD + 1)), f = (int)(e % (hD + 1));
    if (j >= A.nreal_p) return;
    double2 *ao = A.Aout ? A.Aout + q * A.Ao_q + (size_t)j * (2 * D + 1) : nullptr;
    if (zp_cold(A.z, q, j)) {   // gbar 0 (the odd bins in k_vsb_up_odd)
        if (ao) ao[2 * f] = ao[2 * (D - f)] = make_double2(0.0, 0.0);
        return;
    }
    double2 Cf, Cc, Uf, Uc;
    up_pair(A, q, j, f, Cf, Cc);
    if (ao) {
        ao[2 * f] = Cf;
        ao[2 * (D - f)] = Cc;
    }
    inv_input(Cf, Cc, f, A.tw, A.logTW, A.logD, Uf, Uc);
    double2 *u = A.buf + ((size_t)q * A.nreal_p + j) * D;
    u[f] = Uf;
    if (f != 0 && f != hD) u[D - f] = Uc;
}

// after the inverse, where the level above works on coefficients: the
// parents' gbar coefficients (zero for wholly-zero parents)
__global__ void k_vsb_up_mid(VspUpArgs A, int W) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD;
    const int j = (int)(e / W), s = (int)(e % W);
    if (j >= A.nreal_p) return;
    const bool cold = zp_cold(A.z, q, j);
    const double2 *u = A.buf + ((size_t)q * A.nreal_p + j) * D;
    double *go = A.gout + q * A.go_q + (size_t)j * A.gst;
    const double2 v = (!cold && s < D) ? u[s] : make_double2(0.0, 0.0);
    const double inv2D = 1.0 / (2.0 * D);
    const int t0 = 2 * s, t1 = 2 * s + 1;
    if (t0 < A.gst) go[t0] = t0 < A.glen ? v.x * inv2D : 0.0;
    if (t1 < A.gst) go[t1] = t1 < A.glen ? v.y * inv2D : 0.0;
}

__global__ void k_vsb_up_odd(VspUpArgs A) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD, hD = D >> 1;
    const int j = (int)(e / hD), f = (int)(e % hD);
    if (j >= A.nreal_p) return;
    double2 *ao = A.Aout + q * A.Ao_q + (size_t)j * (2 * D + 1);
    if (zp_cold(A.z, q, j)) {
        ao[2 * f + 1] = ao[2 * (D - 1 - f) + 1] = make_double2(0.0, 0.0);
        return;
    }
    const double2 *c = A.buf + ((size_t)q * A.nreal_p + j) * D;
    double2 Hf, Hc;
    odd_bins(c[f], c[D - 1 - f], f, A.tw, A.logTW, A.logD, Hf, Hc);
    ao[2 * f + 1] = Hf;
    ao[2 * (D - 1 - f) + 1] = Hc;
}

// downward, children of degree D > 2 kSpecMaxD: items = children, buf rows of D/2 points
__global__ void k_vsb_dn_in(VspDownArgs A) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD, h = D >> 1, hp = (h + 1) >> 1;
    const int c = (int)(e / hp), f = (int)(e % hp);
    if (c >= A.nreal_c || zp_cold(A.z, q, c)) return;
    const DnView v = dn_view(A, q, c);
    const int fp = h - 1 - f;
    const double2 Y1 = dn_z(v, 2 * f + 1);
    const double2 Y2 = cconj(dn_z(v, 2 * fp + 1));
    double2 Xf, Xc;   // A + i B, conj(A) + i conj(B), B = (Y1 - Y2) conj(w_f)
    mirror_inv_input(cadd(Y1, Y2), csub(Y1, Y2), tw_tangent(A.tw, A.logTW), (long)(2 * f + 1) << (A.logTW - A.logD - 1),
                     A.logTW, Xf, Xc);
    double2 *x = A.buf + ((size_t)q * A.nreal_c + c) * h;
    x[f] = Xf;
    if (fp != f) x[fp] = Xc;
}

// after the inverse: (a - b)[0] parked in the child's first end slot (the
// untwist is the next forward transform's half shift by -1/2 bin)
__global__ void k_vsb_dn_park(VspDownArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD, h = D >> 1;
    if (c >= A.nreal_c || zp_cold(A.z, q, c)) return;
    const double2 *x = A.buf + ((size_t)q * A.nreal_c + c) * h;
    A.Peout[q * A.Peo_q + (size_t)c * 2] = x[0].x * (1.0 / D);
}

// DFT_D(a) by mirror pairs (f, h - f) into the child's spectrum row (no fold correction yet)
__global__ void k_vsb_dn_pf(VspDownArgs A) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int D = 1 << A.logD, h = D >> 1, hq = (h >> 1) + 1;
    const int c = (int)(e / hq), f = (int)(e % hq);
    if (c >= A.nreal_c || zp_cold(A.z, q, c)) return;
    const DnView v = dn_view(A, q, c);
    const double2 *zz = A.buf + ((size_t)q * A.nreal_c + c) * h;
    double2 *out = A.PFout + q * A.PFo_q + (size_t)c * (h + 1);
    const int fp = h - f;
    const double kx = 1.0 / (8.0 * h);
    const double2 zf = zz[f & (h - 1)], zc = cconj(zz[fp & (h - 1)]);
    const double2 E = cadd(zf, zc);
    double r;   // T = r u = -i (zf - zc) e^{-2 pi i f/D}
    const double2 u =
        tanmul_t<-1>(cmul_mi(csub(zf, zc)), tw_tangent(A.tw, A.logTW), (long)f << (A.logTW - A.logD), A.logTW, &r);
    const double2 Yf = dn_z(v, 2 * f);
    const double2 Xf = make_double2(fma(r, u.x, E.x), fma(r, u.y, E.y));
    out[f] = make_double2(fma(kx, Xf.x, 0.5 * Yf.x), fma(kx, Xf.y, 0.5 * Yf.y));
    if (fp != f) {
        const double2 Yc = dn_z(v, 2 * fp);
        const double2 Xc = make_double2(fma(-r, u.x, E.x), fma(r, u.y, -E.y));   // conj(E - T)
        out[fp] = make_double2(fma(kx, Xc.x, 0.5 * Yc.x), fma(kx, Xc.y, 0.5 * Yc.y));
    }
}

// one CTA per child: a[0] by a fixed-order reduction, the ends, the fold correction
constexpr int kFinThreads = 256;
__global__ void __launch_bounds__(kFinThreads) k_vsb_dn_fin(VspDownArgs A) {
    __shared__ double red[kFinThreads];
    __shared__ double delta_s;
    const int q = blockIdx.y, c = blockIdx.x;
    if (c >= A.nreal_c || zp_cold(A.z, q, c)) return;
    const int D = 1 << A.logD, h = D >> 1;
    double2 *pf = A.PFout + q * A.PFo_q + (size_t)c * (h + 1);
    double s = 0.0;
    for (int f = 1 + threadIdx.x; f < h; f += kFinThreads) s += pf[f].x;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kFinThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const DnView v = dn_view(A, q, c);
        double *pe = A.Peout + q * A.Peo_q + (size_t)c * 2;
        const double a0 = (pf[0].x + pf[h].x + 2.0 * red[0]) * (1.0 / D);
        const double yD = a0 - pe[0];
        const double e0 = a0 - v.pbt * v.ps0;
        const double eD = yD - v.pb0 * v.psd;
        delta_s = e0 + eD - a0;
        pe[0] = e0;
        pe[1] = eD;
    }
    __syncthreads();
    const double dl = delta_s;
    for (int f = threadIdx.x; f <= h; f += kFinThreads) pf[f].x += dl;
}

// ------------------------------------------------------------ host
void vjp_spec_set_smem_limits() {
    const int mx = (int)((size_t)kSpecMaxD * sizeof(double2) + sizeof(DnView) + 64);
    cudaFuncSetAttribute(k_vsp_real, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_vsp_up, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_vsp_down, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_vsp_real, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_vsp_up, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_vsp_down, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

static size_t real_smem(int M, int cb) { return (size_t)cb * M * sizeof(double2) + (size_t)cb * sizeof(int); }
static size_t up_smem(int D, int cb) { return (size_t)cb * D * sizeof(double2) + (size_t)cb * sizeof(int); }
static size_t down_smem(int per, int cb) {
    return (size_t)cb * per * sizeof(double2) + (size_t)cb * (sizeof(DnView) + sizeof(int));
}

bool vsp_one_cta(const Plan *p, int l) {
    const long D = p->lv[l - 1].deg;
    return D <= kSpecMaxD;
}

VspRealArgs vsp_gbar_real_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW,
                               size_t *smem) {
    const Level &c = p->lv[l - 1];
    VspRealArgs R{};
    R.x = b.gb[l - 1];
    R.x_q = b.gb_q[l - 1];
    R.xst = b.gb_st[l - 1];
    R.xlen = c.glen;
    R.nreal = c.nreal;
    R.logM = ilog2v(c.deg);
    R.out = b.Gb2[l - 1];
    R.o_q = b.Gb2_q[l - 1];
    R.tw = tw;
    R.logTW = logTW;
    R.z = ZeroPrefix{p->zskip ? p->d_z : nullptr, q0, c.deg};
    R.cb = vsp_cb(1 << R.logM);
    R.nbx = (int)nbv(R.nreal, R.cb);
    if (smem) *smem = real_smem(1 << R.logM, R.cb);
    return R;
}

VspRealArgs vsp_pbar_real_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW,
                               size_t *smem) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    VspRealArgs R{};
    R.x = b.Pb[l];
    R.x_q = pl.P_q;
    R.xst = pl.pst;
    R.xlen = pl.plen;
    R.nreal = pl.nreal;
    R.logM = ilog2v(c.deg);
    R.fold = 1;
    R.out = b.PF[l];
    R.o_q = b.PF_q[l];
    R.ends = b.Pe[l];
    R.e_q = b.Pe_q[l];
    R.tw = tw;
    R.logTW = logTW;
    R.z = ZeroPrefix{p->zskip ? p->d_z : nullptr, q0, pl.deg};
    R.cb = vsp_cb(1 << R.logM);
    R.nbx = (int)nbv(R.nreal, R.cb);
    if (smem) *smem = real_smem(1 << R.logM, R.cb);
    return R;
}

VspUpArgs vsp_up_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW, size_t *smem) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    const bool spec_out = !root && p->lv[l + 1].kind == 2;
    VspUpArgs A{};
    A.A = b.Gb2[l - 1];
    A.A_q = b.Gb2_q[l - 1];
    A.S = c.spec2;
    A.S_q = c.spec2_q;
    A.nreal_c = c.nreal;
    A.nreal_p = pl.nreal;
    A.logD = ilog2v(c.deg);
    if (spec_out) {
        A.Aout = b.Gb2[l];
        A.Ao_q = b.Gb2_q[l];
    } else {
        A.gout = root ? b.root : b.gb[l];
        A.go_q = root ? b.root_q : b.gb_q[l];
        A.gst = root ? b.kst : b.gb_st[l];
        A.glen = root ? p->k : pl.glen;
    }
    A.tw = tw;
    A.logTW = logTW;
    A.z = ZeroPrefix{p->zskip ? p->d_z : nullptr, q0, pl.deg};
    A.cb = vsp_cb(1 << A.logD);
    A.nbx = (int)nbv(A.nreal_p, A.cb);
    if (smem) *smem = up_smem(1 << A.logD, A.cb);
    return A;
}

VspDownArgs vsp_down_args(const Plan *p, const VjpBufs &b, int l, int q0, const double2 *tw, int logTW,
                          size_t *smem) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    VspDownArgs A{};
    A.G = pl.G;
    A.G_q = root ? 0 : pl.G_q;
    if (!root) {
        A.PF = b.PF[l];
        A.PF_q = b.PF_q[l];
        A.Pe = b.Pe[l];
        A.Pe_q = b.Pe_q[l];
    }
    A.A = b.Gb2[l - 1];
    A.A_q = b.Gb2_q[l - 1];
    A.S = c.spec2;
    A.S_q = c.spec2_q;
    A.E = c.ends;
    A.E_q = c.ends_q;
    A.nreal_c = c.nreal;
    A.logD = ilog2v(c.deg);
    const bool spec_out = c.kind == 2;
    if (spec_out) {
        A.PFout = b.PF[l - 1];
        A.PFo_q = b.PF_q[l - 1];
        A.Peout = b.Pe[l - 1];
        A.Peo_q = b.Pe_q[l - 1];
    } else {
        A.Pout = b.Pb[l - 1];
        A.Po_q = c.P_q;
        A.pst = c.pst;
    }
    A.tw = tw;
    A.logTW = logTW;
    A.z = ZeroPrefix{p->zskip ? p->d_z : nullptr, q0, c.deg};
    const int per = spec_out ? (1 << A.logD) / 2 : (1 << A.logD);
    A.cb = vsp_cb(per);
    A.nbx = (int)nbv(A.nreal_c, A.cb);
    if (smem) *smem = down_smem(per, A.cb);
    return A;
}

void launch_worklist_vsp(WOp op, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    switch (op) {
        case WOp::AdjSpecReal:
            kw_vsp_real<<<g, vsp_tpb(smem), smem, st>>>((const VspRealArgs *)desc, tab, q0);
            break;
        case WOp::AdjSpecUp: kw_vsp_up<<<g, vsp_tpb(smem), smem, st>>>((const VspUpArgs *)desc, tab, q0); break;
        case WOp::AdjSpecDown:
            kw_vsp_down<<<g, vsp_tpb(smem), smem, st>>>((const VspDownArgs *)desc, tab, q0);
            break;
        default: break;
    }
}

static void launch_real(const VspRealArgs &R0, int nq, cudaStream_t st, Prof *pr, long &launches) {
    VspRealArgs R = R0;
    const int M = 1 << R.logM;
    R.cb = short_grid_cb(vsp_cb(M), R.nreal, nq);
    R.nbx = (int)nbv(R.nreal, R.cb);
    const size_t sm = real_smem(M, R.cb);
    pr->begin("adj_spec_real", (5.0 * M * R.logM + 20.0 * M) * R.nreal * nq, st);
    k_vsp_real<<<dim3(R.nbx, nq), vsp_tpb(sm), sm, st>>>(R);
    pr->end(st);
    ++launches;
}

void adj_spec_up(Plan *p, const VjpBufs &b, int l, int nq, int q0, const double2 *tw, int logTW, long &launches) {
    const Level &c = p->lv[l - 1], &pl = p->lv[l];
    const bool root = (l == p->L - 1);
    const bool spec_out = !root && p->lv[l + 1].kind == 2;
    const int logD = ilog2v(c.deg), D = 1 << logD;
    const int *zp = p->zskip ? p->d_z : nullptr;
    cudaStream_t st = p->stream;
    Prof *pr = &p->prof;
    if (c.kind != 2)   // the children's gbar as spectra (the band's bottom; D <= kSpecMaxD)
        launch_real(vsp_gbar_real_args(p, b, l, q0, tw, logTW, nullptr), nq, st, pr, launches);
    VspUpArgs A = vsp_up_args(p, b, l, q0, tw, logTW, nullptr);
    const double fl = (spec_out ? 10.0 * D * logD + 40.0 * D : 5.0 * D * logD + 20.0 * D) * pl.nreal * nq;
    if (vsp_one_cta(p, l)) {
        A.cb = short_grid_cb(A.cb, pl.nreal, nq);
        A.nbx = (int)nbv(pl.nreal, A.cb);
        const size_t sm = up_smem(D, A.cb);
        pr->begin("adj_spec_up", fl, st);
        k_vsp_up<<<dim3(A.nbx, nq), vsp_tpb(sm), sm, st>>>(A);
        pr->end(st);
        ++launches;
        return;
    }
    // multi-pass: inverse input, inverse, then coefficients or a half-shifted forward transform and the odd bins
    A.buf = p->d_fa;
    const FftSkip sk{zp, q0, pl.deg, pl.nreal, 0};
    const long items = (long)nq * pl.nreal;
    const double pw = 20.0 * D * pl.nreal * nq;   // pointwise steps
    pr->begin("adj_specbig_up_in", pw, st);
    k_vsb_up_in<<<dim3(nbv((long)pl.nreal * (D / 2 + 1), 256), nq), 256, 0, st>>>(A);
    pr->end(st);
    fft_batched(A.buf, p->d_fc, items, logD, +1, tw, logTW, st, &launches, pr, sk);
    ++launches;
    if (!spec_out) {   // the level above works on coefficients
        const int W = std::max(D, (A.gst + 1) / 2);
        pr->begin("adj_specbig_up_mid", pw, st);
        k_vsb_up_mid<<<dim3(nbv((long)pl.nreal * W, 256), nq), 256, 0, st>>>(A, W);
        pr->end(st);
        ++launches;
        return;
    }
    // odd bins: the forward transform of the twisted packing, the twist
    // e^{-2 pi i s/2D} folded into the transform as its half shift
    fft_batched(A.buf, p->d_fc, items, logD, -1, tw, logTW, st, &launches, pr, sk, +1);
    pr->begin("adj_specbig_up_odd", pw, st);
    k_vsb_up_odd<<<dim3(nbv((long)pl.nreal * (D / 2), 256), nq), 256, 0, st>>>(A);
    pr->end(st);
    ++launches;
    (void)fl;
}

void adj_spec_down(Plan *p, const VjpBufs &b, int l, int nq, int q0, const double2 *tw, int logTW, long &launches) {
    const Level &c = p->lv[l - 1];
    const bool root = (l == p->L - 1);
    const int logD = ilog2v(c.deg), D = 1 << logD, h = D / 2;
    const int *zp = p->zskip ? p->d_z : nullptr;
    cudaStream_t st = p->stream;
    Prof *pr = &p->prof;
    if (!root && p->lv[l + 1].kind != 2)   // the parents' Pbar as folded spectra (the band's top; D <= kSpecMaxD)
        launch_real(vsp_pbar_real_args(p, b, l, q0, tw, logTW, nullptr), nq, st, pr, launches);
    VspDownArgs A = vsp_down_args(p, b, l, q0, tw, logTW, nullptr);
    const bool spec_out = c.kind == 2;
    const double fl = (spec_out ? 10.0 * h * (logD - 1) + 60.0 * h : 5.0 * D * logD + 30.0 * D) * c.nreal * nq;
    const int per = spec_out ? h : D;
    if (per <= kSpecMaxD) {
        A.cb = short_grid_cb(A.cb, c.nreal, nq);
        A.nbx = (int)nbv(c.nreal, A.cb);
        const size_t sm = down_smem(per, A.cb);
        pr->begin("adj_spec_down", fl, st);
        k_vsp_down<<<dim3(A.nbx, nq), vsp_tpb(sm), sm, st>>>(A);
        pr->end(st);
        ++launches;
        return;
    }
    // multi-pass (children beyond 2 kSpecMaxD are always spectral)
    A.buf = p->d_fa;
    const FftSkip sk{zp, q0, c.deg, c.nreal, 0};
    const long items = (long)nq * c.nreal;
    const int lh = logD - 1;
    const double pw = 20.0 * h * c.nreal * nq;   // pointwise steps
    pr->begin("adj_specbig_down_in", pw, st);
    k_vsb_dn_in<<<dim3(nbv((long)c.nreal * ((h + 1) / 2), 256), nq), 256, 0, st>>>(A);
    pr->end(st);
    fft_batched(A.buf, p->d_fc, items, lh, +1, tw, logTW, st, &launches, pr, sk);
    pr->begin("adj_specbig_down_park", 0.0, st);
    k_vsb_dn_park<<<dim3(nbv(c.nreal, 256), nq), 256, 0, st>>>(A);
    pr->end(st);
    fft_batched(A.buf, p->d_fc, items, lh, -1, tw, logTW, st, &launches, pr, sk, -1);   // half-shifted: the untwist
    pr->begin("adj_specbig_down_pf", pw, st);
    k_vsb_dn_pf<<<dim3(nbv((long)c.nreal * (h / 2 + 1), 256), nq), 256, 0, st>>>(A);
    pr->end(st);
    pr->begin("adj_specbig_down_fin", pw, st);
    k_vsb_dn_fin<<<dim3(c.nreal, nq), kFinThreads, 0, st>>>(A);
    pr->end(st);
    launches += 4;
    (void)fl;
}

}  // namespace icmg
