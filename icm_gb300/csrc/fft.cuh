// fft.cuh -- FP64 complex FFT building blocks for sm_103a (device side).
//
// Transforms run in shared memory as in-place radix-4 decimation-in-time
// passes over bit-reversed input (two radix-2 stages fused per pass, so the
// output is in natural order), with one radix-2 pass when log2(M) is odd.
// Twiddles for pointwise steps come from one device table
// tw[t] = exp(-2 pi i t / 2^logTW) and its tangent-form copy; the butterflies
// use the tangent-form tables stored between the two (plain and half-shifted
// sets, below).
#pragma once

#include <cuda_runtime.h>

namespace icmg {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
// multiply by -i and +i
__device__ __forceinline__ double2 cmul_mi(double2 a) { return make_double2(a.y, -a.x); }
__device__ __forceinline__ double2 cmul_pi(double2 a) { return make_double2(-a.y, a.x); }

__device__ __forceinline__ unsigned bitrev(unsigned v, int logM) {
    return logM == 0 ? 0u : (__brev(v) >> (32 - logM));
}

// SIGN = -1: forward (e^{-...}); SIGN = +1: backward (e^{+...}), unnormalised.
template <int SIGN>
__device__ __forceinline__ double2 twmul(double2 a, double2 w) {
    return SIGN < 0 ? cmul(a, w) : cmulc(a, w);
}

// Tangent-form twiddles.  Every twiddle w is stored as w = R r (1 + i tau)
// with R in {1, -i, -1, i} (2-bit code), r >= 1/sqrt(2) and |tau| <= 1, so
// z w = r ((R z) + i tau (R z)): the rotation is a swap/sign change on the
// integer pipe, (1 + i tau) costs 2 FMAs and r folds into the following
// additions.  A radix-4 DIT butterfly then costs 22 FP64 instructions
// (6 for the three (1 + i tau) products, 16 FMAs for the sums with r1, r2 and
// rho = r3 / r1 folded in) instead of 28.
//
// The tables follow the plain table tw[0 .. 2^logTW) in the same allocation:
//   R4[h + j]  j < h, h = 4^m:  {tau1, r1}, {tau2, r2}, {tau3, rho} for the
//              twiddles w^j, w^2j, w^3j of a pass with groups of 4h (w = e^{-2 pi i/4h})
//   R4C[h + j] rotation codes of those three twiddles (bits 0-1, 2-3, 4-5)
//   R2[h + j]  {tau, r} of e^{-2 pi i j/2h} for the final radix-2 pass
//   R2C[h + j] its rotation code
// Two more sets of the same four tables follow for the half-shifted forward
// transforms X(k + sigma/2) = sum_s x_s e^{-2 pi i s (k + sigma/2)/M},
// sigma = +1 or -1 (a DFT of x_s e^{-pi i sigma s/M} without the twist):
// in decimation in time a half shift of the whole transform is a half shift
// of both halves, X(k + 1/2) = E(k + 1/2) + W_M^{k+1/2} O(k + 1/2), so every
// pass keeps its butterflies and takes the twiddles w^{j + sigma/2} (the
// first radix-4 pass then has general twiddles too).
constexpr int kTwMaxH4 = 2048;   // radix-4 passes of transforms up to 8192 points
constexpr int kTwMaxH2 = 4096;   // radix-2 pass of an 8192-point transform

struct GTw {
    double2 a, b, c;
};

struct TwTables {
    const GTw *r4;
    const int *r4c;
    const double2 *r2;
    const int *r2c;
};

// bytes of one set of tangent tables
constexpr size_t kTwSetBytes = sizeof(GTw) * 2 * kTwMaxH4 + sizeof(int) * 2 * kTwMaxH4 +
                               sizeof(double2) * 2 * kTwMaxH2 + sizeof(int) * 2 * kTwMaxH2;
static_assert(kTwSetBytes % 256 == 0, "table sets stay aligned");
// the set of a transform with half shift sigma: 0 plain, 1 for +1/2, 2 for -1/2
__host__ __device__ constexpr int tw_set(int sigma) { return sigma == 0 ? 0 : (sigma > 0 ? 1 : 2); }

__device__ __forceinline__ TwTables tw_tables(const double2 *tw, int logTW, int set = 0) {
    const char *base = (const char *)(tw + (1L << logTW)) + (size_t)set * kTwSetBytes;
    TwTables t;
    t.r4 = (const GTw *)base;
    base += sizeof(GTw) * 2 * kTwMaxH4;
    t.r4c = (const int *)base;
    base += sizeof(int) * 2 * kTwMaxH4;
    t.r2 = (const double2 *)base;
    base += sizeof(double2) * 2 * kTwMaxH2;
    t.r2c = (const int *)base;
    return t;
}

// bytes of the tangent tables that follow the plain table: three sets
constexpr size_t kTwExtraBytes = 3 * kTwSetBytes;

// After the sets: the tangent form of every plain entry, tw[t] = e^{-2 pi i t/N}
// = R r (1 + i tau) with {tau, r} stored and R = (1, -i, -1, i)[tan_code(t)],
// the quarter turn nearest the angle (taken from t, so not stored).
__host__ __device__ __forceinline__ int tan_code(long t, int logTW) {
    return (int)(((8 * t + (1L << logTW) - 1) >> (logTW + 1)) & 3);
}
__device__ __forceinline__ const double2 *tw_tangent(const double2 *tw, int logTW) {
    return (const double2 *)((const char *)(tw + (1L << logTW)) + kTwExtraBytes);
}

__device__ __forceinline__ double dneg_if(double v, int neg) {
    return __longlong_as_double(__double_as_longlong(v) ^ ((long long)neg << 63));
}

// R z for code 0: 1, 1: -i, 2: -1, 3: i (SIGN = +1 uses conj(R): codes 1 <-> 3)
template <int SIGN>
__device__ __forceinline__ double2 rot(double2 z, int code) {
    if (SIGN > 0) code = (4 - code) & 3;
    const int sw = code & 1;
    const double x = sw ? z.y : z.x, y = sw ? z.x : z.y;
    return make_double2(dneg_if(x, code >> 1), dneg_if(y, (code == 1) | (code == 2)));
}

// (R z)(1 + i tau); the inverse transform uses conj: R -> conj R, tau -> -tau
template <int SIGN>
__device__ __forceinline__ double2 tanmul(double2 z, int code, double tau) {
    const double2 v = rot<SIGN>(z, code);
    if (SIGN < 0) return make_double2(fma(-tau, v.y, v.x), fma(tau, v.x, v.y));
    return make_double2(fma(tau, v.y, v.x), fma(-tau, v.x, v.y));
}

// z w_t / r (SIGN < 0) or z conj(w_t) / r (SIGN > 0) for the plain entry
// w_t = tw[t] in tangent form (tt = tw_tangent(tw, logTW)); r goes to *r
template <int SIGN>
__device__ __forceinline__ double2 tanmul_t(double2 z, const double2 *__restrict__ tt, long t, int logTW, double *r) {
    const double2 g = __ldg(&tt[t]);
    *r = g.y;
    return tanmul<SIGN>(z, tan_code(t, logTW), g.x);
}

// Pointwise steps of a real transform of size 2M done as a complex one of
// size M, on a mirror pair of bins.
// Inverse input: Uf = E + i O, Uc = conj(E) + i conj(O), O = Dd conj(w_t),
// the factor r of w_t folded into the sums.
__device__ __forceinline__ void mirror_inv_input(double2 E, double2 Dd, const double2 *__restrict__ tt, long t,
                                                 int logTW, double2 &Uf, double2 &Uc) {
    double r;
    const double2 o = tanmul_t<+1>(Dd, tt, t, logTW, &r);   // O = r o
    Uf = make_double2(fma(-r, o.y, E.x), fma(r, o.x, E.y));
    Uc = make_double2(fma(r, o.y, E.x), fma(r, o.x, -E.y));
}
// Output pair from the forward transform's bins a and b (b already
// conjugated): Hf = kb (Ep + T), Hc = kb conj(Ep - T), Ep = a + b,
// T = -i (a - b) w_t; kb a power of two (exact scaling).
__device__ __forceinline__ void mirror_out_pair(double2 a, double2 b, double kb, const double2 *__restrict__ tt, long t,
                                                int logTW, double2 &Hf, double2 &Hc) {
    const double2 Ek = cscale(cadd(a, b), kb);
    double r;
    const double2 u = tanmul_t<-1>(cmul_mi(csub(a, b)), tt, t, logTW, &r);   // T = r u
    const double rk = r * kb;
    Hf = make_double2(fma(rk, u.x, Ek.x), fma(rk, u.y, Ek.y));
    Hc = make_double2(fma(-rk, u.x, Ek.x), fma(rk, u.y, -Ek.y));
}

// Unpack bin f of a real transform from the complex one z of half the size:
// 0.5 (a + w_t b), a = z_f + conj z_{M-f}, b = -i (z_f - conj z_{M-f}); the
// factors r of w_t and 0.5 folded into one FMA per component.
__device__ __forceinline__ double2 half_sum_tw(double2 a, double2 b, const double2 *__restrict__ tt, long t, int logTW) {
    double r;
    const double2 u = tanmul_t<-1>(b, tt, t, logTW, &r);
    const double hr = 0.5 * r;
    return make_double2(fma(hr, u.x, 0.5 * a.x), fma(hr, u.y, 0.5 * a.y));
}

// the twiddle between the four-step passes, W_M^{n2 (k1 + SHIFT/2)}: index
// into the plain table (SHIFT = 0: n2 k1 mod M, else n2 (2 k1 + SHIFT) mod 2M)
template <int SHIFT>
__device__ __forceinline__ long fft4_tw_index(int n2, int k1, int logM, int logTW) {
    if (SHIFT == 0) return (long)((n2 * k1) & ((1 << logM) - 1)) << (logTW - logM);
    return (long)((n2 * (2 * k1 + SHIFT)) & ((2 << logM) - 1)) << (logTW - logM - 1);
}

// Both bins of an unpack mirror pair (f, M - f): Xf = 0.5 (a + w_t b) and
// Xc = 0.5 conj(a - w_t b), bin M - f of the same real transform.
__device__ __forceinline__ void half_sum_tw_pair(double2 a, double2 b, const double2 *__restrict__ tt, long t,
                                                 int logTW, double2 &Xf, double2 &Xc) {
    double r;
    const double2 u = tanmul_t<-1>(b, tt, t, logTW, &r);
    const double hr = 0.5 * r;
    const double2 a5 = cscale(a, 0.5);
    Xf = make_double2(fma(hr, u.x, a5.x), fma(hr, u.y, a5.y));
    Xc = make_double2(fma(-hr, u.x, a5.x), fma(hr, u.y, -a5.y));
}

// `cnt` transforms of size 2^logM stored back to back in x (shared memory),
// each already in bit-reversed order.  All threads of the block take part;
// the caller synchronises before (after filling x) and this function ends
// with a barrier.  SHIFT = +1 / -1: the forward transform half-shifted by
// +1/2 / -1/2 bin (SIGN = -1 only).
template <int SIGN, int SHIFT = 0>
__device__ void smem_fft_dit(double2 *x, int logM, int cnt, const double2 *__restrict__ tw, int logTW) {
    static_assert(SHIFT == 0 || SIGN < 0, "half-shifted transforms are forward only");
    const TwTables T = tw_tables(tw, logTW, tw_set(SHIFT));
    const int M = 1 << logM;
    int s = 0;
    for (; s + 1 < logM; s += 2) {
        const int h = 1 << s;
        const int nb = cnt << (logM - 2);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 2);
            const int r = b & ((M >> 2) - 1);
            const int j = r & (h - 1);
            const int i = item * M + ((r >> s) << (s + 2)) + j;
            const double2 a = x[i], bq = x[i + h], c = x[i + 2 * h], d = x[i + 3 * h];
            double2 x0, x1, x2, x3;
            if (SHIFT == 0 && h == 1) {   // first pass: all twiddles are 1
                const double2 s0 = cadd(a, bq), d0 = csub(a, bq);
                const double2 s1 = cadd(c, d), d1 = csub(c, d);
                x0 = cadd(s0, s1);
                x2 = csub(s0, s1);
                if (SIGN < 0) { x1 = cadd(d0, cmul_mi(d1)); x3 = csub(d0, cmul_mi(d1)); }
                else { x1 = cadd(d0, cmul_pi(d1)); x3 = csub(d0, cmul_pi(d1)); }
            } else {
                const GTw g = T.r4[h + j];
                const int code = __ldg(&T.r4c[h + j]);
                const double2 uc = tanmul<SIGN>(c, code & 3, g.a.x);          // t1 = R1 r1 (1 + i tau1)
                const double2 ub = tanmul<SIGN>(bq, (code >> 2) & 3, g.b.x);  // t2
                const double2 ud = tanmul<SIGN>(d, (code >> 4) & 3, g.c.x);   // t3, r3 = rho r1
                const double r1 = g.a.y, r2 = g.b.y, rho = g.c.y;
                const double2 s0 = make_double2(fma(r2, ub.x, a.x), fma(r2, ub.y, a.y));
                const double2 d0 = make_double2(fma(-r2, ub.x, a.x), fma(-r2, ub.y, a.y));
                const double2 e = make_double2(fma(rho, ud.x, uc.x), fma(rho, ud.y, uc.y));
                const double2 f = make_double2(fma(-rho, ud.x, uc.x), fma(-rho, ud.y, uc.y));
                x0 = make_double2(fma(r1, e.x, s0.x), fma(r1, e.y, s0.y));
                x2 = make_double2(fma(-r1, e.x, s0.x), fma(-r1, e.y, s0.y));
                if (SIGN < 0) {   // x1 = d0 - i r1 f, x3 = d0 + i r1 f
                    x1 = make_double2(fma(r1, f.y, d0.x), fma(-r1, f.x, d0.y));
                    x3 = make_double2(fma(-r1, f.y, d0.x), fma(r1, f.x, d0.y));
                } else {
                    x1 = make_double2(fma(-r1, f.y, d0.x), fma(r1, f.x, d0.y));
                    x3 = make_double2(fma(r1, f.y, d0.x), fma(-r1, f.x, d0.y));
                }
            }
            x[i] = x0;
            x[i + h] = x1;
            x[i + 2 * h] = x2;
            x[i + 3 * h] = x3;
        }
        __syncthreads();
    }
    if (s < logM) {  // one radix-2 stage left, half size h = M/2
        const int h = 1 << s;
        const int nb = cnt << (logM - 1);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 1);
            const int r = b & ((M >> 1) - 1);
            const int j = r & (h - 1);
            const int i = item * M + ((r >> s) << (s + 1)) + j;
            const double2 a = x[i], bq = x[i + h];
            const double2 g = T.r2[h + j];
            const double2 u = tanmul<SIGN>(bq, __ldg(&T.r2c[h + j]), g.x);
            x[i] = make_double2(fma(g.y, u.x, a.x), fma(g.y, u.y, a.y));
            x[i + h] = make_double2(fma(-g.y, u.x, a.x), fma(-g.y, u.y, a.y));
        }
        __syncthreads();
    }
}

// In-place bit-reversal permutation of `cnt` arrays of 2^logM points with a
// pointwise map applied on the way: slot bitrev(s) <- op(it, s, x[s]).  Each
// thread owns whole pairs (s, bitrev(s)), so there is no read/write race.
template <typename Op>
__device__ void smem_bitrev_map(double2 *x, int logM, int cnt, Op op) {
    const int M = 1 << logM;
    for (int e = threadIdx.x; e < cnt * M; e += blockDim.x) {
        const int it = e >> logM, s = e & (M - 1);
        const int r = (int)bitrev(s, logM);
        if (r < s) continue;
        double2 *xi = x + (size_t)it * M;
        const double2 vs = xi[s], vr = xi[r];
        xi[r] = op(it, s, vs);
        if (r != s) xi[s] = op(it, r, vr);
    }
    __syncthreads();
}

}  // namespace icmg
