// twiddle.cpp -- host construction of the device twiddle tables:
// tw[t] = exp(-2 pi i t / 2^logTW) followed by the tangent-form tables of
// the FFT butterflies (fft.cuh): plain and half-shifted by +-1/2 bin.  Every
// value is computed in long double from an angle folded into [0, pi/4] with
// exact integer reflections, then rounded once to double.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "fft.cuh"

namespace icmg {

// e^{-2 pi i t / N} in long double
static void unit_root_ld(long t, long N, long double *re, long double *im) {
    static const long double two_pi = 6.283185307179586476925286766559005768L;
    t %= N;
    if (t < 0) t += N;
    int conj = 0, neg_c = 0;
    if (2 * t > N) { t = N - t; conj = 1; }
    long num = t, den = N;
    if (4 * t > N) { num = N - 2 * t; den = 2 * N; neg_c = 1; }
    long double c, s;
    if (8 * num > den) {
        const long double b = two_pi * (long double)(den - 4 * num) / (4.0L * (long double)den);
        c = sinl(b);
        s = cosl(b);
    } else {
        const long double a = two_pi * (long double)num / (long double)den;
        c = cosl(a);
        s = sinl(a);
    }
    if (neg_c) c = -c;
    *re = c;
    *im = conj ? s : -s;
}

// w = R r (1 + i tau) with R = 1, -i, -1, i for codes 0..3 and r >= 1/sqrt 2
static void tangent_form(long t, long N, int *code, long double *r, long double *tau) {
    long double wr, wi;
    unit_root_ld(t, N, &wr, &wi);
    const long double vx[4] = {wr, -wi, -wr, wi};   // w / R
    const long double vy[4] = {wi, wr, -wi, -wr};
    int best = 0;
    for (int c = 1; c < 4; ++c)
        if (vx[c] > vx[best]) best = c;
    *code = best;
    *r = vx[best];
    *tau = vy[best] / vx[best];
}

size_t twiddle_bytes(int logTW) { return 2 * sizeof(double2) * ((size_t)1 << logTW) + kTwExtraBytes; }

void fill_twiddles(int logTW, std::vector<unsigned char> &out) {
    const long N = 1L << logTW;
    out.assign(twiddle_bytes(logTW), 0);
    double2 *tw = (double2 *)out.data();
    // and the plain entries in tangent form, the rotation from tan_code
    double2 *tt = (double2 *)(out.data() + sizeof(double2) * (size_t)N + kTwExtraBytes);
    for (long t = 0; t < N; ++t) {
        long double wr, wi;
        unit_root_ld(t, N, &wr, &wi);
        tw[t] = make_double2((double)wr, (double)wi);
        const long double vx[4] = {wr, -wi, -wr, wi};   // w / R
        const long double vy[4] = {wi, wr, -wi, -wr};
        const int c = tan_code(t, logTW);
        tt[t] = make_double2((double)(vy[c] / vx[c]), (double)vx[c]);
    }
    // set 0: twiddles w^j; sets 1 and 2: w^{j + 1/2} and w^{j - 1/2}, the angle
    // (2j + sigma) over twice the group size
    for (int set = 0; set < 3; ++set) {
        const long sigma = set == 0 ? 0 : (set == 1 ? 1 : -1);
        const long m = set == 0 ? 1 : 2;   // angle numerator 2j + sigma over 2N when shifted
        unsigned char *base = out.data() + sizeof(double2) * (size_t)N + (size_t)set * kTwSetBytes;
        GTw *r4 = (GTw *)base;
        base += sizeof(GTw) * 2 * kTwMaxH4;
        int *r4c = (int *)base;
        base += sizeof(int) * 2 * kTwMaxH4;
        double2 *r2 = (double2 *)base;
        base += sizeof(double2) * 2 * kTwMaxH2;
        int *r2c = (int *)base;
        for (long h = 1; h <= kTwMaxH4; h *= 4) {
            for (long j = 0; j < h; ++j) {
                const long t = m * j + sigma;
                int c1, c2, c3;
                long double a1, t1, a2, t2, a3, t3;
                tangent_form(t, m * 4 * h, &c1, &a1, &t1);
                tangent_form(2 * t, m * 4 * h, &c2, &a2, &t2);
                tangent_form(3 * t, m * 4 * h, &c3, &a3, &t3);
                r4[h + j].a = make_double2((double)t1, (double)a1);
                r4[h + j].b = make_double2((double)t2, (double)a2);
                r4[h + j].c = make_double2((double)t3, (double)(a3 / a1));
                r4c[h + j] = c1 | (c2 << 2) | (c3 << 4);
            }
        }
        for (long h = 1; h <= kTwMaxH2; h *= 4) {
            for (long j = 0; j < h; ++j) {
                int c;
                long double a, t;
                tangent_form(m * j + sigma, m * 2 * h, &c, &a, &t);
                r2[h + j] = make_double2((double)t, (double)a);
                r2c[h + j] = c;
            }
        }
    }
}

}  // namespace icmg
