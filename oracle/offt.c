/*
 * offt.c -- FP64 mixed-radix FFT for the CPU oracle (test infrastructure only;
 * see offt.h).  Self-sorting Stockham formulation: each stage reads R inputs
 * at stride m/R, applies the stage twiddles, does an R-point DFT and writes
 * the results at stride Ns (the length already transformed), so input and
 * output are both in natural order and no bit reversal is needed.
 *
 * Twiddles are tabulated once per plan in long double and rounded to double,
 * using the symmetry of the unit circle so every table entry comes from an
 * argument in [0, pi/4].
 */
#include "offt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct offt_plan {
    int n;            /* logical size */
    int real;         /* 1 = real plan */
    int m;            /* size of the complex transform actually run */
    int nf;
    int fac[64];
    double *tw;       /* e^{-2 pi i t/m}, t < m, interleaved re/im */
    double *rtw;      /* real even plans: e^{-2 pi i f/n}, f <= n/2 */
    struct offt_plan *sub;
};

/* e^{-2 pi i t / n}: the angle is folded into [0, pi/4] with exact integer
 * reflections before calling the long-double sine/cosine. */
static void unit_root(long t, long n, double *re, double *im) {
    static const long double two_pi = 6.283185307179586476925286766559005768L;
    t %= n;
    if (t < 0) t += n;
    int conj = 0, neg_c = 0;
    if (2 * t > n) { t = n - t; conj = 1; }          /* theta in [0, pi]     */
    long num = t, den = n;                            /* theta = 2 pi num/den */
    if (4 * t > n) { num = n - 2 * t; den = 2 * n; neg_c = 1; }  /* pi - theta */
    long double c, s;
    if (8 * num > den) {                              /* (pi/4, pi/2]          */
        long double b = two_pi * (long double)(den - 4 * num) / (4.0L * (long double)den);
        c = sinl(b); s = cosl(b);
    } else {
        long double a = two_pi * (long double)num / (long double)den;
        c = cosl(a); s = sinl(a);
    }
    if (neg_c) c = -c;
    *re = (double)c;
    *im = conj ? (double)s : (double)(-s);
}

static int factorise(int m, int *fac) {
    int nf = 0;
    while (m % 4 == 0) { fac[nf++] = 4; m /= 4; }
    static const int primes[] = {2, 3, 5, 7};
    for (int i = 0; i < 4; i++)
        while (m % primes[i] == 0) { fac[nf++] = primes[i]; m /= primes[i]; }
    for (int p = 11; m > 1; p += 2)
        while (m % p == 0) { fac[nf++] = p; m /= p; }
    return nf;
}

static offt_plan *plan_complex(int m) {
    offt_plan *p = (offt_plan *)calloc(1, sizeof(offt_plan));
    p->n = m;
    p->m = m;
    p->nf = factorise(m, p->fac);
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)(m > 0 ? m : 1));
    for (int t = 0; t < m; t++) unit_root(t, m, &p->tw[2 * t], &p->tw[2 * t + 1]);
    return p;
}

offt_plan *offt_plan_c2c(int n) {
    if (n < 1) return NULL;
    return plan_complex(n);
}

offt_plan *offt_plan_real(int n) {
    if (n < 1) return NULL;
    offt_plan *p = (offt_plan *)calloc(1, sizeof(offt_plan));
    p->n = n;
    p->real = 1;
    if (n % 2 == 0 && n >= 2) {
        p->m = n / 2;
        p->sub = plan_complex(n / 2);
        p->rtw = (double *)malloc(sizeof(double) * 2 * (size_t)(n / 2 + 1));
        for (int f = 0; f <= n / 2; f++) unit_root(f, n, &p->rtw[2 * f], &p->rtw[2 * f + 1]);
    } else {
        p->m = n;
        p->sub = plan_complex(n);
    }
    return p;
}

int offt_size(const offt_plan *p) { return p ? p->n : 0; }

int offt_real_scratch(int n) { return 6 * n + 16; }

void offt_destroy(offt_plan *p) {
    if (!p) return;
    if (p->sub) offt_destroy(p->sub);
    free(p->tw);
    free(p->rtw);
    free(p);
}

/* One Stockham pass of radix R over m points: x -> y. */
static void stage(const offt_plan *p, int R, int Ns, const double *x, double *y,
                  int sign) {
    const int m = p->m;
    const int stride = m / R;
    const int twstep = m / (Ns * R);
    double vr[64], vi[64], wr[64], wi[64];
    for (int j = 0; j < stride; j++) {
        const int k = j % Ns;
        for (int r = 0; r < R; r++) {
            double a = x[2 * (j + r * stride)], b = x[2 * (j + r * stride) + 1];
            if (r > 0 && k > 0) {
                long t = ((long)k * r * twstep) % m;
                double c = p->tw[2 * t], s = p->tw[2 * t + 1];
                if (sign > 0) s = -s;
                double na = a * c - b * s;
                double nb = a * s + b * c;
                a = na; b = nb;
            }
            vr[r] = a; vi[r] = b;
        }
        if (R == 2) {
            wr[0] = vr[0] + vr[1]; wi[0] = vi[0] + vi[1];
            wr[1] = vr[0] - vr[1]; wi[1] = vi[0] - vi[1];
        } else if (R == 4) {
            double s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
            double d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
            double s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
            double d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
            /* forward: multiply d1 by -i; backward by +i */
            double rr = (sign < 0) ? d1i : -d1i;
            double ri = (sign < 0) ? -d1r : d1r;
            wr[0] = s0r + s1r; wi[0] = s0i + s1i;
            wr[2] = s0r - s1r; wi[2] = s0i - s1i;
            wr[1] = d0r + rr;  wi[1] = d0i + ri;
            wr[3] = d0r - rr;  wi[3] = d0i - ri;
        } else {
            const int rstep = m / R;
            for (int kk = 0; kk < R; kk++) {
                double sr = 0.0, si = 0.0;
                for (int r = 0; r < R; r++) {
                    long t = ((long)r * kk % R) * rstep;
                    double c = p->tw[2 * t], s = p->tw[2 * t + 1];
                    if (sign > 0) s = -s;
                    sr += vr[r] * c - vi[r] * s;
                    si += vr[r] * s + vi[r] * c;
                }
                wr[kk] = sr; wi[kk] = si;
            }
        }
        const int idxD = (j / Ns) * Ns * R + k;
        for (int r = 0; r < R; r++) {
            y[2 * (idxD + r * Ns)] = wr[r];
            y[2 * (idxD + r * Ns) + 1] = wi[r];
        }
    }
}

void offt_exec_c2c(const offt_plan *p, const double *in, double *out, int sign,
                   double *scratch) {
    const int m = p->m;
    double *a = scratch, *b = scratch + 2 * (size_t)m;
    memcpy(a, in, sizeof(double) * 2 * (size_t)m);
    int Ns = 1;
    for (int s = 0; s < p->nf; s++) {
        stage(p, p->fac[s], Ns, a, b, sign);
        double *t = a; a = b; b = t;
        Ns *= p->fac[s];
    }
    memcpy(out, a, sizeof(double) * 2 * (size_t)m);
}

void offt_exec_r2c(const offt_plan *p, const double *in, double *out,
                   double *scratch) {
    const int n = p->n;
    if (n % 2 != 0 || n < 2) {
        double *z = scratch + 4 * (size_t)n;
        for (int t = 0; t < n; t++) { z[2 * t] = in[t]; z[2 * t + 1] = 0.0; }
        double *Z = scratch + 4 * (size_t)n; /* transform in place through scratch */
        offt_exec_c2c(p->sub, z, Z, -1, scratch);
        for (int f = 0; f <= n / 2; f++) { out[2 * f] = Z[2 * f]; out[2 * f + 1] = Z[2 * f + 1]; }
        return;
    }
    const int h = n / 2;
    double *Z = scratch + 4 * (size_t)h;
    /* z[t] = x[2t] + i x[2t+1] */
    offt_exec_c2c(p->sub, in, Z, -1, scratch);
    for (int f = 0; f <= h; f++) {
        int f1 = f % h, f2 = (h - f) % h;
        double zr = Z[2 * f1], zi = Z[2 * f1 + 1];
        double cr = Z[2 * f2], ci = -Z[2 * f2 + 1];   /* conj(Z[h-f]) */
        double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
        /* O = (Z - conj Z')/(2i) */
        double dr = zr - cr, di = zi - ci;
        double or_ = 0.5 * di, oi = -0.5 * dr;
        double wr = p->rtw[2 * f], wi = p->rtw[2 * f + 1];
        out[2 * f] = er + (or_ * wr - oi * wi);
        out[2 * f + 1] = ei + (or_ * wi + oi * wr);
    }
}

void offt_exec_c2r(const offt_plan *p, const double *in, double *out,
                   double *scratch) {
    const int n = p->n;
    if (n % 2 != 0 || n < 2) {
        double *z = scratch + 4 * (size_t)n;
        for (int f = 0; f < n; f++) {
            if (f <= n / 2) { z[2 * f] = in[2 * f]; z[2 * f + 1] = in[2 * f + 1]; }
            else { z[2 * f] = in[2 * (n - f)]; z[2 * f + 1] = -in[2 * (n - f) + 1]; }
        }
        if (n >= 1) z[1] = 0.0;
        offt_exec_c2c(p->sub, z, z, +1, scratch);
        for (int t = 0; t < n; t++) out[t] = z[2 * t];
        return;
    }
    const int h = n / 2;
    double *U = scratch + 4 * (size_t)h;
    for (int f = 0; f < h; f++) {
        double xr = in[2 * f], xi = in[2 * f + 1];
        double yr = in[2 * (h - f)], yi = -in[2 * (h - f) + 1];   /* conj(X[h-f]) */
        if (f == 0) { xi = 0.0; yi = 0.0; }
        double er = xr + yr, ei = xi + yi;
        double dr = xr - yr, di = xi - yi;
        /* O = (X - conj X') * e^{+2 pi i f/n} */
        double wr = p->rtw[2 * f], wi = -p->rtw[2 * f + 1];
        double or_ = dr * wr - di * wi, oi = dr * wi + di * wr;
        /* U = E + i O */
        U[2 * f] = er - oi;
        U[2 * f + 1] = ei + or_;
    }
    /* in-place through the c2c scratch */
    double *u = U;
    offt_exec_c2c(p->sub, U, u, +1, scratch);
    for (int t = 0; t < h; t++) { out[2 * t] = u[2 * t]; out[2 * t + 1] = u[2 * t + 1]; }
}
