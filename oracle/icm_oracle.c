/*
 * icm_oracle.c -- CPU restatement of the reference's ICM quadrature engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GB300
 * library: tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
 * may call it; the product (icm_gb300/, libicm_gb300.so) never links,
 * loads or calls it.
 *
 * Algorithm followed (reference paths, relative to the Sarose550/ICM tree):
 *   quadrature nodes        src/cpu/icm.c:117-132   (log_Phi, make_nodes)
 *   stack sort              src/cpu/icm.c:2138-2143 (descending); ties broken
 *                           by index as src/gpu/gpu_plan.cu:405-409 does
 *   leaf factors            src/cpu/icm.c:2575-2581 (a = exp(S logv), 0 below -700)
 *   block products          src/cpu/icm.c:2199-2218
 *   tree build              src/cpu/icm.c:1605-1654 (truncated products, root skipped)
 *   propagate               src/cpu/icm.c:1667-1819 (middle products, hot/cold pruning)
 *   divide + dot            src/cpu/icm.c:2230-2302 (forward a>0.5, backward a>1e-15, else shift)
 *   accumulate              src/cpu/icm.c:2584-2589 (non-finite weight -> 0)
 *   subset hot mask         src/cpu/icm.c:2430-2473
 *   closed forms V1, V2     src/cpu/icm.c:145-170
 *
 * Tree geometry is stated in exact-arithmetic terms rather than copied from
 * icm.c's padded layout: a node at level l covers up to B*2^l players; its
 * polynomial keeps min(deg+1, k) coefficients and its g vector min(deg, k)
 * entries.  Coefficients of index >= k never meet a non-zero payout, so
 * this truncation is exact (the reference truncates at k_pad >= k, which is
 * the same in exact arithmetic).  Products use schoolbook arithmetic below
 * `fft_min_deg` and a real FFT of power-of-two size above it.
 */
#include "offt.h"

#include <alloca.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_LEVELS 40

/* ---------------------------------------------------------------- nodes */

static double log_Phi(double y) {
    if (y >= 0) return log1p(-erfc(y / sqrt(2.0)) / 2.0);
    return log(erfc(-y / sqrt(2.0)) / 2.0);
}

void oracle_make_nodes(int Q, double Smax, double *logv, double *w) {
    double y_lo = -7.7;
    double y_hi = sqrt(2.0) * sqrt(log(Smax) + 25.0);
    if (y_hi < 6.5) y_hi = 6.5;
    double h = (y_hi - y_lo) / (Q - 1);
    for (int q = 0; q < Q; q++) {
        double y = y_lo + q * h;
        logv[q] = log_Phi(y);
        w[q] = h * exp(-0.5 * y * y) / sqrt(2 * M_PI);
    }
}

/* ----------------------------------------------------------------- sort */

static const double *g_sort_S;
static int cmp_desc(const void *a, const void *b) {
    int ia = *(const int *)a, ib = *(const int *)b;
    double sa = g_sort_S[ia], sb = g_sort_S[ib];
    if (sa > sb) return -1;
    if (sa < sb) return 1;
    return (ia > ib) - (ia < ib);
}

void oracle_sort_desc(int n, const double *S, int *perm) {
    for (int i = 0; i < n; i++) perm[i] = i;
    g_sort_S = S;
    qsort(perm, (size_t)n, sizeof(int), cmp_desc);
}

/* ------------------------------------------------------------- geometry */

typedef struct {
    int n, k, B, nblocks, L;              /* L levels: 0 (leaves) .. L-1 (root) */
    int nn[ORACLE_MAX_LEVELS];            /* node slots per level (power of 2) */
    int nreal[ORACLE_MAX_LEVELS];         /* real nodes per level */
    long deg[ORACLE_MAX_LEVELS];          /* max players under a node */
    int plen[ORACLE_MAX_LEVELS];          /* polynomial coefficients kept */
    int glen[ORACLE_MAX_LEVELS];          /* g entries kept */
    int fftn[ORACLE_MAX_LEVELS];          /* FFT size at parent level l (0 = schoolbook) */
    size_t poff[ORACLE_MAX_LEVELS], goff[ORACLE_MAX_LEVELS];
    size_t ptotal, gtotal;
} Geom;

static int next_pow2(long v) { int p = 1; while (p < v) p <<= 1; return p; }

static void geom_init(Geom *G, int n, int k, int B, int fft_min_deg) {
    memset(G, 0, sizeof(*G));
    G->n = n; G->k = k; G->B = B;
    G->nblocks = (n + B - 1) / B;
    int Nt = next_pow2(G->nblocks);
    int L = 1;
    while ((1 << (L - 1)) < Nt) L++;
    G->L = L;
    size_t po = 0, go = 0;
    for (int l = 0; l < L; l++) {
        G->nn[l] = Nt >> l;
        G->nreal[l] = (l == 0) ? G->nblocks : (G->nreal[l - 1] + 1) / 2;
        G->deg[l] = (long)B << l;
        G->plen[l] = (int)((G->deg[l] + 1 < k) ? G->deg[l] + 1 : k);
        G->glen[l] = (int)((G->deg[l] < k) ? G->deg[l] : k);
        G->poff[l] = po; po += (size_t)G->nreal[l] * G->plen[l];
        G->goff[l] = go; go += (size_t)G->nreal[l] * G->glen[l];
        G->fftn[l] = 0;
        if (l >= 1 && fft_min_deg > 0 && G->deg[l - 1] >= fft_min_deg) {
            int lc = G->plen[l - 1], gc = G->glen[l - 1];
            long need = 2L * lc - 2;
            if (gc + lc - 1 > need) need = gc + lc - 1;
            G->fftn[l] = next_pow2(need);
        }
    }
    G->ptotal = po; G->gtotal = go;
}

/* ------------------------------------------------------ per-thread state */

typedef struct {
    double *a, *blockP, *P, *g, *inner;
    offt_plan *plan[ORACLE_MAX_LEVELS];
    double *fa, *fb, *fg, *rb, *scratch;
    int maxfft;
} Work;

static void work_init(Work *W, const Geom *G) {
    memset(W, 0, sizeof(*W));
    W->a = (double *)malloc(sizeof(double) * (size_t)G->n);
    W->inner = (double *)malloc(sizeof(double) * (size_t)G->n);
    W->blockP = (double *)calloc((size_t)G->nblocks * (G->B + 1), sizeof(double));
    W->P = (double *)calloc(G->ptotal + 1, sizeof(double));
    W->g = (double *)calloc(G->gtotal + 1, sizeof(double));
    int mx = 2;
    for (int l = 1; l < G->L; l++)
        if (G->fftn[l]) {
            W->plan[l] = offt_plan_real(G->fftn[l]);
            if (G->fftn[l] > mx) mx = G->fftn[l];
        }
    W->maxfft = mx;
    W->fa = (double *)malloc(sizeof(double) * (size_t)(mx + 2));
    W->fb = (double *)malloc(sizeof(double) * (size_t)(mx + 2));
    W->fg = (double *)malloc(sizeof(double) * (size_t)(mx + 2));
    W->rb = (double *)malloc(sizeof(double) * (size_t)(mx + 2));
    W->scratch = (double *)malloc(sizeof(double) * (size_t)offt_real_scratch(mx));
}

static void work_free(Work *W, const Geom *G) {
    for (int l = 0; l < G->L; l++) offt_destroy(W->plan[l]);
    free(W->a); free(W->inner); free(W->blockP); free(W->P); free(W->g);
    free(W->fa); free(W->fb); free(W->fg); free(W->rb); free(W->scratch);
}

/* ------------------------------------------------------------ kernels */

/* c = a*b mod x^lp, a and b of length lc (icm.c:465-480 polymul_modk) */
static void mul_school(const double *a, const double *b, int lc, double *c, int lp) {
    memset(c, 0, sizeof(double) * (size_t)lp);
    for (int i = 0; i < lc && i < lp; i++) {
        double ai = a[i];
        int jmax = lc;
        if (i + jmax > lp) jmax = lp - i;
        for (int j = 0; j < jmax; j++) c[i + j] += ai * b[j];
    }
}

/* out[m] = sum_j P[j] g[m+j], g zero beyond lg (icm.c:489-507 correlate_school) */
static void corr_school(const double *g, int lg, const double *P, int lp, double *out, int lo) {
    for (int m = 0; m < lo; m++) {
        double s = 0.0;
        int jmax = lp;
        if (m + jmax > lg) jmax = lg - m;
        for (int j = 0; j < jmax; j++) s += P[j] * g[m + j];
        out[m] = s;
    }
}

static void spec_of(Work *W, int l, int N, const double *x, int lx, double *X) {
    memcpy(W->rb, x, sizeof(double) * (size_t)lx);
    memset(W->rb + lx, 0, sizeof(double) * (size_t)(N - lx));
    offt_exec_r2c(W->plan[l], W->rb, X, W->scratch);
}

/* FFT product with the two end coefficients taken directly */
static void mul_fft(Work *W, int l, const double *a, const double *b, int lc, double *c, int lp) {
    int N = W->plan[l] ? offt_size(W->plan[l]) : 0;
    spec_of(W, l, N, a, lc, W->fa);
    spec_of(W, l, N, b, lc, W->fb);
    for (int f = 0; f <= N / 2; f++) {
        double ar = W->fa[2 * f], ai = W->fa[2 * f + 1];
        double br = W->fb[2 * f], bi = W->fb[2 * f + 1];
        W->fg[2 * f] = ar * br - ai * bi;
        W->fg[2 * f + 1] = ar * bi + ai * br;
    }
    offt_exec_c2r(W->plan[l], W->fg, W->rb, W->scratch);
    double inv = 1.0 / N;
    int lim = lp < N ? lp : N;
    for (int t = 0; t < lim; t++) c[t] = W->rb[t] * inv;
    for (int t = lim; t < lp; t++) c[t] = 0.0;
    c[0] = a[0] * b[0];
    if (lp > N) c[N] = a[lc - 1] * b[lc - 1];   /* only when 2*lc-2 == N */
}

/* out[m] = sum_j P[j] g[m+j] through an FFT of size N >= lo + lP - 1 */
static void corr_fft(Work *W, int l, const double *G, const double *P, int lP, double *out, int lo) {
    int N = offt_size(W->plan[l]);
    spec_of(W, l, N, P, lP, W->fa);
    for (int f = 0; f <= N / 2; f++) {
        double gr = G[2 * f], gi = G[2 * f + 1];
        double pr = W->fa[2 * f], pi = W->fa[2 * f + 1];
        W->fb[2 * f] = gr * pr + gi * pi;        /* G * conj(P) */
        W->fb[2 * f + 1] = gi * pr - gr * pi;
    }
    offt_exec_c2r(W->plan[l], W->fb, W->rb, W->scratch);
    double inv = 1.0 / N;
    for (int m = 0; m < lo; m++) out[m] = W->rb[m] * inv;
}

/* --------------------------------------------------------------- engine */

static void run_node(const Geom *G, Work *W, const double *S_sorted, double logv,
                     const double *payout, uint8_t *const *hot, const uint8_t *active) {
    const int n = G->n, k = G->k, B = G->B;
    double *a = W->a;
    for (int i = 0; i < n; i++) {
        double arg = S_sorted[i] * logv;
        a[i] = (arg < -700) ? 0 : exp(arg);
    }
    /* leaves: block products (icm.c:2199-2224) */
    for (int b = 0; b < G->nblocks; b++) {
        int start = b * B, end = start + B;
        if (end > n) end = n;
        int bs = end - start;
        double *P = W->blockP + (size_t)b * (B + 1);
        memset(P, 0, sizeof(double) * (size_t)(B + 1));
        P[0] = 1.0;
        for (int j = start; j < end; j++) {
            double aj = a[j], bj = 1 - aj;
            for (int m = bs; m >= 1; m--) P[m] = aj * P[m] + bj * P[m - 1];
            P[0] *= aj;
        }
        double *leaf = W->P + G->poff[0] + (size_t)b * G->plen[0];
        int cp = B + 1 < G->plen[0] ? B + 1 : G->plen[0];
        memcpy(leaf, P, sizeof(double) * (size_t)cp);
        for (int t = cp; t < G->plen[0]; t++) leaf[t] = 0.0;
    }
    /* build levels 1..L-2; the root product is never read (icm.c:1605-1654) */
    for (int l = 1; l < G->L - 1; l++) {
        int lc = G->plen[l - 1], lp = G->plen[l];
        for (int j = 0; j < G->nreal[l]; j++) {
            const double *Lc = W->P + G->poff[l - 1] + (size_t)(2 * j) * lc;
            double *out = W->P + G->poff[l] + (size_t)j * lp;
            if (2 * j + 1 >= G->nreal[l - 1]) {
                int cp = lc < lp ? lc : lp;
                memcpy(out, Lc, sizeof(double) * (size_t)cp);
                for (int t = cp; t < lp; t++) out[t] = 0.0;
            } else {
                const double *Rc = Lc + lc;
                if (G->fftn[l]) mul_fft(W, l, Lc, Rc, lc, out, lp);
                else mul_school(Lc, Rc, lc, out, lp);
            }
        }
    }
    /* propagate (icm.c:1667-1819) */
    {
        int top = G->L - 1;
        double *groot = W->g + G->goff[top];
        int gl = G->glen[top];
        for (int m = 0; m < gl; m++) groot[m] = (m < k) ? payout[m] : 0.0;
    }
    for (int l = G->L - 1; l >= 1; l--) {
        int lc = G->plen[l - 1], gc = G->glen[l - 1], gp = G->glen[l];
        const uint8_t *hc = hot ? hot[l - 1] : NULL;
        for (int j = 0; j < G->nreal[l]; j++) {
            const double *gpar = W->g + G->goff[l] + (size_t)j * gp;
            double *gL = W->g + G->goff[l - 1] + (size_t)(2 * j) * gc;
            int right = (2 * j + 1 < G->nreal[l - 1]);
            int lhot = !hc || hc[2 * j];
            int rhot = right && (!hc || hc[2 * j + 1]);
            if (!right) {
                if (lhot) {
                    int cp = gc < gp ? gc : gp;
                    memcpy(gL, gpar, sizeof(double) * (size_t)cp);
                    for (int t = cp; t < gc; t++) gL[t] = 0.0;
                } else {
                    memset(gL, 0, sizeof(double) * (size_t)gc);
                }
                continue;
            }
            double *gR = gL + gc;
            const double *PL = W->P + G->poff[l - 1] + (size_t)(2 * j) * lc;
            const double *PR = PL + lc;
            if (G->fftn[l] && (lhot || rhot)) {
                int N = offt_size(W->plan[l]);
                spec_of(W, l, N, gpar, gp, W->fg);
                if (lhot) corr_fft(W, l, W->fg, PR, lc, gL, gc); else memset(gL, 0, sizeof(double) * (size_t)gc);
                if (rhot) corr_fft(W, l, W->fg, PL, lc, gR, gc); else memset(gR, 0, sizeof(double) * (size_t)gc);
            } else {
                if (lhot) corr_school(gpar, gp, PR, lc, gL, gc); else memset(gL, 0, sizeof(double) * (size_t)gc);
                if (rhot) corr_school(gpar, gp, PL, lc, gR, gc); else memset(gR, 0, sizeof(double) * (size_t)gc);
            }
        }
    }
    /* divide + dot (icm.c:2230-2302) */
    const double *gleaf = W->g + G->goff[0];
    int gl0 = G->glen[0];
    double *Qarr = (double *)alloca(sizeof(double) * (size_t)(B + 1));
    for (int b = 0; b < G->nblocks; b++) {
        int start = b * B, end = start + B;
        if (end > n) end = n;
        int bs = end - start;
        if (active) {
            int any = 0;
            for (int j = start; j < end; j++) if (active[j]) { any = 1; break; }
            if (!any) { for (int j = start; j < end; j++) W->inner[j] = 0.0; continue; }
        }
        const double *P = W->blockP + (size_t)b * (B + 1);
        const double *g = gleaf + (size_t)b * gl0;
        int pk = bs < k ? bs : k;
        for (int jj = 0; jj < bs; jj++) {
            int i = start + jj;
            if (active && !active[i]) { W->inner[i] = 0.0; continue; }
            double ai = a[i], bi = 1 - ai, eq = 0.0;
            if (ai > 0.5) {
                double ia = 1.0 / ai, c = -bi * ia;
                double Qv = P[0] * ia;
                eq = g[0] * Qv;
                for (int m = 1; m < pk; m++) { Qv = c * Qv + P[m] * ia; eq += g[m] * Qv; }
            } else if (ai > 1e-15) {
                double ib = 1.0 / bi, c = -ai * ib;
                double Qp = P[bs] * ib;
                Qarr[bs - 1] = Qp;
                for (int m = bs - 2; m >= 0; m--) { Qp = c * Qp + P[m + 1] * ib; Qarr[m] = Qp; }
                for (int m = 0; m < pk; m++) eq += g[m] * Qarr[m];
            } else {
                for (int m = 0; m < pk; m++) eq += g[m] * P[m + 1];
            }
            W->inner[i] = eq;
        }
    }
}

/*
 * Full or subset equity (icm_equity / icm_equity_subset semantics).
 * targets == NULL: all players.  Non-target entries are written as 0.
 * Returns 0 on success, -1 on bad arguments.
 */
int oracle_equity(int n, const double *S, int Q, const double *payout, int k,
                  int B, int fft_min_deg, const int *targets, int n_targets,
                  int nthreads, double *equity) {
    if (n < 1 || k < 1 || k > n || Q < 1 || B < 1 || !S || !payout || !equity) return -1;
    if (B > n) B = n;
    int *perm = (int *)malloc(sizeof(int) * (size_t)n);
    double *Ss = (double *)malloc(sizeof(double) * (size_t)n);
    oracle_sort_desc(n, S, perm);
    double Smax = 0;
    for (int i = 0; i < n; i++) { Ss[i] = S[perm[i]]; if (S[i] > Smax) Smax = S[i]; }
    double *logv = (double *)malloc(sizeof(double) * (size_t)Q);
    double *wq = (double *)malloc(sizeof(double) * (size_t)Q);
    oracle_make_nodes(Q, Smax, logv, wq);

    Geom G;
    geom_init(&G, n, k, B, fft_min_deg);

    uint8_t *active = NULL, *hotdata = NULL;
    uint8_t *hot[ORACLE_MAX_LEVELS] = {0};
    if (targets) {
        uint8_t *act0 = (uint8_t *)calloc((size_t)n, 1);
        for (int t = 0; t < n_targets; t++)
            if (targets[t] >= 0 && targets[t] < n) act0[targets[t]] = 1;
        active = (uint8_t *)calloc((size_t)n, 1);
        for (int i = 0; i < n; i++) active[i] = act0[perm[i]];
        free(act0);
        size_t tot = 0;
        for (int l = 0; l < G.L; l++) tot += (size_t)G.nn[l];
        hotdata = (uint8_t *)calloc(tot, 1);
        uint8_t *ptr = hotdata;
        for (int l = 0; l < G.L; l++) { hot[l] = ptr; ptr += G.nn[l]; }
        for (int b = 0; b < G.nblocks; b++) {
            int s = b * B, e = s + B;
            if (e > n) e = n;
            for (int j = s; j < e; j++) if (active[j]) { hot[0][b] = 1; break; }
        }
        for (int l = 1; l < G.L; l++)
            for (int j = 0; j < G.nn[l]; j++) {
                int lft = (2 * j < G.nn[l - 1]) ? hot[l - 1][2 * j] : 0;
                int rgt = (2 * j + 1 < G.nn[l - 1]) ? hot[l - 1][2 * j + 1] : 0;
                hot[l][j] = (uint8_t)(lft | rgt);
            }
    }

    int nt = nthreads > 0 ? nthreads : 1;
#ifndef _OPENMP
    nt = 1;
#endif
    if (nt > Q) nt = Q;
    double *acc = (double *)calloc((size_t)nt * n, sizeof(double));

#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        Work W;
        work_init(&W, &G);
        double *eq = acc + (size_t)tid * n;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int q = 0; q < Q; q++) {
            if (wq[q] == 0) continue;
            run_node(&G, &W, Ss, logv[q], payout, targets ? hot : NULL, active);
            double inv_v = exp(-logv[q]);
            for (int i = 0; i < n; i++) {
                double pw = wq[q] * Ss[i] * W.a[i] * inv_v;
                if (!isfinite(pw)) pw = 0;
                eq[i] += pw * W.inner[i];
            }
        }
        work_free(&W, &G);
    }
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (int t = 0; t < nt; t++) s += acc[(size_t)t * n + i];
        equity[perm[i]] = s;
    }
    if (targets)
        for (int i = 0; i < n; i++) if (!active[i]) equity[perm[i]] = 0.0;
    free(acc); free(perm); free(Ss); free(logv); free(wq); free(active); free(hotdata);
    return 0;
}

/*
 * O(n^2)-per-node engine: full product, then divide per player
 * (icm.c:1880-1914 engine_naive_ctx), same quadrature and accumulation.
 * An independent second check of the tree engine at small n.
 */
int oracle_equity_naive(int n, const double *S, int Q, const double *payout, int k,
                        double *equity) {
    if (n < 1 || k < 1 || k > n || Q < 1) return -1;
    double Smax = 0;
    for (int i = 0; i < n; i++) if (S[i] > Smax) Smax = S[i];
    double *logv = (double *)malloc(sizeof(double) * (size_t)Q);
    double *wq = (double *)malloc(sizeof(double) * (size_t)Q);
    oracle_make_nodes(Q, Smax, logv, wq);
    double *a = (double *)malloc(sizeof(double) * (size_t)n);
    double *P = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *Qv = (double *)malloc(sizeof(double) * (size_t)n);
    memset(equity, 0, sizeof(double) * (size_t)n);
    int pk = k < n ? k : n;
    for (int q = 0; q < Q; q++) {
        if (wq[q] == 0) continue;
        for (int i = 0; i < n; i++) {
            double arg = S[i] * logv[q];
            a[i] = (arg < -700) ? 0 : exp(arg);
        }
        memset(P, 0, sizeof(double) * (size_t)(n + 1));
        P[0] = 1;
        for (int j = 0; j < n; j++) {
            double aj = a[j], bj = 1 - aj;
            for (int m = (j + 1 < n ? j + 1 : n); m >= 1; m--) P[m] = aj * P[m] + bj * P[m - 1];
            P[0] *= aj;
        }
        double inv_v = exp(-logv[q]);
        for (int i = 0; i < n; i++) {
            double ai = a[i], bi = 1 - ai;
            if (ai > 0.5) {
                double ia = 1 / ai, c = -bi * ia;
                Qv[0] = P[0] * ia;
                for (int m = 1; m < n; m++) Qv[m] = c * Qv[m - 1] + P[m] * ia;
            } else if (ai > 1e-15) {
                double ib = 1 / bi, c = -ai * ib;
                Qv[n - 1] = P[n] * ib;
                for (int m = n - 2; m >= 0; m--) Qv[m] = c * Qv[m + 1] + P[m + 1] * ib;
            } else {
                for (int m = 0; m < n; m++) Qv[m] = P[m + 1];
            }
            double e = 0;
            for (int m = 0; m < pk; m++) e += payout[m] * Qv[m];
            double pw = wq[q] * S[i] * a[i] * inv_v;
            if (!isfinite(pw)) pw = 0;
            equity[i] += pw * e;
        }
    }
    free(logv); free(wq); free(a); free(P); free(Qv);
    return 0;
}

/* ----------------------------------------------------------- closed forms */

/* V1_i = 1 + sum_{j != i} S_i/(S_i+S_j): equity under payout[m] = n-m
 * (icm.c:145-152).  Kahan-compensated. */
void oracle_v1(int n, const double *S, int n_idx, const int *idx, double *V1, int nthreads) {
    int cnt = idx ? n_idx : n;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int t = 0; t < cnt; t++) {
        int i = idx ? idx[t] : t;
        double s = 1.0, c = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double y = S[i] / (S[i] + S[j]) - c;
            double tt = s + y;
            c = (tt - s) - y;
            s = tt;
        }
        V1[t] = s;
    }
}

/* V2_i = sum_{j<l; j,l != i} S_i/(S_i+S_j+S_l): equity under payout
 * C(n-1-m, 2) (icm.c:158-170).  O(n^2) per requested index, inner sums in
 * double, outer sum Kahan-compensated. */
void oracle_v2(int n, const double *S, int n_idx, const int *idx, double *V2, int nthreads) {
    int cnt = idx ? n_idx : n;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int t = 0; t < cnt; t++) {
        int i = idx ? idx[t] : t;
        double s = 0.0, c = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double inner = 0.0, base = S[i] + S[j];
            for (int l = j + 1; l < n; l++) {
                if (l == i) continue;
                inner += S[i] / (base + S[l]);
            }
            double y = inner - c;
            double tt = s + y;
            c = (tt - s) - y;
            s = tt;
        }
        V2[t] = s;
    }
}
