// tune.cpp -- the tuner table (the analogue of the reference's FFTW wisdom,
// src/cpu/icm.c:184-192) and the search that fills it.
//
// The table maps a size class of tournaments to the choices that shape the
// tree: the leaf block size B and the child degree at which tree levels
// switch from schoolbook to FFT products (fft_min_degree), and per tree level
// whether an untruncated FFT level may be carried in the frequency domain
// (spectral) or stays on coefficients, and the complex points per CTA of its
// one-CTA FFT launches.  A size class is (ceil(log2 n), k/n bucket) with
// buckets k/n <= 1/64, <= 1/8, <= 1/2, > 1/2.  The search times every
// (B, fft_min_degree) pair on the caller's stacks and payouts (CUDA events
// around the kernel sequence, best of several runs), keeps the fastest, then
// walks the levels of that tree from the bottom up and keeps a level's
// alternative (coefficients instead of spectra; 1024, 2048 or 8192 points per
// CTA instead of 4096) where it is faster by more than 1%.  Results of
// different level kinds differ by rounding only, and the points per CTA do
// not change them at all, so every choice is a pure speed decision.
//
// File format (text, one entry per line; '#' starts a comment):
//   block_size <B>            global defaults (also set by icm_gb300_set_config)
//   fft_min_degree <d>
//   q_chunk <q>
//   tune <log2n> <kbucket> <B> <fft_min_degree> <ms>
//   tune_level <log2n> <kbucket> <level> <spectral 0|1> <cta_points> <ms>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"

namespace icmg {

// bumped by every change to the table, so cached plans can tell that their
// block size or crossover may be stale
std::atomic<long> g_tune_generation{0};

namespace {
struct TuneEntry {
    int log2n, kbucket, B, fft_min;
    double ms;
};
struct LevelEntry {
    int log2n, kbucket, level, spectral, pts;
    double ms;
};
std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;
std::vector<LevelEntry> g_tune_lv;

bool valid_pts(int v) { return v == 0 || v == 1024 || v == 2048 || v == 4096 || v == 8192; }

int log2ceil(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
}  // namespace

int tune_kbucket(int n, int k) {
    const double r = (double)k / (double)n;
    return r <= 1.0 / 64 ? 0 : r <= 1.0 / 8 ? 1 : r <= 0.5 ? 2 : 3;
}

// Built-in choices for GB300, consulted after the caller's table: the
// fastest (B, fft_min_degree) of the search space measured on one GB300
// (device time per solve, Q = 256, plans resident), kept only where the
// choice also held up inside batches and VJPs.  Classes without an entry use
// B = 8, fft_min_degree = 64.
//   class (ceil log2 n, k/n bucket)   measured shape            default -> chosen (ms)
//   (16, 3)                           n = k = 65536             18.96 -> 18.86
//   (20, 0), (20, 3)                  n = 2^20, k = 1000 / n    161.8 -> 160.6, 380.0 -> 376.5
// Crossover 128 was faster for single solves of n = 3000-20000 at k = 0.15 n
// (up to 6%), but made the 4096-tournament batch slower (2.133 -> 2.200 s:
// more schoolbook levels, which pack worse in work lists) and the n = 16384,
// k = 2000 VJP slower, so those classes keep the defaults.
namespace {
const TuneEntry kBuiltin[] = {{16, 3, 4, 64, 0.0}, {20, 0, 4, 64, 0.0}, {20, 3, 4, 64, 0.0}};
}

void tune_builtin(int n, int k, int *B, int *fft_min) {
    *B = 0;
    *fft_min = 0;
    const int ln = log2ceil(n), kb = tune_kbucket(n, k);
    for (const TuneEntry &e : kBuiltin)
        if (e.log2n == ln && e.kbucket == kb) {
            *B = e.B;
            *fft_min = e.fft_min;
        }
}

// the table's choice for (n, k); 0 where the table has no entry
void tune_lookup(int n, int k, int *B, int *fft_min) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    *B = 0;
    *fft_min = 0;
    const int ln = log2ceil(n), kb = tune_kbucket(n, k);
    for (const TuneEntry &e : g_tune)
        if (e.log2n == ln && e.kbucket == kb) {
            *B = e.B;
            *fft_min = e.fft_min;
        }
}

// the table's per-level entry for (n, k)'s class: 1 and its fields, else 0
int tune_level_lookup(int n, int k, int level, int *spectral, int *pts) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const int ln = log2ceil(n), kb = tune_kbucket(n, k);
    int found = 0;
    for (const LevelEntry &e : g_tune_lv)
        if (e.log2n == ln && e.kbucket == kb && e.level == level) {
            if (spectral) *spectral = e.spectral;
            if (pts) *pts = e.pts;
            found = 1;
        }
    return found;
}

int tune_cta_points(int n, int k, int level) {
    int sp = 1, pts = 0;
    return tune_level_lookup(n, k, level, &sp, &pts) ? pts : 0;
}

int tune_spectral_ok(int n, int k, int level) {
    int sp = 1, pts = 0;
    return tune_level_lookup(n, k, level, &sp, &pts) ? sp : 1;
}

static void put_level(int ln, int kb, int level, int spectral, int pts, double ms) {
    for (LevelEntry &e : g_tune_lv)
        if (e.log2n == ln && e.kbucket == kb && e.level == level) {
            e = {ln, kb, level, spectral, pts, ms};
            return;
        }
    g_tune_lv.push_back({ln, kb, level, spectral, pts, ms});
}

void tune_record_level(int n, int k, int level, int spectral, int pts, double ms) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ++g_tune_generation;
    put_level(log2ceil(n), tune_kbucket(n, k), level, spectral, pts, ms);
}

void tune_erase_level(int n, int k, int level) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ++g_tune_generation;
    const int ln = log2ceil(n), kb = tune_kbucket(n, k);
    g_tune_lv.erase(std::remove_if(g_tune_lv.begin(), g_tune_lv.end(),
                                   [&](const LevelEntry &e) {
                                       return e.log2n == ln && e.kbucket == kb && e.level == level;
                                   }),
                    g_tune_lv.end());
}

void tune_record(int n, int k, int B, int fft_min, double ms) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ++g_tune_generation;
    const int ln = log2ceil(n), kb = tune_kbucket(n, k);
    for (TuneEntry &e : g_tune)
        if (e.log2n == ln && e.kbucket == kb) {
            e = {ln, kb, B, fft_min, ms};
            return;
        }
    g_tune.push_back({ln, kb, B, fft_min, ms});
}

int tune_load(const char *path, std::string &err) {
    ++g_tune_generation;
    FILE *f = fopen(path, "r");
    if (!f) { err = std::string("cannot open ") + path; return -1; }
    char line[512];
    int nent = 0;
    while (fgets(line, sizeof line, f)) {
        char *hash = strchr(line, '#');
        if (hash) *hash = 0;
        char key[64];
        if (sscanf(line, "%63s", key) != 1) continue;
        long v = 0;
        if (!strcmp(key, "tune_level")) {
            int ln, kb, lev, sp, pts;
            double ms = 0.0;
            if (sscanf(line, "%*s %d %d %d %d %d %lf", &ln, &kb, &lev, &sp, &pts, &ms) >= 5 && ln >= 0 && ln < 40 &&
                kb >= 0 && kb <= 3 && lev >= 0 && lev < kMaxLevels && (sp == 0 || sp == 1) && valid_pts(pts)) {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                put_level(ln, kb, lev, sp, pts, ms);
                ++nent;
            }
        } else if (!strcmp(key, "tune")) {
            int ln, kb, B, fm;
            double ms = 0.0;
            if (sscanf(line, "%*s %d %d %d %d %lf", &ln, &kb, &B, &fm, &ms) >= 4 && ln >= 0 && ln < 40 && kb >= 0 &&
                kb <= 3 && (B == 4 || B == 8 || B == 16 || B == 32) && fm >= 1) {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                bool found = false;
                for (TuneEntry &e : g_tune)
                    if (e.log2n == ln && e.kbucket == kb) { e = {ln, kb, B, fm, ms}; found = true; }
                if (!found) g_tune.push_back({ln, kb, B, fm, ms});
                ++nent;
            }
        } else if (sscanf(line, "%*s %ld", &v) == 1) {
            if (!strcmp(key, "block_size")) g_config.block_size = (int)v;
            else if (!strcmp(key, "fft_min_degree")) g_config.fft_min_degree = (int)v;
            else if (!strcmp(key, "q_chunk")) g_config.q_chunk = (int)v;
        }
    }
    fclose(f);
    return nent;
}

int tune_save(const char *path, std::string &err) {
    FILE *f = fopen(path, "w");
    if (!f) { err = std::string("cannot write ") + path; return -1; }
    fprintf(f, "# icm_gb300 tuner table: tune <ceil log2 n> <k/n bucket 0..3> <block size> <fft_min_degree> <ms>\n");
    fprintf(f, "#   tune_level <ceil log2 n> <k/n bucket> <level> <spectral 0|1> <cta_points> <ms>\n");
    if (g_config.block_size > 0) fprintf(f, "block_size %d\n", g_config.block_size);
    if (g_config.fft_min_degree > 0) fprintf(f, "fft_min_degree %d\n", g_config.fft_min_degree);
    if (g_config.q_chunk > 0) fprintf(f, "q_chunk %d\n", g_config.q_chunk);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const TuneEntry &e : g_tune) fprintf(f, "tune %d %d %d %d %.6f\n", e.log2n, e.kbucket, e.B, e.fft_min, e.ms);
    for (const LevelEntry &e : g_tune_lv)
        fprintf(f, "tune_level %d %d %d %d %d %.6f\n", e.log2n, e.kbucket, e.level, e.spectral, e.pts, e.ms);
    fclose(f);
    return (int)(g_tune.size() + g_tune_lv.size());
}

void tune_clear() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    ++g_tune_generation;
    g_tune.clear();
    g_tune_lv.clear();
}

// best device ms of a plan over `runs` timed runs after one warm-up; <0 on error
static double time_plan(int n, const double *S, int Q, const double *payout, int k, int runs, std::vector<double> &out,
                        std::string &err, Plan **keep = nullptr) {
    Plan *p = plan_create(n, S, k, nullptr, err);
    if (!p) return -1.0;
    double t = 1e300;
    for (int r = 0; r <= std::max(1, runs); ++r) {   // first run warms caches and pools
        if (plan_run(p, Q, payout, out.data(), nullptr, err) != 0) {
            plan_destroy(p);
            return -1.0;
        }
        if (r) t = std::min(t, p->last_device_ms);
    }
    if (keep) *keep = p;
    else plan_destroy(p);
    return t;
}

// Time every (B, fft_min_degree) candidate on (S, payout) and record the
// best; then, on that tree, try each FFT level's alternatives bottom-up and
// record those that are faster by more than 1%.
int tune_search(int n, const double *S, int Q, const double *payout, int k, int runs, int *bestB, int *best_fft,
                double *best_ms, std::string &err) {
    static const int kB[] = {4, 8, 16};
    static const int kF[] = {16, 32, 64, 128};
    const IcmGb300Config saved = g_config;
    std::vector<double> out(n);
    double best = 1e300;
    int bB = 0, bF = 0;
    for (int L = 0; L < kMaxLevels; ++L) tune_erase_level(n, k, L);   // searched afresh
    for (int B : kB) {
        for (int F : kF) {
            g_config.block_size = B;
            g_config.fft_min_degree = F;
            const double t = time_plan(n, S, Q, payout, k, runs, out, err);
            if (t < 0) { g_config = saved; return -1; }
            if (t < best) { best = t; bB = B; bF = F; }
        }
    }
    // per-level alternatives on the chosen tree (the configuration's own
    // per-level override is off while searching)
    g_config.block_size = bB;
    g_config.fft_min_degree = bF;
    g_config.cta_points = 0;
    Plan *shape = nullptr;
    if (time_plan(n, S, Q, payout, k, 0, out, err, &shape) < 0) { g_config = saved; return -1; }
    const int L = shape->L;
    std::vector<int> kinds(L);
    for (int l = 0; l < L; ++l) kinds[l] = shape->lv[l].kind;
    plan_destroy(shape);
    for (int l = 1; l < L; ++l) {
        if (kinds[l] != 2) continue;   // the choices below concern spectral levels
        struct Cand { int sp, pts; };
        const Cand cands[] = {{1, 1024}, {1, 2048}, {1, 8192}, {0, 0}};
        int keep_sp = 1, keep_pts = 0;
        for (const Cand &c : cands) {
            tune_record_level(n, k, l, c.sp, c.pts, 0.0);
            const double t = time_plan(n, S, Q, payout, k, runs, out, err);
            if (t < 0) { tune_erase_level(n, k, l); g_config = saved; return -1; }
            if (t < 0.99 * best) { best = t; keep_sp = c.sp; keep_pts = c.pts; }
        }
        if (keep_sp == 1 && keep_pts == 0) tune_erase_level(n, k, l);
        else tune_record_level(n, k, l, keep_sp, keep_pts, best);
    }
    g_config = saved;
    tune_record(n, k, bB, bF, best);
    *bestB = bB;
    *best_fft = bF;
    *best_ms = best;
    return 0;
}

}  // namespace icmg
