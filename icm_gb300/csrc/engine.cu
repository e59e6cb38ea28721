// engine.cu -- plans (geometry, buffers) and the per-call launch sequence.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>

#include <unistd.h>

#include "engine.h"
#include "kernels.h"

namespace icmg {

IcmGb300Config g_config = {};
int g_device = -1;

// Device allocations of plans, batches and VJPs go through dev_alloc, so a
// test can make the n-th one fail as an exhausted allocator would
// (icm_gb300_test_fail_allocation); 0 = no injected failure.
static std::atomic<int> g_fail_alloc{0};
void set_alloc_failure(int nth) { g_fail_alloc.store(nth > 0 ? nth : 0); }
cudaError_t dev_alloc(void **ptr, size_t bytes, cudaStream_t st, bool pooled) {
    int c = g_fail_alloc.load();
    while (c > 0 && !g_fail_alloc.compare_exchange_weak(c, c - 1)) {}
    if (c == 1) return cudaErrorMemoryAllocation;
    return pooled ? cudaMallocAsync(ptr, bytes, st) : cudaMalloc(ptr, bytes);
}

static double now_ns() {
    return (double)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// ------------------------------------------------------------ nodes
// erfc-trapezoid rule in probit space (reference src/cpu/icm.c:117-132):
// y_q = y_lo + q h on [-7.7, max(6.5, sqrt(2) sqrt(ln Smax + 25))],
// logv_q = log Phi(y_q), w_q = h phi(y_q).
static double log_Phi(double y) {
    if (y >= 0) return std::log1p(-std::erfc(y / std::sqrt(2.0)) / 2.0);
    return std::log(std::erfc(-y / std::sqrt(2.0)) / 2.0);
}

// tanh-sinh rule on v in (0, 1) (the reference's accuracy study,
// tools/accuracy_bench.c:52-90, offered behind IcmGb300Config.quadrature):
// v = (1 + tanh t) / 2 with t = pi/2 sinh x, x = -5.5 + q h on [-5.5, 5.5],
// w = h (pi/2) cosh x / (2 cosh^2 t).  Here log v = -log1p(e^{-2t}) and
// 1 / (2 cosh^2 t) = 2 e^{-2|t|} / (1 + e^{-2|t|})^2, so both ends keep full
// precision; nodes whose weight underflows get w = 0 (skipped).  The nodes do
// not depend on the stacks.
static void make_nodes_tanh_sinh(int Q, std::vector<double> &logv, std::vector<double> &w) {
    const double x_max = 5.5;
    const double h = 2.0 * x_max / (Q - 1);
    logv.resize(Q);
    w.resize(Q);
    for (int q = 0; q < Q; ++q) {
        const double x = -x_max + q * h;
        const double t = 0.5 * M_PI * std::sinh(x);
        const double e = std::exp(-2.0 * std::fabs(t));
        logv[q] = (t >= 0) ? -std::log1p(e) : 2.0 * t - std::log1p(e);
        w[q] = h * 0.5 * M_PI * std::cosh(x) * (2.0 * e / ((1.0 + e) * (1.0 + e)));
        if (!(logv[q] < 0.0) || !std::isfinite(logv[q])) w[q] = 0.0;
    }
}

void make_nodes(int Q, double Smax, std::vector<double> &logv, std::vector<double> &w) {
    if (g_config.quadrature == 1) {
        make_nodes_tanh_sinh(Q, logv, w);
        return;
    }
    const double y_lo = -7.7;
    double y_hi = std::sqrt(2.0) * std::sqrt(std::log(Smax) + 25.0);
    if (y_hi < 6.5) y_hi = 6.5;
    const double h = (y_hi - y_lo) / (Q - 1);
    logv.resize(Q);
    w.resize(Q);
    for (int q = 0; q < Q; ++q) {
        const double y = y_lo + q * h;
        logv[q] = log_Phi(y);
        w[q] = h * std::exp(-0.5 * y * y) / std::sqrt(2 * M_PI);
    }
}

// players (sorted by stack, descending) whose leaf factor is exactly 0: the
// leaf kernel sets a = 0 when S logv < -700, a prefix since S logv grows
// along the sorted order (logv < 0; rounding of the product is monotone)
int zero_prefix(const double *S_sorted, int n, double logv) {
    int lo = 0, hi = n;   // first index with S logv >= -700
    while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (S_sorted[mid] * logv < -700.0) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------ twiddles
// tables built by twiddle.cpp; one allocation per device, grown on demand
static std::mutex g_tw_mu;
static double2 *g_tw[64] = {};   // per device
static int g_tw_log[64] = {};

const double2 *twiddles(int logN, cudaStream_t s, std::string &err, int *logTW) {
    std::lock_guard<std::mutex> lk(g_tw_mu);
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) { err = "device index out of range"; return nullptr; }
    if (g_tw[dev] && g_tw_log[dev] >= logN) { *logTW = g_tw_log[dev]; return g_tw[dev]; }
    const int L = std::max(logN, 14);
    std::vector<unsigned char> h;
    fill_twiddles(L, h);
    double2 *d = nullptr;
    cudaError_t e = cudaMalloc(&d, h.size());
    if (e != cudaSuccess) { err = std::string("twiddle table: ") + cudaGetErrorString(e); return nullptr; }
    e = cudaMemcpyAsync(d, h.data(), h.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = std::string("twiddle upload: ") + cudaGetErrorString(e); cudaFree(d); return nullptr; }
    // older tables stay allocated: plans in flight may still read them
    g_tw[dev] = d;
    g_tw_log[dev] = L;
    *logTW = L;
    return d;
}

// ------------------------------------------------------------ plans
static int pow2_ge(long v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}
static int ilog2(long v) {
    int l = 0;
    while ((1L << l) < v) ++l;
    return l;
}
static int round2(int v) { return (v + 1) & ~1; }

int select_block_size(int n, int k) {
    int B = g_config.block_size;
    if (B <= 0) {   // the tuner table's choice for this size class, the built-in one, else 8
        int tF = 0;
        tune_lookup(n, k, &B, &tF);
        if (B <= 0) tune_builtin(n, k, &B, &tF);
        if (B <= 0) B = 8;
    }
    if (B <= 4) B = 4;
    else if (B <= 8) B = 8;
    else if (B <= 16) B = 16;
    else B = 32;
    return B;
}

// complex points per CTA of level l's one-CTA FFT launches: the
// configuration's value, else the tuner table's for the level, else 4096
int select_cta_points(int n, int k, int l) {
    int v = g_config.cta_points;
    if (v <= 0) v = tune_cta_points(n, k, l);
    if (v != 1024 && v != 2048 && v != 8192) v = 4096;
    return v;
}

int select_fft_min(int n, int k) {
    if (g_config.fft_min_degree > 0) return g_config.fft_min_degree;
    int tB = 0, tF = 0;
    tune_lookup(n, k, &tB, &tF);
    if (tF <= 0) tune_builtin(n, k, &tB, &tF);
    return tF > 0 ? tF : 64;
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// host barrier for the sort's worker threads (generation counter)
namespace {
struct HostBarrier {
    std::atomic<int> count{0}, gen{0};
    int T;
    explicit HostBarrier(int t) : T(t) {}
    void wait() {
        const int g = gen.load(std::memory_order_acquire);
        if (count.fetch_add(1, std::memory_order_acq_rel) == T - 1) {
            count.store(0, std::memory_order_relaxed);
            gen.fetch_add(1, std::memory_order_acq_rel);
        } else {
            while (gen.load(std::memory_order_acquire) == g) std::this_thread::yield();
        }
    }
};

// Worker threads kept for the life of the process, parked on a condition
// variable between jobs: run(T, fn) calls fn(t) for t in [0, T), t = 0 on the
// calling thread, and returns when all have returned.  One job at a time; a
// caller that finds the pool busy (another host thread sorting) or runs in a
// forked child gets threads of its own instead.  fn must not throw.  The pool
// is never destroyed (its workers outlive static destructors at exit).
class HostPool {
  public:
    static HostPool &get() {
        static HostPool *pool = new HostPool();
        return *pool;
    }
    void run(int T, const std::function<void(int)> &fn) {
        if (T <= 1) {
            fn(0);
            return;
        }
        std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
        if (!busy.owns_lock() || getpid() != pid_) {
            std::vector<std::thread> th;
            for (int t = 1; t < T; ++t) th.emplace_back(fn, t);
            fn(0);
            for (auto &x : th) x.join();
            return;
        }
        while (nthreads_ < T - 1) {
            const int id = ++nthreads_;
            std::thread([this, id] { loop(id); }).detach();
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &fn;
            active_ = T;
            left_.store(T - 1, std::memory_order_relaxed);
            ++gen_;
        }
        cv_.notify_all();
        fn(0);
        while (left_.load(std::memory_order_acquire) > 0) std::this_thread::yield();
    }

  private:
    HostPool() : pid_(getpid()) {}
    void loop(int id) {
        long seen = 0;
        for (;;) {
            const std::function<void(int)> *f = nullptr;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (id >= active_) continue;   // not needed by this job
                f = job_;
            }
            (*f)(id);
            left_.fetch_sub(1, std::memory_order_acq_rel);
        }
    }
    std::mutex busy_, m_;
    std::condition_variable cv_;
    const std::function<void(int)> *job_ = nullptr;
    long gen_ = 0;
    int active_ = 0, nthreads_ = 0;
    std::atomic<int> left_{0};
    const pid_t pid_;
};
}  // namespace

// perm: player indices by stack, descending, ties by index.  Positive finite
// doubles order like their bit patterns, so sorting the complemented bits
// ascending, stably, gives that order.  T threads (a persistent pool) each
// take a contiguous chunk of the players:
//   1. keys, and their range: the 12 bits below the highest bit in which any
//      two keys differ form the bucket digit (the keys' common high bits and
//      everything below the digit aside);
//   2. per-thread histograms; offsets bucket-major, thread-minor, so the
//      scatter into buckets keeps index order within a bucket;
//   3. each thread sorts whole buckets (split among threads by count) by
//      (key, index): insertion sort up to 32 players, std::sort above.
// Stacks spread over many binades fill the 4096 buckets evenly (the bit
// patterns grow like log S).  Where one bucket would hold more than
// max(4096, n / 4T) players (many near-equal stacks beside a far outlier)
// the threads run a stable LSD radix sort over all 64 bits instead (11-bit
// digits, digits shared by every key skipped).  Small fields use a
// comparison sort with the same total order.
static thread_local int t_sort_cap = 0;   // 0: no cap
SortThreadCap::SortThreadCap(int cap) : prev(t_sort_cap) { t_sort_cap = cap; }
SortThreadCap::~SortThreadCap() { t_sort_cap = prev; }

static inline bool bad_stack(double v) { return !(v > 0.0) || !std::isfinite(v); }
static inline double key_stack(uint64_t k) {   // the stack whose sort key is k (keys are ~bits)
    const uint64_t b = ~k;
    double v;
    std::memcpy(&v, &b, sizeof v);
    return v;
}

int sort_players_desc(const double *S, int n, std::vector<int> &perm, double *S_sorted) {
    perm.resize(n);
    if (n <= 4096) {
        int bad = -1;
        for (int i = 0; i < n && bad < 0; ++i)
            if (bad_stack(S[i])) bad = i;
        std::vector<std::pair<double, int>> kv(n);
        for (int i = 0; i < n; ++i) kv[i] = {S[i], i};
        std::sort(kv.begin(), kv.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
            return a.first > b.first || (a.first == b.first && a.second < b.second);
        });
        for (int i = 0; i < n; ++i) perm[i] = kv[i].second;
        if (S_sorted)
            for (int i = 0; i < n; ++i) S_sorted[i] = kv[i].first;
        return bad;
    }
    constexpr int kDig = 12, kNB = 1 << kDig;                      // bucket digit
    constexpr int kBits = 11, kBuckets = 1 << kBits, kPasses = (64 + kBits - 1) / kBits;   // LSD
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    int T = n < 16384 ? 1 : std::min({hw, 16, n / 4096});   // measured crossover on the Grace host
    if (t_sort_cap > 0) T = std::min(T, t_sort_cap);
    std::vector<uint64_t> key(n), key2(n);
    std::vector<int> idx(n), idx2(n);
    std::vector<uint32_t> hist((size_t)T * kNB), offs((size_t)T * kNB), bstart(kNB + 1);
    std::vector<uint64_t> lo(T), hi(T);
    std::vector<int> brange(T + 1), bad_t(T, -1);
    const int cap = std::max(4096, n / (4 * T));   // largest bucket the bucket sort takes
    std::vector<std::pair<uint64_t, int>> scratch((size_t)T * cap);
    uint64_t kmin = 0;
    int shift = 0, nb = 1;
    bool lsd = false;
    uint8_t skip[kPasses] = {};
    HostBarrier bar(T);
    auto sync = [&] {
        if (T > 1) bar.wait();
    };
    auto work = [&](int t) {
        const int i0 = (int)((long)n * t / T), i1 = (int)((long)n * (t + 1) / T);
        uint64_t mn = ~0ull, mx = 0;
        int bad = -1;
        for (int i = i0; i < i1; ++i) {
            if (bad < 0 && bad_stack(S[i])) bad = i;
            uint64_t b;
            std::memcpy(&b, S + i, sizeof b);
            const uint64_t k = ~b;
            key[i] = k;
            idx[i] = i;
            mn = std::min(mn, k);
            mx = std::max(mx, k);
        }
        bad_t[t] = bad;
        lo[t] = mn;
        hi[t] = mx;
        sync();
        if (t == 0) {
            kmin = *std::min_element(lo.begin(), lo.end());
            const uint64_t span = *std::max_element(hi.begin(), hi.end()) - kmin;
            int bits = 0;
            while (bits < 64 && (span >> bits) != 0) ++bits;
            shift = std::max(0, bits - kDig);
            nb = (int)(span >> shift) + 1;
        }
        sync();
        uint32_t *h = hist.data() + (size_t)t * kNB;
        std::fill(h, h + nb, 0u);
        for (int i = i0; i < i1; ++i) ++h[(key[i] - kmin) >> shift];
        sync();
        if (t == 0) {   // bucket starts, the largest bucket, bucket ranges of ~n/T players
            uint32_t sum = 0, big = 0;
            for (int b = 0; b < nb; ++b) {
                bstart[b] = sum;
                uint32_t c = 0;
                for (int u = 0; u < T; ++u) c += hist[(size_t)u * kNB + b];
                big = std::max(big, c);
                sum += c;
            }
            bstart[nb] = sum;
            lsd = big > (uint32_t)cap;
            int b = 0;
            for (int u = 0; u < T; ++u) {
                const long want = (long)n * u / T;
                while (b < nb && bstart[b] < want) ++b;
                brange[u] = b;
            }
            brange[T] = nb;
        }
        sync();
        if (!lsd) {
            uint32_t *of = offs.data() + (size_t)t * kNB;
            for (int b = 0; b < nb; ++b) {
                uint32_t o = bstart[b];
                for (int u = 0; u < t; ++u) o += hist[(size_t)u * kNB + b];
                of[b] = o;
            }
            for (int i = i0; i < i1; ++i) {
                const uint64_t k = key[i];
                const uint32_t o = of[(k - kmin) >> shift]++;
                key2[o] = k;
                idx2[o] = i;
            }
            sync();
            for (int b = brange[t]; b < brange[t + 1]; ++b) {
                const int s0 = (int)bstart[b], e0 = (int)bstart[b + 1];
                if (e0 - s0 <= 32) {   // insertion sort; index order already holds among equal keys
                    for (int i = s0 + 1; i < e0; ++i) {
                        const uint64_t k = key2[i];
                        const int x = idx2[i];
                        int j = i - 1;
                        while (j >= s0 && key2[j] > k) {
                            key2[j + 1] = key2[j];
                            idx2[j + 1] = idx2[j];
                            --j;
                        }
                        key2[j + 1] = k;
                        idx2[j + 1] = x;
                    }
                } else {   // (key, index) pairs in this thread's scratch
                    std::pair<uint64_t, int> *kv = scratch.data() + (size_t)t * cap;
                    for (int i = s0; i < e0; ++i) kv[i - s0] = {key2[i], idx2[i]};
                    std::sort(kv, kv + (e0 - s0));
                    for (int i = s0; i < e0; ++i) {
                        key2[i] = kv[i - s0].first;
                        idx2[i] = kv[i - s0].second;
                    }
                }
            }
            sync();
            std::copy(idx2.begin() + i0, idx2.begin() + i1, perm.begin() + i0);
            if (S_sorted)   // the sorted stacks from the sorted keys: no gather
                for (int i = i0; i < i1; ++i) S_sorted[i] = key_stack(key2[i]);
            return;
        }
        // LSD radix sort over all digits (keys and indices in key / idx)
        uint64_t *k = key.data(), *k2 = key2.data();
        int *x = idx.data(), *x2 = idx2.data();
        for (int d = 0; d < kPasses; ++d) {
            const int sh = d * kBits;
            std::fill(h, h + kBuckets, 0u);
            for (int i = i0; i < i1; ++i) ++h[(k[i] >> sh) & (kBuckets - 1)];
            sync();
            if (t == 0) {   // offsets: digit-major, thread-minor
                uint32_t sum = 0;
                int used = 0;
                for (int b = 0; b < kBuckets; ++b) {
                    uint32_t tot = 0;
                    for (int u = 0; u < T; ++u) {
                        uint32_t &c = hist[(size_t)u * kNB + b];
                        const uint32_t cnt = c;
                        c = sum + tot;
                        tot += cnt;
                    }
                    used += tot != 0;
                    sum += tot;
                }
                skip[d] = used <= 1;   // one digit value: the order stays
            }
            sync();
            if (!skip[d]) {
                for (int i = i0; i < i1; ++i) {
                    const uint32_t o = h[(k[i] >> sh) & (kBuckets - 1)]++;
                    k2[o] = k[i];
                    x2[o] = x[i];
                }
                std::swap(k, k2);
                std::swap(x, x2);
            }
            sync();
        }
        if (t == 0) {
            std::copy(x, x + n, perm.begin());
            if (S_sorted)
                for (int i = 0; i < n; ++i) S_sorted[i] = key_stack(k[i]);
        }
    };
    HostPool::get().run(T, work);
    for (int v : bad_t)   // threads hold increasing index ranges
        if (v >= 0) return v;
    return -1;
}

// the inverse of p->perm, built when a subset query first needs it after a sort
void plan_inv_perm(Plan *p) {
    if ((int)p->inv_perm.size() == p->n) return;
    p->inv_perm.resize(p->n);
    for (int i = 0; i < p->n; ++i) p->inv_perm[p->perm[i]] = i;
}

int plan_geometry(Plan *p, int n, const double *S, int k, std::string &err) {
    if (n < 1 || k < 1 || k > n || !S) {
        err = "invalid plan arguments n=" + std::to_string(n) + " k=" + std::to_string(k);
        return -1;
    }
    p->n = n;
    p->k = k;
    p->B = select_block_size(n, k);
    p->fft_min_deg = select_fft_min(n, k);
    p->spectral = g_config.coefficient_fft_only != 1 && !p->coeff_only;
    p->zskip = g_config.disable_zero_prefix != 1;
    const int B = p->B;

    // descending stacks, ties by original index (reference gpu_plan.cu:405-409);
    // the sort also checks the stacks and writes them in sorted order
    p->S_sorted.resize(n);
    const int bad = sort_players_desc(S, n, p->perm, p->S_sorted.data());
    if (bad >= 0) {
        err = "stacks must be finite and positive (S[" + std::to_string(bad) + "])";
        return -1;
    }
    p->inv_perm.clear();
    p->Smax = p->S_sorted[0];

    // geometry: node at level l covers B << l players
    p->nblocks = (n + B - 1) / B;
    const int Nt = pow2_ge(p->nblocks);
    p->L = ilog2(Nt) + 1;
    if (p->L > kMaxLevels) { err = "tournament too large"; return -1; }
    // a VJP plan's spectral band may reach the root only when the root's
    // children are untruncated
    const bool vjp_root_spec = p->L >= 2 && ((long)B << (p->L - 2)) + 1 <= k;
    for (int l = 0; l < p->L; ++l) {
        Level &v = p->lv[l];
        v.nreal = (l == 0) ? p->nblocks : (p->lv[l - 1].nreal + 1) / 2;
        v.deg = (long)B << l;
        v.plen = (int)std::min<long>(v.deg + 1, k);
        v.glen = (int)std::min<long>(v.deg, k);
        v.pst = round2(v.plen);
        v.gst = round2(v.glen);
        if (l >= 1) {
            const Level &c = p->lv[l - 1];
            v.npairs = c.nreal / 2;
            const bool can_fft = c.deg >= p->fft_min_deg;
            // spectral when the children's and this level's products are exact
            // (not truncated at k) and the transforms fit one CTA
            // children beyond one CTA's transform use the multi-pass kernels,
            // which hand g spectra (not coefficients) to a spectral level below
            // (a parent truncated at k is fine: its build writes coefficients,
            // and a truncated parent never has a spectral level above it)
            bool spec = p->spectral && can_fft && c.deg + 1 <= k;
            if (c.deg > kSpecMaxD) spec = spec && l - 1 >= 1 && p->lv[l - 1].kind == 2;
            if (p->vjp) {
                // single VJP plans: spectral from the configured child degree up
                // (the forward tuner table does not apply); a spectral band that
                // ends below the root (children truncated at k above it) stays
                // within one-CTA transforms, where its top level converts the
                // coefficient Pbar handed down to it
                if (g_config.vjp_spectral_min_degree > 0) spec = spec && c.deg >= g_config.vjp_spectral_min_degree;
                if (!vjp_root_spec) spec = spec && c.deg <= kSpecMaxD;
            } else if (spec && !tune_spectral_ok(n, k, l)) {
                spec = false;   // the tuner table keeps it on coefficients
            }
            v.kind = spec ? 2 : (can_fft ? 1 : 0);
            v.cta_pts = select_cta_points(n, k, l);
            v.fft = (v.kind == 1) ? 1 : 0;
            if (v.fft) {
                long need = std::max<long>(2L * c.plen - 2, (long)c.glen + c.plen - 1);
                v.fftn = std::max(4, pow2_ge(need));
            }
        }
    }
    // bottom schoolbook levels fused into the subtree kernels (never the root,
    // whose product is not built; at most the levels one CTA of blocks spans)
    p->Lf = 0;
    if (g_config.enable_subtree == 1)
        for (int l = 1; l <= std::min(p->L - 2, kSubMaxLevels) && p->lv[l].kind == 0; ++l) p->Lf = l;
    // per-node element counts
    size_t per_q = 0;
    size_t fa = 0, fb = 0;
    for (int l = 0; l < p->L; ++l) {
        Level &v = p->lv[l];
        if (l <= p->L - 2 || l == 0) {   // level 0 always exists (leaf blocks)
            v.P_q = (size_t)v.nreal * v.pst;
            v.g_q = (size_t)v.nreal * v.gst;
        }
        if (l >= 1 && v.fft) {
            v.spec_q = (size_t)2 * v.npairs * (v.fftn / 2 + 1);
            fa = std::max(fa, (size_t)v.npairs * v.fftn);
            fb = std::max(fb, (size_t)v.npairs * (v.fftn / 2));
        }
        if (l + 1 < p->L && p->lv[l + 1].kind == 2) {   // parent level is spectral
            v.spec2_q = (size_t)v.nreal * (v.deg + 1);
            v.ends_q = (size_t)v.nreal * 2;
        }
        if (v.kind == 2) {
            v.G_q = (size_t)v.nreal * (v.deg / 2 + 1);
            const Level &c = p->lv[l - 1];
            if (c.deg > kSpecMaxD) {   // multi-pass build and propagate buffers
                fa = std::max(fa, (size_t)v.nreal * (size_t)c.deg);
                fa = std::max(fa, (size_t)c.nreal * (size_t)(c.deg / 2));
            }
            if (v.deg / 2 > kSpecMaxD) fa = std::max(fa, (size_t)v.nreal * (size_t)(v.deg / 2));
        }
        per_q += (v.P_q + v.g_q + v.ends_q) * 8 + (v.spec_q + v.spec2_q + v.G_q) * 16 + 1024;
    }
    per_q += (size_t)p->nblocks * (B + 1) * 8 + 1024;
    per_q += (fa * 2 + fb) * 16;
    p->tree_q_bytes = per_q;
    p->fa_elems = fa;
    p->fb_elems = fb;
    // engine: the small path, the linear engine or the tree
    const int eng = g_config.engine;
    p->small = eng != 2 && plan_small_ok(p);
    p->linear = !p->coeff_only && !p->vjp && !p->small && k <= kLinearMaxK &&
                (eng == 2 || (eng == 0 && plan_linear_auto(n, k)));
    return 0;
}

// Invariants of a plan's geometry that the kernels rely on (host only; the
// counterpart of the reference's planner checks, tools/test_gpu_wrap_feasibility.cu
// and gpu_internal.h:321-342).  0 when all hold, else -1 and the first
// violation in `why`.
int plan_check_geometry(const Plan *p, std::string &why) {
    auto bad = [&](int l, const std::string &m) {
        why = "level " + std::to_string(l) + ": " + m;
        return -1;
    };
    const int k = p->k, B = p->B, L = p->L;
    if (p->nblocks != (p->n + B - 1) / B) return bad(0, "block count");
    if (p->lv[L - 1].nreal != 1) return bad(L - 1, "the root level has more than one node");
    for (int l = 0; l < L; ++l) {
        const Level &v = p->lv[l];
        if (v.deg != ((long)B << l)) return bad(l, "degree");
        if (l == 0 ? v.nreal != p->nblocks : v.nreal != (p->lv[l - 1].nreal + 1) / 2) return bad(l, "node count");
        if (v.plen != (int)std::min<long>(v.deg + 1, k) || v.glen != (int)std::min<long>(v.deg, k))
            return bad(l, "truncation lengths");
        if (v.pst < v.plen || v.gst < v.glen || (v.pst & 1) || (v.gst & 1)) return bad(l, "row strides");
        if (l == 0) continue;
        const Level &c = p->lv[l - 1];
        if (v.npairs != c.nreal / 2) return bad(l, "pair count");
        const int gpl = (l == L - 1) ? k : v.glen;   // the parent's g (the payout at the root)
        if (c.glen > gpl) return bad(l, "a child's g is longer than its parent's");
        if (v.kind == 1) {
            const long N = v.fftn;
            if (N < 4 || (N & (N - 1))) return bad(l, "FFT size is not a power of two");
            // product: degree 2(lc - 1), one wrapped term at N = 2(lc - 1) is corrected
            if (N < 2L * c.plen - 2) return bad(l, "FFT size below the product");
            // middle product (and its transpose in the VJP): no wrap at all
            if (N < (long)c.glen + c.plen - 1 || gpl > N) return bad(l, "FFT size below the correlation");
        } else if (v.kind == 2) {
            if (c.plen != c.deg + 1) return bad(l, "spectral level over truncated children");
            if (c.deg > kSpecMaxD && !(l - 1 >= 1 && c.kind == 2))
                return bad(l, "multi-pass spectral level without spectral children");
            if (p->coeff_only || !p->spectral) return bad(l, "spectral level in a coefficient-only plan");
            // a VJP band ending below the root converts its top's Pbar and
            // writes its top's gbar coefficients in one CTA
            if (p->vjp && l < L - 1 && p->lv[l + 1].kind != 2 && c.deg > kSpecMaxD)
                return bad(l, "VJP spectral band ends on a multi-pass level below the root");
            if (p->vjp && c.deg < 4) return bad(l, "VJP spectral level below degree 4");
        } else if (v.kind != 0) {
            return bad(l, "unknown level kind");
        } else if (c.deg >= p->fft_min_deg) {
            return bad(l, "schoolbook level above the FFT crossover");
        }
    }
    if (p->Lf > 0) {
        if (p->Lf > L - 2) return bad(p->Lf, "subtree reaches the root");
        for (int l = 1; l <= p->Lf; ++l)
            if (p->lv[l].kind != 0) return bad(l, "subtree over a non-schoolbook level");
    }
    if (p->small && p->linear) return bad(0, "two engines chosen");
    return 0;
}

// tree buffers for chunks of qc nodes: leaf block products, per-level
// polynomials, spectra and end coefficients, FFT work buffers
size_t plan_tree_layout(Plan *p, int qc, char *base) {
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_bp = take(sizeof(double) * (size_t)qc * p->nblocks * (p->B + 1));
    size_t o_P[kMaxLevels], o_g[kMaxLevels], o_spec[kMaxLevels], o_s2[kMaxLevels], o_en[kMaxLevels],
        o_G[kMaxLevels];
    for (int l = 0; l < p->L; ++l) {
        const Level &v = p->lv[l];
        o_P[l] = v.P_q ? take(sizeof(double) * (size_t)qc * v.P_q) : 0;
        o_g[l] = v.g_q ? take(sizeof(double) * (size_t)qc * v.g_q) : 0;
        o_spec[l] = v.spec_q ? take(sizeof(double2) * (size_t)qc * v.spec_q) : 0;
        o_s2[l] = v.spec2_q ? take(sizeof(double2) * (size_t)qc * v.spec2_q) : 0;
        o_en[l] = v.ends_q ? take(sizeof(double) * (size_t)qc * v.ends_q) : 0;
        // the root's G (the payout's spectrum) is shared by all nodes of a chunk
        const size_t gq = (l == p->L - 1) ? 1 : (size_t)qc;
        o_G[l] = v.G_q ? take(sizeof(double2) * gq * v.G_q) : 0;
    }
    const size_t fa = p->fa_elems, fb = p->fb_elems;
    const size_t o_fa = fa ? take(sizeof(double2) * (size_t)qc * fa) : 0;
    const size_t o_fb = fa ? take(sizeof(double2) * (size_t)qc * std::max(fa, fb)) : 0;
    const size_t o_fc = fa ? take(sizeof(double2) * (size_t)qc * fa) : 0;
    if (!base) return off;
    p->d_blockP = (double *)(base + o_bp);
    for (int l = 0; l < p->L; ++l) {
        Level &v = p->lv[l];
        v.P = v.P_q ? (double *)(base + o_P[l]) : nullptr;
        v.g = v.g_q ? (double *)(base + o_g[l]) : nullptr;
        v.spec = v.spec_q ? (double2 *)(base + o_spec[l]) : nullptr;
        v.spec2 = v.spec2_q ? (double2 *)(base + o_s2[l]) : nullptr;
        v.ends = v.ends_q ? (double *)(base + o_en[l]) : nullptr;
        v.G = v.G_q ? (double2 *)(base + o_G[l]) : nullptr;
    }
    p->fft_work = std::max(fa, fb) * qc;
    if (fa) {
        p->d_fa = (double2 *)(base + o_fa);
        p->d_fb = (double2 *)(base + o_fb);
        p->d_fc = (double2 *)(base + o_fc);
    }
    return off;
}

static bool root_gspec_forkable(const Plan *p);

int chunk_piece_nodes(const Plan *p, int i, int np, int r) {
    const int cap = (i + 1 < p->nparts ? p->part_off[i + 1] : p->qc) - p->part_off[i];
    return (i + 1 == np) ? r : std::min(cap, (r + np - i - 1) / (np - i));
}

static void swap_view(Plan *p, ChunkView &v) {
    for (int l = 0; l < p->L; ++l) std::swap(p->lv[l], v.lv[l]);
    std::swap(p->d_a, v.a);
    std::swap(p->d_contrib, v.contrib);
    std::swap(p->d_blockP, v.blockP);
    std::swap(p->d_fa, v.fa);
    std::swap(p->d_fb, v.fb);
    std::swap(p->d_fc, v.fc);
    std::swap(p->stream, v.st);
}

PieceScope::PieceScope(Plan *plan, const ChunkView *view) : p(plan), on(view != nullptr) {
    if (on) {
        saved = *view;
        swap_view(p, saved);
    }
}

PieceScope::~PieceScope() {
    if (on) swap_view(p, saved);
}

// The buffers of node slots [off, off + slots) of a plan's chunk: every
// per-node pointer shifted by off nodes (the root's shared spectrum stays);
// false if any of them would leave the arena's first arena_bytes.
static bool make_chunk_view(const Plan *p, int off, int slots, size_t arena_bytes, ChunkView &v) {
    const size_t h = (size_t)off, m = (size_t)slots, n = (size_t)p->n;
    const size_t bp = (size_t)p->nblocks * (p->B + 1), fb = std::max(p->fa_elems, p->fb_elems);
    for (int l = 0; l < p->L; ++l) {
        Level &x = v.lv[l];
        x = p->lv[l];
        if (x.P) x.P += h * x.P_q;
        if (x.g) x.g += h * x.g_q;
        if (x.spec) x.spec += h * x.spec_q;
        if (x.spec2) x.spec2 += h * x.spec2_q;
        if (x.ends) x.ends += h * x.ends_q;
        if (x.G && l != p->L - 1) x.G += h * x.G_q;
    }
    v.a = p->d_a + h * n;
    v.contrib = p->d_contrib + h * n;
    v.blockP = p->d_blockP + h * bp;
    if (p->d_fa) {
        v.fa = p->d_fa + h * p->fa_elems;
        v.fb = p->d_fb + h * fb;
        v.fc = p->d_fc + h * p->fa_elems;
    }
    const char *lo = p->arena, *hi = p->arena + arena_bytes;
    auto inside = [&](const void *q, size_t bytes) {
        return !q || ((const char *)q >= lo && (const char *)q + bytes <= hi);
    };
    bool ok = inside(v.a, 8 * m * n) && inside(v.contrib, 8 * m * n) && inside(v.blockP, 8 * m * bp) &&
              inside(v.fa, 16 * m * p->fa_elems) && inside(v.fb, 16 * m * fb) && inside(v.fc, 16 * m * p->fa_elems);
    for (int l = 0; l < p->L; ++l) {
        const Level &x = v.lv[l];
        ok = ok && inside(x.P, 8 * m * x.P_q) && inside(x.g, 8 * m * x.g_q) && inside(x.spec, 16 * m * x.spec_q) &&
             inside(x.spec2, 16 * m * x.spec2_q) && inside(x.ends, 8 * m * x.ends_q) &&
             inside(x.G, 16 * (l == p->L - 1 ? 1 : m) * x.G_q);
    }
    return ok;
}

Plan *plan_create(int n, const double *S, int k, const IcmGpuOptions *opts, std::string &err, bool coeff_only,
                  double q_bytes_scale, size_t budget_bytes, bool vjp) {
    Plan *p = new Plan();
    if (opts) p->opts = *opts;
    p->opts.device_id = g_device;
    p->coeff_only = coeff_only;
    p->vjp = vjp;
    if (plan_geometry(p, n, S, k, err) != 0) { delete p; return nullptr; }
    const int B = p->B;
    const int Nt = 1 << (p->L - 1);
    const size_t tree_q = p->linear ? linear_ck_per_node(n, k) * sizeof(double) : p->tree_q_bytes;
    const size_t per_q = (size_t)((double)(tree_q + (size_t)2 * n * 8 + 1024) * q_bytes_scale);

    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    size_t budget = budget_bytes           ? budget_bytes
                    : g_config.max_device_bytes ? g_config.max_device_bytes
                                                : std::min<size_t>((size_t)(free_b * 0.6), (size_t)48 << 30);
    int qc = (int)std::min<size_t>(256, std::max<size_t>(1, budget / std::max<size_t>(per_q, 1)));
    if (g_config.q_chunk > 0) qc = std::min(qc, g_config.q_chunk);
    p->qc = qc;

    // arena: per-plan arrays, then the tree buffers
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    const size_t o_S = take(sizeof(double) * n), o_perm = take(sizeof(int) * n);
    const size_t o_pay = take(sizeof(double) * k), o_acc = take(sizeof(double) * n);
    const size_t o_out = take(sizeof(double) * n), o_act = take(n);
    size_t hot_total = 0;
    for (int l = 0; l < p->L; ++l) { p->hot_off[l] = hot_total; hot_total += (size_t)(Nt >> l); }
    const size_t o_hot = take(hot_total);
    const size_t o_a = take(sizeof(double) * (size_t)qc * n);
    const size_t o_con = take(sizeof(double) * (size_t)qc * n);
    // the linear engine keeps checkpoints instead of a tree
    const size_t o_tree = p->linear ? 0 : take(plan_tree_layout(p, qc, nullptr));
    const size_t o_ck = p->linear ? take(sizeof(double) * (size_t)qc * linear_ck_per_node(n, k)) : 0;
    const size_t o_cnt = take(sizeof(unsigned));
    (void)B;

    // stream-ordered allocation from the device's default pool, whose release
    // threshold icm_gpu_init raises so that freed arenas are kept for the next
    // plan (icm_gpu_release_pooled_memory returns them to the driver);
    // memory_strategy 1 asks for plain cudaMalloc instead
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        p->pooled = p->opts.memory_strategy != 1;
        e = dev_alloc((void **)&p->arena, off, p->stream, p->pooled);
    }
    if (e != cudaSuccess) {
        err = "device allocation of " + std::to_string(off) + " bytes failed: " + cudaGetErrorString(e);
        if (p->stream) cudaStreamDestroy(p->stream);
        delete p;
        return nullptr;
    }
    p->arena_bytes = off;
    p->peak_bytes = (double)off;
    if (!p->small && !p->linear && root_gspec_forkable(p)) {   // stream and events for the root's spectrum
        e = cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess && !p->ev_join) e = cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            err = std::string("side stream: ") + cudaGetErrorString(e);
            plan_destroy(p);
            return nullptr;
        }
    }
    char *A = p->arena;
    p->d_S = (double *)(A + o_S);
    p->d_perm = (int *)(A + o_perm);
    p->d_payout = (double *)(A + o_pay);
    p->d_acc = (double *)(A + o_acc);
    p->d_out = (double *)(A + o_out);
    p->d_active = (uint8_t *)(A + o_act);
    p->d_hot = (uint8_t *)(A + o_hot);
    p->d_a = (double *)(A + o_a);
    p->d_contrib = (double *)(A + o_con);
    if (p->linear) p->d_ck = (double *)(A + o_ck);
    else plan_tree_layout(p, qc, A + o_tree);
    p->d_counter = (unsigned *)(A + o_cnt);
    // after the arena's pointers: the views offset them
    // default: four pieces from n = 6000, two below (measured on GB300 with
    // one / two / four pieces: n = 16384 4.92 / 4.01 / 3.75 ms; n = 8000,
    // k = 1200 2.51 / 2.02 / 1.92 ms; n = 4096, k = 40 0.62 / 0.55 / 0.57 ms;
    // n = 2000 0.59 / 0.52 / 0.59 ms)
    const int want = g_config.chunk_streams > 0 ? g_config.chunk_streams : n >= 6000 ? 4 : 2;
    const int np = std::min({want, kMaxChunkParts, qc});
    if (!p->small && !p->linear && p->Lf == 0 && np >= 2 && !p->opts.verbose) {
        for (int i = 0; i < np; ++i) p->part_off[i] = i * (qc / np);
        for (int i = 1; i < np; ++i) {
            const int slots = (i + 1 < np ? p->part_off[i + 1] : qc) - p->part_off[i];
            if (!make_chunk_view(p, p->part_off[i], slots, off, p->part[i])) {
                err = "internal: a chunk view leaves the plan's arena";
                plan_destroy(p);
                return nullptr;
            }
            e = cudaStreamCreateWithFlags(&p->part[i].st, cudaStreamNonBlocking);
            if (e != cudaSuccess) break;
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_split, cudaEventDisableTiming);
        for (int i = 0; i < np && e == cudaSuccess; ++i)
            e = cudaEventCreateWithFlags(&p->ev_acc[i], cudaEventDisableTiming);
        if (e == cudaSuccess && !p->ev_join) e = cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            err = std::string("chunk streams: ") + cudaGetErrorString(e);
            plan_destroy(p);
            return nullptr;
        }
        p->nparts = np;
    }
    e = cudaMemsetAsync(p->d_counter, 0, sizeof(unsigned), p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_S, p->S_sorted.data(), sizeof(double) * n, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_perm, p->perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        err = std::string("plan upload: ") + cudaGetErrorString(e);
        plan_destroy(p);
        return nullptr;
    }
    if (p->opts.verbose) {
        fprintf(stderr, "icm_gb300 plan: n=%d k=%d B=%d L=%d qc=%d arena=%.1f MB\n", n, k, p->B, p->L, qc,
                off / 1e6);
        for (int l = 0; l < p->L; ++l) {
            const Level &v = p->lv[l];
            fprintf(stderr, "  level %2d nreal=%7d deg=%8ld plen=%7d glen=%7d %s N=%d\n", l, v.nreal, v.deg,
                    v.plen, v.glen, v.kind == 2 ? "spectral" : (v.fft ? "fft" : "school"), v.fftn);
        }
    }
    return p;
}

void plan_destroy(Plan *p) {
    if (!p) return;
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->graph) cudaGraphExecDestroy(p->graph);
    if (p->d_node) cudaFreeAsync(p->d_node, p->stream);
    if (p->arena) {
        if (p->pooled) {
            cudaFreeAsync(p->arena, p->stream);
            cudaStreamSynchronize(p->stream);
        } else {
            cudaFree(p->arena);
        }
    }
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->ev_in) cudaEventDestroy(p->ev_in);
    if (p->ev_out) cudaEventDestroy(p->ev_out);
    for (cudaEvent_t ev : p->stage_ev) cudaEventDestroy(ev);
    if (p->ev_split) cudaEventDestroy(p->ev_split);
    for (int i = 0; i < kMaxChunkParts; ++i) {
        if (p->ev_acc[i]) cudaEventDestroy(p->ev_acc[i]);
        if (p->part[i].st) {
            cudaStreamSynchronize(p->part[i].st);
            cudaStreamDestroy(p->part[i].st);
        }
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    if (p->side) {
        cudaStreamSynchronize(p->side);
        cudaStreamDestroy(p->side);
    }
    for (cudaEvent_t ev : p->prof.pool) cudaEventDestroy(ev);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

// the root's payout spectrum can run beside the build: a one-kernel spectral
// root writes only its own G buffer
static bool root_gspec_forkable(const Plan *p) {
    const int L = p->L;
    return L >= 2 && p->Lf < L - 1 && p->lv[L - 1].kind == 2 && p->lv[L - 1].deg / 2 <= kSpecMaxD;
}

int plan_restack(Plan *p, const double *S, std::string &err) {
    const int n = p->n;
    const int bad = sort_players_desc(S, n, p->perm, p->S_sorted.data());
    if (bad >= 0) {
        err = "stacks must be finite and positive (S[" + std::to_string(bad) + "])";
        return -1;
    }
    p->inv_perm.clear();
    p->Smax = p->S_sorted[0];
    cudaError_t e = cudaMemcpyAsync(p->d_S, p->S_sorted.data(), sizeof(double) * n, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_perm, p->perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, p->stream);
    if (e != cudaSuccess) { err = std::string("stack upload: ") + cudaGetErrorString(e); return -1; }
    return 0;
}

// subset: active players (sorted order) and per-level hot bitmaps
// (reference src/cpu/icm.c:2430-2473)
int plan_set_targets(Plan *p, const int *targets, int n_targets, std::string &err) {
    const int n = p->n, B = p->B;
    plan_inv_perm(p);
    std::vector<uint8_t> act(n, 0);
    for (int t = 0; t < n_targets; ++t) {
        const int o = targets[t];
        if (o >= 0 && o < n) act[p->inv_perm[o]] = 1;
    }
    const int Nt = 1 << (p->L - 1);
    size_t total = 0;
    for (int l = 0; l < p->L; ++l) total += (size_t)(Nt >> l);
    std::vector<uint8_t> hot(total, 0);
    for (int b = 0; b < p->nblocks; ++b) {
        const int s = b * B, e = std::min(n, s + B);
        for (int j = s; j < e; ++j)
            if (act[j]) { hot[p->hot_off[0] + b] = 1; break; }
    }
    for (int l = 1; l < p->L; ++l) {
        const int nc = Nt >> (l - 1), np = Nt >> l;
        for (int j = 0; j < np; ++j) {
            const int lft = (2 * j < nc) ? hot[p->hot_off[l - 1] + 2 * j] : 0;
            const int rgt = (2 * j + 1 < nc) ? hot[p->hot_off[l - 1] + 2 * j + 1] : 0;
            hot[p->hot_off[l] + j] = (uint8_t)(lft | rgt);
        }
    }
    cudaError_t e = cudaMemcpyAsync(p->d_active, act.data(), n, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_hot, hot.data(), total, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) { err = std::string("subset upload: ") + cudaGetErrorString(e); return -1; }
    p->subset = true;
    return 0;
}

// one chunk of nq nodes starting at active-node index q0
// share of a level's (tree node, chunk node) pairs outside the zero prefix:
// the work the pruned kernels actually do, for the profiler's flop counts
static double hot_frac(const Plan *p, int q0, int nq, long span, int nreal) {
    if (!p->zskip || nreal <= 0 || span <= 0 || p->h_z.empty()) return 1.0;
    double hot = 0.0;
    for (int q = 0; q < nq; ++q) hot += nreal - std::min<long>(nreal, p->h_z[q0 + q] / span);
    return hot / ((double)nq * nreal);
}

// a stage boundary of the current chunk (opts.verbose only)
static void stage_mark(Plan *p, cudaStream_t st) {
    if (!p->opts.verbose) return;
    if (p->stage_used == p->stage_ev.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        p->stage_ev.push_back(e);
    }
    cudaEventRecord(p->stage_ev[p->stage_used++], st);
}

void run_chunk(Plan *p, int q0, int nq, const double2 *tw, int logTW, bool first, bool divide,
               const ChunkView *view, cudaEvent_t acc_wait, cudaEvent_t acc_done) {
    // the chunk's buffers: the plan's own, or a piece's view of them (node slots from its offset)
    cudaStream_t st = view ? view->st : p->stream;
    const int L = p->L;
    Level *lv = view ? const_cast<Level *>(view->lv) : p->lv;
    double *d_a = view ? view->a : p->d_a, *d_contrib = view ? view->contrib : p->d_contrib;
    double *d_blockP = view ? view->blockP : p->d_blockP;
    double2 *d_fa = view ? view->fa : p->d_fa, *d_fb = view ? view->fb : p->d_fb;
    double2 *d_fc = view ? view->fc : p->d_fc;
    Prof *pr = &p->prof;
    const int *zp = p->zskip ? p->d_z : nullptr;   // zero-prefix pruning (one-CTA levels)
    auto frac = [&](long span, int nreal) { pr->scale = zp ? hot_frac(p, q0, nq, span, nreal) : 1.0; };
    const int Lf = p->Lf;
    SubArgs SA{};
    SubFlops SF{};
    if (Lf >= 1) {   // leaf blocks and the bottom schoolbook levels in one kernel
        SA = sub_args(p, Lf, p->d_S, p->d_node, d_a, (size_t)p->n, p->subset ? p->d_active : nullptr,
                      d_contrib, !divide, divide, &SF);
        double fl = SF.leaf;
        for (int l = 1; l <= Lf; ++l)
            fl += SF.build[l] * (zp ? hot_frac(p, q0, nq, lv[l].deg, lv[l].nreal) : 1.0);
        pr->scale = 1.0;
        launch_sub_build(SA, nq, q0, st, pr, fl);
    } else {
        launch_leaf(p->B, p->n, p->nblocks, p->d_S, p->d_node, q0, nq, d_a, d_blockP, lv[0].P, lv[0].pst,
                    lv[0].plen, st, pr);
    }
    ++p->launches;
    if (divide) stage_mark(p, st);   // end of the block build
    if (L >= 2 && lv[1].kind == 2) {
        frac(lv[0].deg, lv[0].nreal);
        launch_spec_init(lv[0], nq, tw, logTW, st, pr, zp, q0);
        ++p->launches;
    }
    for (int l = 1; l <= L - 2; ++l) {
        frac(lv[l].deg, lv[l].nreal);   // builds decide per parent
        if (l <= Lf) {   // built by the subtree kernel
            if (l == Lf && lv[l + 1].kind == 2) {
                launch_spec_init(lv[l], nq, tw, logTW, st, pr, zp, q0);
                ++p->launches;
            }
            continue;
        }
        if (lv[l].kind == 2) {
            if (lv[l - 1].deg > kSpecMaxD) {
                launch_specbig_build(lv[l - 1], lv[l], lv[l + 1].kind != 2, nq, d_fa, d_fc, tw, logTW, st,
                                     &p->launches, pr, zp, q0);
            } else {
                launch_spec_build(lv[l - 1], lv[l], lv[l + 1].kind != 2, nq, tw, logTW, st, pr, zp, q0);
                ++p->launches;
            }
        } else if (lv[l].fft) {
            launch_fft_build(lv[l - 1], lv[l], nq, d_fa, d_fb, d_fc, false, tw, logTW, st, &p->launches, pr,
                             zp, q0);
            if (lv[l - 1].nreal & 1) {
                launch_school_build(lv[l - 1], lv[l], nq, lv[l].npairs, st, pr, zp, q0);
                ++p->launches;
            }
        } else {
            launch_school_build(lv[l - 1], lv[l], nq, 0, st, pr, zp, q0);
            ++p->launches;
        }
        if (lv[l].kind != 2 && lv[l + 1].kind == 2) {
            launch_spec_init(lv[l], nq, tw, logTW, st, pr, zp, q0);
            ++p->launches;
        }
    }
    pr->scale = 1.0;
    if (L >= 2 && lv[L - 1].fft)
        launch_fft_build(lv[L - 2], lv[L - 1], nq, d_fa, d_fb, d_fc, true, tw, logTW, st, &p->launches, pr);
    if (divide) stage_mark(p, st);   // end of the tree build
    for (int l = L - 1; l >= 1 + Lf; --l) {
        const bool root = (l == L - 1);
        const double *gp = root ? p->d_payout : lv[l].g;
        const size_t gp_q = root ? 0 : lv[l].g_q;
        const int gst_p = root ? 0 : lv[l].gst;
        const int gpl = root ? p->k : lv[l].glen;
        const uint8_t *hot_c = p->subset ? p->d_hot + p->hot_off[l - 1] : nullptr;
        frac(lv[l].deg, lv[l].nreal);   // propagates decide per parent (multi-pass: per child, close)
        if (root) pr->scale = 1.0;
        if (lv[l].kind == 2) {
            // the parent's g spectrum: the payout's at the root, converted from
            // coefficients below a coefficient level, else left by the level above
            if (root && p->root_forked) {
                cudaStreamWaitEvent(st, p->ev_join, 0);   // computed beside the build
            } else if (root || lv[l + 1].kind != 2) {
                const uint8_t *hot_p = p->subset ? p->d_hot + p->hot_off[l] : nullptr;
                if (lv[l].deg / 2 > kSpecMaxD) {
                    int logd = 0;
                    while ((1L << logd) < lv[l].deg) ++logd;
                    launch_gspecbig_init(gp, gp_q, gst_p, gpl, lv[l].nreal, logd, lv[l].G, root ? 0 : lv[l].G_q,
                                         root ? 1 : nq, hot_p, d_fa, d_fc, tw, logTW, st, &p->launches, pr,
                                         root ? nullptr : zp, q0);
                } else {
                    // the root's spectrum is shared by the chunk's nodes: never pruned
                    launch_gspec_init(gp, gp_q, gst_p, gpl, lv[l].nreal, lv[l], lv[l].G, root ? 0 : lv[l].G_q,
                                      root ? 1 : nq, hot_p, tw, logTW, st, pr, root ? nullptr : zp, q0);
                    ++p->launches;
                }
            }
            if (lv[l - 1].deg > kSpecMaxD) {
                launch_specbig_prop(lv[l].G, root ? 0 : lv[l].G_q, lv[l - 1], nq, hot_c, d_fa, d_fc, tw, logTW,
                                    st, &p->launches, pr, zp, q0);
            } else {
                launch_spec_prop(lv[l].G, root ? 0 : lv[l].G_q, lv[l - 1], lv[l], l - 1 >= 1 && lv[l - 1].kind == 2,
                                 nq, hot_c, tw, logTW, st, pr, zp, q0);
                ++p->launches;
            }
        } else if (lv[l].fft) {
            launch_fft_prop(gp, gp_q, gst_p, gpl, lv[l - 1], lv[l], nq, hot_c, d_fa, d_fb, d_fc, tw, logTW,
                            st, &p->launches, pr, zp, q0);
            if (lv[l - 1].nreal & 1) {
                launch_school_prop(gp, gp_q, gst_p, gpl, lv[l - 1], nq, hot_c, 2 * lv[l].npairs, st, pr, zp, q0);
                ++p->launches;
            }
        } else {
            launch_school_prop(gp, gp_q, gst_p, gpl, lv[l - 1], nq, hot_c, 0, st, pr, zp, q0);
            ++p->launches;
        }
    }
    if (divide) stage_mark(p, st);   // end of the propagate
    pr->scale = 1.0;
    if (Lf >= 1) {   // the bottom levels' propagate and (with divide) the division in one kernel
        double fl = 0.0, hotp = 1.0;
        for (int l = 1; l <= Lf; ++l)
            fl += SF.prop[l] * (zp ? hot_frac(p, q0, nq, lv[l - 1].deg, lv[l - 1].nreal) : 1.0);
        if (zp) {
            double hot = 0.0;
            for (int q = 0; q < nq; ++q) hot += p->n - p->h_z[q0 + q];
            hotp = hot / ((double)nq * p->n);
        }
        launch_sub_prop(SA, nq, q0, st, pr, fl + SF.divide * hotp);
        ++p->launches;
        if (!divide) return;
        if (acc_wait) cudaStreamWaitEvent(st, acc_wait, 0);
        launch_accumulate(p->n, nq, d_contrib, p->d_acc, first ? 1 : 0, st, pr);
        if (acc_done) cudaEventRecord(acc_done, st);
        ++p->launches;
        return;
    }
    if (!divide) return;
    if (zp) {   // players with a leaf factor of 0 skip the division
        double hot = 0.0;
        for (int q = 0; q < nq; ++q) hot += p->n - p->h_z[q0 + q];
        pr->scale = hot / ((double)nq * p->n);
    }
    const double *g0 = (L == 1) ? p->d_payout : lv[0].g;
    const size_t g0_q = (L == 1) ? 0 : lv[0].g_q;
    const int gst0 = (L == 1) ? 0 : lv[0].gst;
    launch_divide(p->B, p->n, p->k, p->nblocks, p->d_S, p->d_node, q0, nq, d_a, d_blockP, g0, g0_q, gst0,
                  p->subset ? p->d_active : nullptr, d_contrib, st, pr);
    pr->scale = 1.0;
    if (acc_wait) cudaStreamWaitEvent(st, acc_wait, 0);
    launch_accumulate(p->n, nq, d_contrib, p->d_acc, first ? 1 : 0, st, pr);
    if (acc_done) cudaEventRecord(acc_done, st);
    p->launches += 2;
}

// the kernel sequence of one run over nact active nodes (all chunks, the
// ordered node sums and the scatter)
static void enqueue_plan(Plan *p, int nact, const double2 *tw, int logTW) {
    if (p->small && nact > 0) {   // one launch per chunk; its last CTA sums and scatters
        SmallArgs A = small_args(p, p->d_S, p->d_node, p->d_payout, p->d_contrib, (size_t)p->n,
                                 p->subset ? p->d_active : nullptr);
        A.counter = p->d_counter;
        A.acc = p->d_acc;
        A.out = p->d_out;
        A.perm = p->d_perm;
        const double fq = small_flops(p);
        for (int q0 = 0; q0 < nact; q0 += p->qc) {
            const int nq = std::min(p->qc, nact - q0);
            A.first = q0 == 0;
            A.last = q0 + nq >= nact;
            launch_small(A, nq, q0, p->stream, &p->prof, fq);
            ++p->launches;
        }
    } else if (p->linear) {   // one warp per node, then the ordered sum
        const LinearArgs A = linear_args(p, p->d_S, p->d_node, p->d_payout, p->d_a, p->d_contrib, (size_t)p->n,
                                         p->subset ? p->d_active : nullptr, p->d_ck, p->zskip ? p->d_z : nullptr);
        const double fq = linear_flops(p);
        for (int q0 = 0; q0 < nact; q0 += p->qc) {
            const int nq = std::min(p->qc, nact - q0);
            launch_linear(A, nq, q0, p->stream, &p->prof, fq);
            launch_accumulate(p->n, nq, p->d_contrib, p->d_acc, q0 == 0 ? 1 : 0, p->stream, &p->prof);
            p->launches += 2;
        }
        launch_scatter(p->n, p->d_acc, p->d_perm, p->subset ? p->d_active : nullptr, p->d_out, p->stream);
        ++p->launches;
    } else {
        p->root_forked = false;
        if (nact > 0 && p->side) {   // the payout's spectrum beside the build
            const int l = p->L - 1;
            cudaEventRecord(p->ev_fork, p->stream);
            cudaStreamWaitEvent(p->side, p->ev_fork, 0);
            launch_gspec_init(p->d_payout, 0, 0, p->k, p->lv[l].nreal, p->lv[l], p->lv[l].G, 0, 1,
                              p->subset ? p->d_hot + p->hot_off[l] : nullptr, tw, logTW, p->side, &p->prof,
                              nullptr, 0);
            cudaEventRecord(p->ev_join, p->side);
            ++p->launches;
            p->root_forked = true;
        }
        if (p->nparts >= 2 && nact >= 2 && !p->prof.on) {   // (per-kernel profiles: one stream)
            const int L = p->L, l = L - 1, np = std::min(p->nparts, nact);
            if (!p->root_forked && L >= 2 && p->lv[l].kind == 2) {
                // a multi-pass root spectrum: once, before the pieces (they share it)
                int logd = 0;
                while ((1L << logd) < p->lv[l].deg) ++logd;
                launch_gspecbig_init(p->d_payout, 0, 0, p->k, p->lv[l].nreal, logd, p->lv[l].G, 0, 1,
                                     p->subset ? p->d_hot + p->hot_off[l] : nullptr, p->d_fa, p->d_fc, tw, logTW,
                                     p->stream, &p->launches, &p->prof, nullptr, 0);
                cudaEventRecord(p->ev_join, p->stream);
                p->root_forked = true;
            }
            // every chunk in up to np pieces, one per stream (streams that get no
            // piece are not forked); the node sums stay in node order: each
            // piece's accumulate waits for the one before it
            cudaEventRecord(p->ev_split, p->stream);
            for (int i = 1; i < np; ++i) cudaStreamWaitEvent(p->part[i].st, p->ev_split, 0);
            cudaEvent_t prev = nullptr;
            for (int q0 = 0; q0 < nact; q0 += p->qc) {
                int q = q0, r = std::min(p->qc, nact - q0);
                for (int i = 0; i < np && r > 0; ++i) {
                    const int m = chunk_piece_nodes(p, i, np, r);
                    run_chunk(p, q, m, tw, logTW, q == 0, true, i ? &p->part[i] : nullptr, prev, p->ev_acc[i]);
                    prev = p->ev_acc[i];
                    q += m;
                    r -= m;
                }
            }
            cudaStreamWaitEvent(p->stream, prev, 0);
        } else {
            for (int q0 = 0; q0 < nact; q0 += p->qc) {
                const int nq = std::min(p->qc, nact - q0);
                stage_mark(p, p->stream);   // chunk start
                run_chunk(p, q0, nq, tw, logTW, q0 == 0, true);
                stage_mark(p, p->stream);   // end of the leaf extraction (division and node sum)
            }
        }
        launch_scatter(p->n, p->d_acc, p->d_perm, p->subset ? p->d_active : nullptr, p->d_out, p->stream);
        ++p->launches;
    }
}

cudaError_t plan_dev_events(Plan *p) {
    cudaError_t e = cudaSuccess;
    if (!p->ev_in) e = cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess && !p->ev_out) e = cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming);
    return e;
}

int plan_run(Plan *p, int Q, const double *payout, double *equity, IcmGpuRunStats *stats, std::string &err,
             int q_begin, int q_end, const DevIO *dev) {
    if (!p || Q < 1 || !payout || !equity) { err = "invalid arguments"; return -1; }
    if (q_end < 0) q_end = Q;
    if (q_begin < 0 || q_begin > q_end || q_end > Q) { err = "invalid node range"; return -1; }
    const double t0 = now_ns();
    const long tma0 = g_tma_launches.load();
    p->launches = 0;
    std::vector<double> logv, w;
    make_nodes(Q, p->Smax, logv, w);
    std::vector<double> node;
    node.reserve(3 * (size_t)Q);
    for (int q = q_begin; q < q_end; ++q) {
        if (w[q] == 0.0) continue;   // the reference skips zero-weight nodes
        node.push_back(logv[q]);
        node.push_back(w[q]);
        node.push_back(std::exp(-logv[q]));
    }
    const int nact = (int)(node.size() / 3);
    cudaError_t e = cudaSuccess;
    if (nact > p->qmax) {
        // stream-ordered from the pool: no device-wide synchronisation
        if (p->d_node) cudaFreeAsync(p->d_node, p->stream);
        p->d_node = nullptr;
        p->d_z = nullptr;
        const size_t nb = sizeof(double) * 3 * (size_t)std::max(nact, 1);
        e = dev_alloc((void **)&p->d_node, nb + sizeof(int) * (size_t)std::max(nact, 1), p->stream, true);
        if (e != cudaSuccess) { err = std::string("node buffer: ") + cudaGetErrorString(e); return -1; }
        p->d_z = (int *)((char *)p->d_node + nb);
        p->qmax = nact;
    }
    p->h_z.resize(nact);
    for (int j = 0; j < nact; ++j) p->h_z[j] = zero_prefix(p->S_sorted.data(), p->n, node[3 * j]);
    if (nact)
        e = cudaMemcpyAsync(p->d_node, node.data(), sizeof(double) * node.size(), cudaMemcpyHostToDevice, p->stream);
    if (nact && e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_z, p->h_z.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, p->stream);
    if (dev) {   // the caller's payout is ready once its stream reaches this point
        if (e == cudaSuccess) e = plan_dev_events(p);
        if (e == cudaSuccess) e = cudaEventRecord(p->ev_in, dev->st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(p->stream, p->ev_in, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_payout, payout, sizeof(double) * p->k, cudaMemcpyDeviceToDevice, p->stream);
    } else if (e == cudaSuccess) {
        e = cudaMemcpyAsync(p->d_payout, payout, sizeof(double) * p->k, cudaMemcpyHostToDevice, p->stream);
    }
    if (e != cudaSuccess) { err = std::string("upload: ") + cudaGetErrorString(e); return -1; }
    int logNeed = 12, logTW = 0;
    for (int l = 1; l < p->L; ++l) {
        if (p->lv[l].fft) logNeed = std::max(logNeed, ilog2(p->lv[l].fftn));
        if (p->lv[l].kind == 2) logNeed = std::max(logNeed, ilog2(2 * p->lv[l].deg));
    }
    const double2 *tw = twiddles(logNeed, p->stream, err, &logTW);
    if (!tw) return -1;
    if (nact == 0) {
        e = cudaMemsetAsync(p->d_acc, 0, sizeof(double) * p->n, p->stream);
        if (e != cudaSuccess) { err = cudaGetErrorString(e); return -1; }
    }
    if (!p->ev0) { cudaEventCreate(&p->ev0); cudaEventCreate(&p->ev1); }
    p->prof.used = 0;
    p->prof.recs.clear();
    // enable_graphs: the sequence is captured once per node count (and node
    // buffer) and replayed; kernels read payouts and nodes from the plan's
    // buffers, which every run refills before the launch
    p->stage_used = 0;
    const bool use_graph = p->opts.enable_graphs == 1 && !p->prof.on && !p->opts.verbose && nact > 0;
    if (use_graph && (!p->graph || p->graph_nq != nact || p->graph_node != p->d_node || p->graph_subset != p->subset)) {
        if (p->graph) cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
        cudaGraph_t g = nullptr;
        const long l0 = p->launches;
        e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_plan(p, nact, tw, logTW);
            e = cudaStreamEndCapture(p->stream, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&p->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(e); return -1; }
        p->graph_nq = nact;
        p->graph_node = p->d_node;
        p->graph_subset = p->subset;
        p->graph_launches = p->launches - l0;
        p->graph_tma = g_tma_launches.load() != tma0;
        p->launches = l0;
    }
    cudaEventRecord(p->ev0, p->stream);
    if (use_graph) {
        e = cudaGraphLaunch(p->graph, p->stream);
        if (e != cudaSuccess) { err = std::string("graph launch: ") + cudaGetErrorString(e); return -1; }
        p->launches += p->graph_launches;
    } else {
        enqueue_plan(p, nact, tw, logTW);
    }
    cudaEventRecord(p->ev1, p->stream);
    e = cudaGetLastError();
    if (dev) {   // equities into the caller's buffer; its stream waits for them
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(equity, p->d_out, sizeof(double) * p->n, cudaMemcpyDeviceToDevice, p->stream);
        if (e == cudaSuccess) e = cudaEventRecord(p->ev_out, p->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(dev->st, p->ev_out, 0);
        if (e != cudaSuccess) { err = std::string("execution: ") + cudaGetErrorString(e); return -1; }
        if (!p->prof.on) {   // no wait: the device time of this run is not read
            if (stats) {
                memset(stats, 0, sizeof(*stats));
                stats->total_ns = now_ns() - t0;
                stats->peak_vram_bytes = (size_t)p->peak_bytes;
                stats->engine = 1;
                stats->B = p->B;
            }
            return 0;
        }
        e = cudaStreamSynchronize(p->stream);
    } else {
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(equity, p->d_out, sizeof(double) * p->n, cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    }
    if (e != cudaSuccess) { err = std::string("execution: ") + cudaGetErrorString(e); return -1; }
    if (g_tma_launches.load() != tma0 || (use_graph && p->graph_tma)) {   // a TMA column pass ran: did every tile copy complete?
        const int f = tma_take_failures();
        if (f != 0) {
            err = "TMA tile copies of " + std::to_string(f) + " CTAs did not complete within the wait limit";
            return -1;
        }
    }
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        p->last_device_ms = ms;
    }
    if (p->prof.on) {
        for (const ProfRec &r : p->prof.recs) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.a, r.b);
            Plan::KStat *ks = nullptr;
            for (auto &x : p->kstats)
                if (x.name == r.name) ks = &x;
            if (!ks) { p->kstats.push_back({r.name, 0.0, 0, 0.0}); ks = &p->kstats.back(); }
            ks->ms += ms;
            ks->launches += 1;
            ks->flops += r.flops;
        }
    }
    const double t1 = now_ns();
    for (double &m : p->stage_ms) m = 0.0;
    for (size_t c = 0; c + 5 <= p->stage_used; c += 5)   // per chunk: 5 stage boundaries
        for (int st = 0; st < 4; ++st) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, p->stage_ev[c + st], p->stage_ev[c + st + 1]) == cudaSuccess)
                p->stage_ms[st] += ms;
        }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->total_ns = t1 - t0;
        stats->peak_vram_bytes = (size_t)p->peak_bytes;
        stats->engine = 1;
        stats->B = p->B;
        // stage times on the instrumented (verbose) path, as the reference reports them
        stats->block_build_ns = p->stage_ms[0] * 1e6;
        stats->tree_build_ns = p->stage_ms[1] * 1e6;
        stats->tree_propagate_cached_ns = p->stage_ms[2] * 1e6;
        stats->leaf_extract_ns = p->stage_ms[3] * 1e6;
    }
    return 0;
}

}  // namespace icmg
