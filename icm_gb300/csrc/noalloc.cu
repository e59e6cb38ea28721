// noalloc.cu -- icm_gpu_equity_noalloc: the equity solve for callers that
// cannot allocate device memory.
//
// Who needs it: hosts that forbid device allocation after start-up (real-time
// or embedded services that size every buffer once, so that a solve can never
// fail or stall on an allocator), and processes whose device memory belongs to
// another allocator (a framework's caching pool that has reserved the GPU's
// memory, where a cudaMalloc of our own would either fail or break the pool's
// budget and fragment it).  For them this entry point computes the same
// equities as icm_equity, for tournaments of up to kNoallocMaxN players, using
// only memory that already exists: the caller's host arrays and one
// file-scope device array, g_noalloc_scratch, of kNoallocBytes.  That array is
// part of the library image, so every GPU that loads libicm_gb300.so holds it
// until the process exits.
//
// The call makes no cudaMalloc, cudaFree, stream or event creation, and no
// allocating library call.  Everything it needs on the device (sorted
// stacks, quadrature nodes, twiddles, tree levels, FFT work buffers,
// per-node partials) is carved from the scratch array; the quadrature nodes
// are processed in chunks sized so the carve fits.  It runs on the library's
// device (the one icm_gpu_init chose; device 0 when nothing was initialised),
// restores the caller's current device before returning, puts its copies and
// launches on the legacy default stream, and returns after the result is on
// the host.  Its tree uses coefficient-FFT levels throughout (no spectral
// levels, which need per-plan buffers), with the block size and FFT crossover
// the allocating path picks, so its equities agree with icm_equity's to
// rounding (about 1e-13 relative), not bit for bit.
//
// Set-up: the first call on a device, with that device current, resolves the
// array's device address with cudaGetSymbolAddress (the host-side name of a
// __device__ array is only a stand-in, not a device address) and caches it,
// once per device under a lock.  That first call should come before any stream
// capture begins.
//
// Every call shares the one array and overwrites what the previous call left
// there (the accumulator is cleared by each call); calls that overlap on the
// GPU (two host threads at once) race and corrupt each other.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"

namespace icmg {

constexpr int kNoallocMaxN = 4096;                 // players
constexpr int kNoallocMaxQ = 4096;                 // quadrature nodes
constexpr size_t kNoallocBytes = (size_t)32 << 20; // 32 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

static std::mutex g_noalloc_mu;        // guards the per-device address cache

// host copy of the twiddle tables per table size, built once (the upload
// reads it on every call; entries are never replaced)
static const std::vector<unsigned char> &host_twiddles(int logTW) {
    static std::mutex mu;
    static std::vector<unsigned char> tabs[32];
    std::lock_guard<std::mutex> lock(mu);
    if (tabs[logTW].empty()) fill_twiddles(logTW, tabs[logTW]);
    return tabs[logTW];
}
static char *g_noalloc_ptr[64] = {};   // device address per device, set up once

// The scratch array's device address on the current device (resolved once per
// device, with that device current); nullptr with the reason in err.
static char *noalloc_scratch(std::string &err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return nullptr; }
    if (dev < 0 || dev >= 64) { err = "device index out of range"; return nullptr; }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev]) return g_noalloc_ptr[dev];
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
        err = std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e);
        return nullptr;
    }
    g_noalloc_ptr[dev] = (char *)ptr;
    return g_noalloc_ptr[dev];
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Geometry of the same tree the allocating path builds (engine.cu), with
// every buffer placed inside [base, base + kNoallocBytes).
struct NoallocPlan {
    int n, k, B, nblocks, L, qc, logTW;
    Level lv[kMaxLevels];
    double *d_S, *d_payout, *d_a, *d_blockP, *d_contrib, *d_acc, *d_out, *d_node;
    int *d_perm;
    double2 *tw, *fa, *fb, *fc;
};

static int noalloc_plan(NoallocPlan &p, int n, int k, int nact, char *base, std::string &err) {
    p.n = n;
    p.k = k;
    p.B = select_block_size(n, k);
    const int B = p.B;
    const int fft_min = select_fft_min(n, k);   // the allocating path's crossover
    p.nblocks = (n + B - 1) / B;
    int Nt = 1;
    while (Nt < p.nblocks) Nt <<= 1;
    p.L = 1;
    while ((1 << (p.L - 1)) < Nt) ++p.L;
    size_t fa = 0, fb = 0, per_q = 0;
    int logN = 12;
    for (int l = 0; l < p.L; ++l) {
        Level &v = p.lv[l];
        v = Level();
        v.nreal = (l == 0) ? p.nblocks : (p.lv[l - 1].nreal + 1) / 2;
        v.deg = (long)B << l;
        v.plen = (int)std::min<long>(v.deg + 1, k);
        v.glen = (int)std::min<long>(v.deg, k);
        v.pst = (v.plen + 1) & ~1;
        v.gst = (v.glen + 1) & ~1;
        if (l >= 1) {
            const Level &c = p.lv[l - 1];
            v.npairs = c.nreal / 2;
            v.fft = (c.deg >= fft_min) ? 1 : 0;
            if (v.fft) {
                const long need = std::max<long>(2L * c.plen - 2, (long)c.glen + c.plen - 1);
                int N = 4;
                while (N < need) N <<= 1;
                v.fftn = N;
                int lg = 0;
                while ((1 << lg) < N) ++lg;
                logN = std::max(logN, lg);
            }
        }
        if (l <= p.L - 2 || l == 0) {
            v.P_q = (size_t)v.nreal * v.pst;
            v.g_q = (size_t)v.nreal * v.gst;
        }
        if (l >= 1 && v.fft) {
            v.spec_q = (size_t)2 * v.npairs * (v.fftn / 2 + 1);
            fa = std::max(fa, (size_t)v.npairs * v.fftn);
            fb = std::max(fb, (size_t)v.npairs * (v.fftn / 2));
        }
        per_q += al256(v.P_q * 8) + al256(v.g_q * 8) + al256(v.spec_q * 16);
    }
    per_q += al256((size_t)n * 8) * 2 + al256((size_t)p.nblocks * (B + 1) * 8);
    per_q += al256(fa * 16) * 2 + al256(std::max(fa, fb) * 16);
    p.logTW = logN;
    const size_t fixed = al256((size_t)n * 8) * 3 + al256((size_t)n * 4) + al256((size_t)k * 8) +
                         al256((size_t)3 * std::max(nact, 1) * 8) + al256(twiddle_bytes(logN)) +
                         (size_t)kMaxLevels * 3 * 256 + 4096;
    if (fixed + per_q > kNoallocBytes) {
        err = "tournament needs " + std::to_string(fixed + per_q) + " bytes of scratch for one node; the "
              "no-allocation scratch holds " + std::to_string(kNoallocBytes);
        return -1;
    }
    p.qc = (int)std::min<size_t>(256, (kNoallocBytes - fixed) / per_q);
    size_t off = 0;
    auto take = [&](size_t bytes) { char *r = base + off; off += al256(bytes); return r; };
    p.d_S = (double *)take((size_t)n * 8);
    p.d_acc = (double *)take((size_t)n * 8);
    p.d_out = (double *)take((size_t)n * 8);
    p.d_perm = (int *)take((size_t)n * 4);
    p.d_payout = (double *)take((size_t)k * 8);
    p.d_node = (double *)take((size_t)3 * std::max(nact, 1) * 8);
    p.tw = (double2 *)take(twiddle_bytes(logN));
    p.d_a = (double *)take((size_t)p.qc * n * 8);
    p.d_contrib = (double *)take((size_t)p.qc * n * 8);
    p.d_blockP = (double *)take((size_t)p.qc * p.nblocks * (B + 1) * 8);
    for (int l = 0; l < p.L; ++l) {
        Level &v = p.lv[l];
        v.P = v.P_q ? (double *)take((size_t)p.qc * v.P_q * 8) : nullptr;
        v.g = v.g_q ? (double *)take((size_t)p.qc * v.g_q * 8) : nullptr;
        v.spec = v.spec_q ? (double2 *)take((size_t)p.qc * v.spec_q * 16) : nullptr;
    }
    p.fa = fa ? (double2 *)take((size_t)p.qc * fa * 16) : nullptr;
    p.fb = fa ? (double2 *)take((size_t)p.qc * std::max(fa, fb) * 16) : nullptr;
    p.fc = fa ? (double2 *)take((size_t)p.qc * fa * 16) : nullptr;
    if (off > kNoallocBytes) { err = "no-allocation scratch layout overflow"; return -1; }
    return 0;
}

}  // namespace icmg

using namespace icmg;

namespace icmg {
void api_set_error(const std::string &e);   // api.cpp: the text icm_gpu_last_error returns
}

// The solve behind icm_gpu_equity_noalloc.
static int noalloc_solve(int n, const double *S, int Q, const double *payout, int k, double *equity) {
    std::string err;
    auto fail = [&](const std::string &m) {
        api_set_error("icm_gpu_equity_noalloc: " + m);
        return -1;
    };
    if (n < 1 || k < 1 || k > n || Q < 1 || !S || !payout || !equity) return fail("invalid arguments (need 1 <= k <= n, Q >= 1)");
    if (n > kNoallocMaxN)
        return fail("n=" + std::to_string(n) + " exceeds the no-allocation limit of " + std::to_string(kNoallocMaxN) +
                    " players; use icm_equity");
    if (Q > kNoallocMaxQ)
        return fail("Q=" + std::to_string(Q) + " exceeds the no-allocation limit of " + std::to_string(kNoallocMaxQ));
    for (int i = 0; i < n; ++i)
        if (!(S[i] > 0.0) || !std::isfinite(S[i])) return fail("stacks must be finite and positive");
    if (g_device < 0 && icm_gpu_init(0) != 1) return fail("no usable CUDA device");
    if (cudaSetDevice(g_device) != cudaSuccess) return fail("cudaSetDevice failed");
    char *scratch = noalloc_scratch(err);
    if (!scratch) return fail(err);

    // host-side preparation: sort (descending, ties by index), nodes, twiddles
    std::vector<int> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    std::sort(perm.begin(), perm.end(), [S](int a, int b) { return S[a] > S[b] || (S[a] == S[b] && a < b); });
    std::vector<double> Ss(n);
    for (int i = 0; i < n; ++i) Ss[i] = S[perm[i]];
    std::vector<double> logv, w, node;
    make_nodes(Q, Ss[0], logv, w);
    for (int q = 0; q < Q; ++q) {
        if (w[q] == 0.0) continue;
        node.push_back(logv[q]);
        node.push_back(w[q]);
        node.push_back(std::exp(-logv[q]));
    }
    const int nact = (int)(node.size() / 3);
    NoallocPlan p;
    if (noalloc_plan(p, n, k, nact, scratch, err) != 0) return fail(err);
    const std::vector<unsigned char> &tw = host_twiddles(p.logTW);

    cudaStream_t st = 0;   // legacy default stream: no stream creation
    cudaError_t e = cudaMemcpyAsync(p.d_S, Ss.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p.d_perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p.d_payout, payout, sizeof(double) * k, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nact)
        e = cudaMemcpyAsync(p.d_node, node.data(), sizeof(double) * node.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p.tw, tw.data(), tw.size(), cudaMemcpyHostToDevice, st);
    // the accumulator must start at zero when no node has weight
    if (e == cudaSuccess) e = cudaMemsetAsync(p.d_acc, 0, sizeof(double) * n, st);
    if (e != cudaSuccess) return fail(std::string("upload: ") + cudaGetErrorString(e));

    Prof off;   // timing disabled: no events
    long launches = 0;
    Level *lv = p.lv;
    const int L = p.L;
    for (int q0 = 0; q0 < nact; q0 += p.qc) {
        const int nq = std::min(p.qc, nact - q0);
        launch_leaf(p.B, n, p.nblocks, p.d_S, p.d_node, q0, nq, p.d_a, p.d_blockP, lv[0].P, lv[0].pst, lv[0].plen,
                    st, &off);
        for (int l = 1; l <= L - 2; ++l) {
            if (lv[l].fft) {
                launch_fft_build(lv[l - 1], lv[l], nq, p.fa, p.fb, p.fc, false, p.tw, p.logTW, st, &launches, &off);
                if (lv[l - 1].nreal & 1) launch_school_build(lv[l - 1], lv[l], nq, lv[l].npairs, st, &off);
            } else {
                launch_school_build(lv[l - 1], lv[l], nq, 0, st, &off);
            }
        }
        if (L >= 2 && lv[L - 1].fft)
            launch_fft_build(lv[L - 2], lv[L - 1], nq, p.fa, p.fb, p.fc, true, p.tw, p.logTW, st, &launches, &off);
        for (int l = L - 1; l >= 1; --l) {
            const bool root = (l == L - 1);
            const double *gp = root ? p.d_payout : lv[l].g;
            const size_t gp_q = root ? 0 : lv[l].g_q;
            const int gst_p = root ? 0 : lv[l].gst;
            const int gpl = root ? k : lv[l].glen;
            if (lv[l].fft) {
                launch_fft_prop(gp, gp_q, gst_p, gpl, lv[l - 1], lv[l], nq, nullptr, p.fa, p.fb, p.fc, p.tw, p.logTW,
                                st, &launches, &off);
                if (lv[l - 1].nreal & 1)
                    launch_school_prop(gp, gp_q, gst_p, gpl, lv[l - 1], nq, nullptr, 2 * lv[l].npairs, st, &off);
            } else {
                launch_school_prop(gp, gp_q, gst_p, gpl, lv[l - 1], nq, nullptr, 0, st, &off);
            }
        }
        const double *g0 = (L == 1) ? p.d_payout : lv[0].g;
        launch_divide(p.B, n, k, p.nblocks, p.d_S, p.d_node, q0, nq, p.d_a, p.d_blockP, g0, (L == 1) ? 0 : lv[0].g_q,
                      (L == 1) ? 0 : lv[0].gst, nullptr, p.d_contrib, st, &off);
        launch_accumulate(n, nq, p.d_contrib, p.d_acc, q0 == 0 ? 1 : 0, st, &off);
    }
    launch_scatter(n, p.d_acc, p.d_perm, nullptr, p.d_out, st);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(equity, p.d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(std::string("execution: ") + cudaGetErrorString(e));
    return 0;
}

// See icm_gb300.h.  Host arrays in and out; 0 on success, -1 on failure with
// the reason in icm_gpu_last_error().  The caller's current device is restored
// before returning; a C++ exception (a host allocation that fails) becomes -1.
extern "C" int icm_gpu_equity_noalloc(int n, const double *S, int Q, const double *payout, int k,
                                      double *equity) {
    int caller_dev = -1;
    if (cudaGetDevice(&caller_dev) != cudaSuccess) caller_dev = -1;
    int rc = -1;
    try {
        rc = noalloc_solve(n, S, Q, payout, k, equity);
    } catch (const std::exception &e) {
        api_set_error(std::string("icm_gpu_equity_noalloc: ") + e.what());
        rc = -1;
    } catch (...) {
        api_set_error("icm_gpu_equity_noalloc: unknown error");
        rc = -1;
    }
    if (caller_dev >= 0) cudaSetDevice(caller_dev);
    return rc;
}
