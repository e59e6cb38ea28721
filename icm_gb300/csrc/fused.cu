// fused.cu -- one-kernel FFT tree levels for real FFT sizes N <= kFusedMaxN.
//
// Build (parents of two children of length lc, product truncated to lp):
//   load z[t] = L[t] + i R[t] (bit-reversed into shared memory)
//   -> forward complex FFT of size N
//   -> both children's real spectra S_L, S_R (written to the spectrum cache
//      for the propagate pass) and the half-size inverse input
//      U[f] = E[f] + i O[f] of the product spectrum C = S_L S_R
//   -> inverse complex FFT of size N/2 -> product coefficients, with
//      coefficient 0 (and N when lp > N) taken directly from the children.
// Propagate (parent g of length gpl, children g of length gcl):
//   load w[t] = g[2t] + i g[2t+1] -> forward FFT of size N/2 -> parent real
//   spectrum G -> Z = G conj(S_R) + i G conj(S_L) over all N bins
//   -> inverse FFT of size N -> g_L = Re z / N, g_R = Im z / N.
// Each CTA handles `cb` parents of one quadrature node (cb N <= kFusedPts =
// 2048 complex points, or one parent at N >= 4096; 2048 rather than 4096
// measured 0.4% faster on the batched workload: 49 KB of shared memory per
// CTA instead of 98 KB), so every level is one launch per
// direction and no intermediate spectrum leaves shared memory except the
// children's spectra the propagate pass reuses.
#include <algorithm>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"

namespace icmg {

constexpr int kFusedMaxN = 8192;
constexpr int kFusedThreads = 256;
constexpr int kFusedThreadsMax = 512;   // CTAs alone on an SM (8192-point items) take twice the warps
static inline int fused_tpb(size_t smem) { return smem > kOneCtaSmem ? kFusedThreadsMax : kFusedThreads; }

// complex points per CTA of the one-kernel FFT levels (items = kFusedPts / N;
// one 8192-point item alone)
constexpr int kFusedPts = 2048;
__host__ __device__ __forceinline__ int fused_cb(int N) { return N >= kFusedPts ? 1 : kFusedPts / N; }


// Every item (pair of children) of a CTA is described by a view staged in
// shared memory after the transforms, so a CTA may hold items of different
// tournaments (packed work lists); wholly-zero items are pruned per item.
constexpr size_t kFusedViewBytes = 80;
constexpr size_t kFusedItemBytes = kFusedViewBytes + sizeof(int);
static inline size_t fused_smem_cb(int N, int cb) { return (size_t)cb * ((N + N / 2) * sizeof(double2) + kFusedItemBytes); }
static inline size_t fused_smem_v(int N) { return fused_smem_cb(N, fused_cb(N)); }

struct FbView {
    const double *L;   // left child coefficients (the right child's follow at + pst_c)
    double *out;       // parent coefficients (null: spectra only)
    double2 *sL;       // children's spectra cache (the right child's at + h + 1)
    long deg;          // parent degree (wholly-zero parents are x^deg)
    int pst_c, lc, pst_p, lp, cold;
};
static_assert(sizeof(FbView) <= kFusedViewBytes, "view size");
struct FpView {
    const double *g;   // parent g (the payout at the root)
    const double2 *sL; // children's spectra (the right child's at + h + 1)
    double *out0;      // g row of child 2j (child 2j+1's at + gst_c)
    int gpl, gst_c, gcl;
    int zero[2];       // subset-cold child: its g is zero
    int cold;          // wholly-zero parent: skipped
};
static_assert(sizeof(FpView) <= kFusedViewBytes, "view size");
__device__ __forceinline__ bool fitem_skip(const FbView &v) { return v.cold; }
__device__ __forceinline__ bool fitem_skip(const FpView &v) { return v.cold || (v.zero[0] && v.zero[1]); }

template <class View>
__device__ __forceinline__ int fpartition(const View *V, int *idx, int cnt) {
    __shared__ int nhot_s;
    if (threadIdx.x == 0) {
        int h = 0;
        for (int it = 0; it < cnt; ++it)
            if (!fitem_skip(V[it])) idx[h++] = it;
        int c = h;
        for (int it = 0; it < cnt; ++it)
            if (fitem_skip(V[it])) idx[c++] = it;
        nhot_s = h;
    }
    __syncthreads();
    return nhot_s;
}

__device__ __forceinline__ void fb_fill(const FusedBuildArgs &A, int q, int q0, int j, int h, FbView &v) {
    v.L = A.Pc + q * A.Pc_q + (size_t)(2 * j) * A.pst_c;
    v.out = A.spectra_only ? nullptr : A.Pp + q * A.Pp_q + (size_t)j * A.pst_p;
    v.sL = A.spec + (2 * ((size_t)q * A.npairs + j)) * (size_t)(h + 1);
    v.deg = A.z.span;
    v.pst_c = A.pst_c;
    v.lc = A.lc;
    v.pst_p = A.pst_p;
    v.lp = A.lp;
    const ZeroPrefix z{A.z.zp, q0, A.z.span};
    v.cold = (!A.spectra_only && zp_cold(z, q, j)) ? 1 : 0;
}

__device__ __forceinline__ void fp_fill(const FusedPropArgs &A, int q, int q0, int j, int h, FpView &v) {
    v.g = A.gp + q * A.gp_q + (size_t)j * A.gst_p;
    v.sL = A.spec + (2 * ((size_t)q * A.npairs + j)) * (size_t)(h + 1);
    v.out0 = A.gc + q * A.gc_q + (size_t)(2 * j) * A.gst_c;
    v.gpl = A.gpl;
    v.gst_c = A.gst_c;
    v.gcl = A.gcl;
    v.zero[0] = (A.hot_c && !A.hot_c[2 * j]) ? 1 : 0;
    v.zero[1] = (A.hot_c && !A.hot_c[2 * j + 1]) ? 1 : 0;
    const ZeroPrefix z{A.z.zp, q0, A.z.span};
    v.cold = zp_cold(z, q, j) ? 1 : 0;
}

// build of the items idx[0, nh) (wholly-zero ones idx[nh, cnt) written as monomials)
__device__ void fused_build_core(const FbView *V, const int *idx, int cnt, int nh, int cb, int logN,
                                 const double2 *__restrict__ tw, int logTW, double2 *sm, bool spectra_only) {
    const int N = 1 << logN, h = N >> 1;
    double2 *Z = sm;                   // cb x N
    double2 *U = sm + (size_t)cb * N;  // cb x h
    if (nh < cnt) {
        int maxpst = 0;
        for (int r = nh; r < cnt; ++r) maxpst = max(maxpst, V[idx[r]].pst_p);
        for (int e = threadIdx.x; e < (cnt - nh) * maxpst; e += blockDim.x) {
            const FbView &v = V[idx[nh + e / maxpst]];
            const int t = e % maxpst;
            if (t < v.pst_p) v.out[t] = (t == v.deg && t < v.lp) ? 1.0 : 0.0;   // x^deg
        }
    }
    if (nh == 0) return;
    // 1. children into bit-reversed slots
    for (int e = threadIdx.x; e < nh * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const FbView &v = V[idx[it]];
        Z[e] = (t < v.lc) ? make_double2(v.L[t], v.L[v.pst_c + t]) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, nh, tw, logTW);
    // 2. spectra of both children and the half-size inverse input of their
    //    product, by mirror pairs of bins (f, h - f), f <= h/2
    const double2 *tt = tw_tangent(tw, logTW);
    const int hp = (h >> 1) + 1;
    for (int e = threadIdx.x; e < nh * hp; e += blockDim.x) {
        const int it = e / hp, f = e - it * hp;
        const double2 *z = Z + (size_t)it * N;
        const int fc = h - f;
        const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
        const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
        const double2 SLf = cscale(cadd(zf, cconj(zn)), 0.5);
        const double2 SRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
        const double2 SLc = cscale(cadd(zc, cconj(zcn)), 0.5);
        const double2 SRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
        double2 *sL = V[idx[it]].sL;
        double2 *sR = sL + (h + 1);
        sL[f] = SLf;
        sR[f] = SRf;
        if (fc != f) { sL[fc] = SLc; sR[fc] = SRc; }   // f = 0: bin h
        if (spectra_only) continue;
        const double2 Cf = cmul(SLf, SRf), Cc = cmul(SLc, SRc);
        double2 E = cadd(Cf, cconj(Cc)), D = csub(Cf, cconj(Cc));
        if (f == 0) { E.y = 0.0; D.y = 0.0; }
        double2 Uf, Uc;   // O = D e^{+2 pi i f/N}; Uc is U[h - f]
        mirror_inv_input(E, D, tt, (long)f << (logTW - logN), logTW, Uf, Uc);
        U[(size_t)it * h + bitrev(f, logN - 1)] = Uf;
        if (f != 0 && fc != f) U[(size_t)it * h + bitrev(fc, logN - 1)] = Uc;
    }
    if (spectra_only) return;
    __syncthreads();
    smem_fft_dit<+1>(U, logN - 1, nh, tw, logTW);
    // 3. product coefficients (endpoints from the children directly)
    int maxpst = 0;
    for (int it = 0; it < nh; ++it) maxpst = max(maxpst, V[idx[it]].pst_p);
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < nh * maxpst; e += blockDim.x) {
        const int it = e / maxpst, t = e - it * maxpst;
        const FbView &v = V[idx[it]];
        if (t >= v.pst_p) continue;
        double val = 0.0;
        if (t < v.lp) {
            const double *L = v.L;
            const int pst_c = v.pst_c, lc = v.lc;
            if (t == 0) val = L[0] * L[pst_c];
            else if (t == N) val = L[lc - 1] * L[pst_c + lc - 1];
            else if (t < N) {
                const double2 uv = U[(size_t)it * h + (t >> 1)];
                val = ((t & 1) ? uv.y : uv.x) * inv;
            }
        }
        v.out[t] = val;
    }
}

// propagate of the items idx[0, nh) (the others: nothing below them is read)
__device__ void fused_prop_core(const FpView *V, const int *idx, int nh, int cb, int logN,
                                const double2 *__restrict__ tw, int logTW, double2 *sm) {
    const int N = 1 << logN, h = N >> 1;
    double2 *Z = sm;                   // cb x N
    double2 *W = sm + (size_t)cb * N;  // cb x h
    if (nh == 0) return;
    // 1. parent g as w[t] = g[2t] + i g[2t+1], bit-reversed
    for (int e = threadIdx.x; e < nh * h; e += blockDim.x) {
        const int it = e / h, s = e - it * h;
        const int t = (int)bitrev(s, logN - 1);
        const FpView &v = V[idx[it]];
        const int t0 = 2 * t, t1 = 2 * t + 1;
        W[e] = make_double2(t0 < v.gpl ? v.g[t0] : 0.0, t1 < v.gpl ? v.g[t1] : 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(W, logN - 1, nh, tw, logTW);
    // 2. G by mirror pairs of bins (f, h - f), f <= h/2 (G[h - f] =
    //    conj(Ev - w Od) / 2), then Z = G conj(S_R) + i G conj(S_L) over all N
    //    bins (bit-reversed)
    const double2 *tt = tw_tangent(tw, logTW);
    const int hp = (h >> 1) + 1;
    for (int e = threadIdx.x; e < nh * hp; e += blockDim.x) {
        const int it = e / hp, f = e - it * hp;
        const int fc = h - f;
        const double2 *w = W + (size_t)it * h;
        const double2 *sL = V[idx[it]].sL;
        const double2 *sR = sL + (h + 1);
        double2 *z = Z + (size_t)it * N;
        const double2 wf = w[f], wc = w[fc & (h - 1)];
        const double2 Ev = cadd(wf, cconj(wc)), Od = cmul_mi(csub(wf, cconj(wc)));   // both doubled
        double r;
        const double2 u = tanmul_t<-1>(Od, tt, (long)f << (logTW - logN), logTW, &r);
        const double hr = 0.5 * r;
        const double2 E5 = cscale(Ev, 0.5);
        const double2 Gf = make_double2(fma(hr, u.x, E5.x), fma(hr, u.y, E5.y));
        const double2 Gc = make_double2(fma(-hr, u.x, E5.x), fma(hr, u.y, -E5.y));
        auto bin = [&](int b, double2 G) {   // bins b and N - b
            const double2 YL = cmulc(G, sR[b]), YR = cmulc(G, sL[b]);
            z[bitrev(b, logN)] = cadd(YL, cmul_pi(YR));
            if (b != 0 && b != h) z[bitrev(N - b, logN)] = cadd(cconj(YL), cmul_pi(cconj(YR)));
        };
        bin(f, Gf);
        if (fc != f) bin(fc, Gc);   // f = 0: bin h (W[h mod h] = W[0]; e^{-i pi} = -1)
    }
    __syncthreads();
    smem_fft_dit<+1>(Z, logN, nh, tw, logTW);
    // 3. children's g
    int maxgst = 0;
    for (int it = 0; it < nh; ++it) maxgst = max(maxgst, V[idx[it]].gst_c);
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < nh * 2 * maxgst; e += blockDim.x) {
        const int it = e / (2 * maxgst), r = e - it * 2 * maxgst;
        const int side = r / maxgst, m = r - side * maxgst;
        const FpView &v = V[idx[it]];
        if (m >= v.gst_c) continue;
        double val = 0.0;
        if (m < v.gcl && !v.zero[side]) {
            const double2 zv = Z[(size_t)it * N + m];
            val = (side ? zv.y : zv.x) * inv;
        }
        v.out0[side * v.gst_c + m] = val;
    }
}

__device__ void fused_build_body(const FusedBuildArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int N = 1 << A.logN, h = N >> 1;
    const int cb = A.cb;
    const int j0 = bx * cb;
    const int cnt = min(cb, A.npairs - j0);
    if (cnt <= 0) return;
    FbView *V = reinterpret_cast<FbView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kFusedViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) fb_fill(A, q, A.z.q0, j0 + it, h, V[it]);
    __syncthreads();
    const int nh = fpartition(V, idx, cnt);
    fused_build_core(V, idx, cnt, nh, cb, A.logN, A.tw, A.logTW, sm, A.spectra_only != 0);
}

__device__ void fused_prop_body(const FusedPropArgs &A, int bx, int q) {
    extern __shared__ double2 sm[];
    const int N = 1 << A.logN, h = N >> 1;
    const int cb = A.cb;
    const int j0 = bx * cb;
    const int cnt = min(cb, A.npairs - j0);
    if (cnt <= 0) return;
    FpView *V = reinterpret_cast<FpView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kFusedViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) fp_fill(A, q, A.z.q0, j0 + it, h, V[it]);
    __syncthreads();
    const int nh = fpartition(V, idx, cnt);
    fused_prop_core(V, idx, nh, cb, A.logN, A.tw, A.logTW, sm);
}

// packed: slots[s] = (descriptor, pair); a launch shares N and spectra_only
__device__ void fused_build_packed(const FusedBuildArgs *__restrict__ Dsc, const int2 *__restrict__ slots, int nslots,
                                   int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const FusedBuildArgs &A0 = Dsc[slots[0].x];
    const int N = 1 << A0.logN, h = N >> 1;
    const int cb = fused_cb(N);
    const int s0 = bx * cb;
    const int cnt = min(cb, nslots - s0);
    if (cnt <= 0) return;
    FbView *V = reinterpret_cast<FbView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kFusedViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        fb_fill(Dsc[sl.x], q, q0, sl.y, h, V[it]);
    }
    __syncthreads();
    const int nh = fpartition(V, idx, cnt);
    fused_build_core(V, idx, cnt, nh, cb, A0.logN, A0.tw, A0.logTW, sm, A0.spectra_only != 0);
}

__device__ void fused_prop_packed(const FusedPropArgs *__restrict__ Dsc, const int2 *__restrict__ slots, int nslots,
                                  int bx, int q, int q0) {
    extern __shared__ double2 sm[];
    const FusedPropArgs &A0 = Dsc[slots[0].x];
    const int N = 1 << A0.logN, h = N >> 1;
    const int cb = fused_cb(N);
    const int s0 = bx * cb;
    const int cnt = min(cb, nslots - s0);
    if (cnt <= 0) return;
    FpView *V = reinterpret_cast<FpView *>(sm + (size_t)cb * (N + h));
    int *idx = reinterpret_cast<int *>(reinterpret_cast<char *>(V) + (size_t)cb * kFusedViewBytes);
    for (int it = threadIdx.x; it < cnt; it += blockDim.x) {
        const int2 sl = slots[s0 + it];
        fp_fill(Dsc[sl.x], q, q0, sl.y, h, V[it]);
    }
    __syncthreads();
    const int nh = fpartition(V, idx, cnt);
    fused_prop_core(V, idx, nh, cb, A0.logN, A0.tw, A0.logTW, sm);
}

__global__ void __launch_bounds__(kFusedThreadsMax) k_fused_build(FusedBuildArgs A) { fused_build_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kFusedThreadsMax) k_fused_prop(FusedPropArgs A) { fused_prop_body(A, blockIdx.x, blockIdx.y); }

size_t fused_smem_bytes(int N) { return fused_smem_v(N); }
static size_t fused_smem_v_max() {
    size_t mx = 0;
    for (int N = 8; N <= kFusedMaxN; N *= 2) mx = std::max(mx, fused_smem_v(N));
    return mx;
}

bool fused_ok(int N) { return N >= 8 && N <= kFusedMaxN; }

__global__ void __launch_bounds__(kFusedThreadsMax)
kw_fused_build_packed(const FusedBuildArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    fused_build_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}
__global__ void __launch_bounds__(kFusedThreadsMax)
kw_fused_prop_packed(const FusedPropArgs *__restrict__ D, const int2 *__restrict__ slots, int nslots, int q0) {
    fused_prop_packed(D, slots, nslots, blockIdx.x, blockIdx.y, q0);
}

void launch_packed_fused(WOp op, const void *desc, const int2 *slots, int nslots, int cb, int nq, int q0, size_t smem,
                         cudaStream_t st) {
    if (nslots <= 0 || nq <= 0) return;
    const dim3 g((nslots + cb - 1) / cb, nq);
    if (op == WOp::FusedBuild)
        kw_fused_build_packed<<<g, fused_tpb(smem), smem, st>>>((const FusedBuildArgs *)desc, slots, nslots, q0);
    else
        kw_fused_prop_packed<<<g, fused_tpb(smem), smem, st>>>((const FusedPropArgs *)desc, slots, nslots, q0);
}

void fused_set_smem_limits() {
    const int mx = (int)fused_smem_v_max();
    cudaFuncSetAttribute(kw_fused_build_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_fused_prop_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fused_build, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fused_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

static int ilog2i(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

FusedBuildArgs fused_build_args(const Level &c, const Level &p, bool spectra_only, const double2 *tw, int logTW,
                                double *fq, size_t *smem) {
    const int N = p.fftn, logN = ilog2i(N);
    const int cb = fused_cb(N);
    // transforms: forward N (5 N log N) and inverse N/2; spectra/product ~40 flops per bin
    if (fq) *fq = (5.0 * N * logN + (spectra_only ? 8.0 : 40.0 + 2.5 * logN) * (N / 2)) * p.npairs;
    if (smem) *smem = fused_smem_v(N);
    return FusedBuildArgs{c.P, c.P_q, c.pst, c.plen, p.npairs, logN, p.P, p.P_q, p.pst, p.plen, p.spec, tw, logTW,
                          spectra_only ? 1 : 0, (p.npairs + cb - 1) / cb, ZeroPrefix{nullptr, 0, p.deg}, cb};
}

FusedPropArgs fused_prop_args(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p,
                              const uint8_t *hot_c, const double2 *tw, int logTW, double *fq, size_t *smem) {
    const int N = p.fftn, logN = ilog2i(N);
    const int cb = fused_cb(N);
    if (fq) *fq = (5.0 * N * logN + 2.5 * N * (logN - 1) + 40.0 * (N / 2)) * p.npairs;
    if (smem) *smem = fused_smem_v(N);
    return FusedPropArgs{gp, gp_q, gst_p, gpl, p.npairs, logN, p.spec, c.g, c.g_q, c.gst, c.glen, hot_c, tw, logTW,
                         (p.npairs + cb - 1) / cb, ZeroPrefix{nullptr, 0, p.deg}, cb};
}

void launch_fused_build(const Level &c, const Level &p, int nq, bool spectra_only, const double2 *tw, int logTW,
                        cudaStream_t st, Prof *pr, const int *zp, int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    FusedBuildArgs A = fused_build_args(c, p, spectra_only, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(A.cb, p.npairs, nq);
    A.nbx = (p.npairs + A.cb - 1) / A.cb;
    sm = fused_smem_cb(1 << A.logN, A.cb);
    pr->begin(spectra_only ? "fused_spectra" : "fused_build", fq * nq, st);
    k_fused_build<<<dim3(A.nbx, nq), fused_tpb(sm), sm, st>>>(A);
    pr->end(st);
}

void launch_fused_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                       const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr, const int *zp,
                       int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    FusedPropArgs A = fused_prop_args(gp, gp_q, gst_p, gpl, c, p, hot_c, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    A.cb = short_grid_cb(A.cb, p.npairs, nq);
    A.nbx = (p.npairs + A.cb - 1) / A.cb;
    sm = fused_smem_cb(1 << A.logN, A.cb);
    pr->begin("fused_prop", fq * nq, st);
    k_fused_prop<<<dim3(A.nbx, nq), fused_tpb(sm), sm, st>>>(A);
    pr->end(st);
}


}  // namespace icmg
