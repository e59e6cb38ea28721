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
// Each CTA handles `cb` parents of one quadrature node (cb N <= 4096 complex
// points, or one parent at N = 8192), so every level is one launch per
// direction and no intermediate spectrum leaves shared memory except the
// children's spectra the propagate pass reuses.
#include "engine.h"
#include "fft.cuh"
#include "kernels.h"

namespace icmg {

constexpr int kFusedMaxN = 8192;
constexpr int kFusedThreads = 256;

__device__ __forceinline__ int fused_cb(int N) { return N >= 8192 ? 1 : 4096 / N; }

// shared memory per CTA: cb items, each N complex (forward) + N/2 complex (inverse)
static inline size_t fused_smem(int N) {
    const int cb = N >= 8192 ? 1 : 4096 / N;
    return (size_t)cb * (N + N / 2) * sizeof(double2);
}

__device__ void fused_build_body(const FusedBuildArgs &A, int bx, int q) {
    const auto Pc = A.Pc;
    const auto Pc_q = A.Pc_q;
    const auto pst_c = A.pst_c;
    const auto lc = A.lc;
    const auto npairs = A.npairs;
    const auto logN = A.logN;
    const auto Pp = A.Pp;
    const auto Pp_q = A.Pp_q;
    const auto pst_p = A.pst_p;
    const auto lp = A.lp;
    const auto spec = A.spec;
    const auto tw = A.tw;
    const auto logTW = A.logTW;
    const auto spectra_only = A.spectra_only;

    extern __shared__ double2 sm[];
    const int N = 1 << logN, h = N >> 1;
    const int cb = fused_cb(N);
        const int j0 = bx * cb;
    const int cnt = min(cb, npairs - j0);
    double2 *Z = sm;                 // cb x N
    double2 *U = sm + (size_t)cb * N; // cb x h
    const double *base = Pc + q * Pc_q;
    if (!spectra_only && zp_cold(A.z, q, j0 + cnt - 1)) {   // every parent x^deg (its spectra are never read)
        for (int e = threadIdx.x; e < cnt * pst_p; e += blockDim.x) {
            const int it = e / pst_p, t = e - it * pst_p;
            Pp[q * Pp_q + (size_t)(j0 + it) * pst_p + t] = (t == A.z.span && t < lp) ? 1.0 : 0.0;
        }
        return;
    }
    // 1. children into bit-reversed slots
    for (int e = threadIdx.x; e < cnt * N; e += blockDim.x) {
        const int it = e >> logN, s = e & (N - 1);
        const int t = (int)bitrev(s, logN);
        const double *L = base + (size_t)(2 * (j0 + it)) * pst_c;
        Z[e] = (t < lc) ? make_double2(L[t], L[pst_c + t]) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(Z, logN, cnt, tw, logTW);
    // 2. spectra of both children; half-size inverse input of their product
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e / h, f = e - it * h;
        const double2 *z = Z + (size_t)it * N;
        const int fc = h - f;
        const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
        const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
        const double2 SLf = cscale(cadd(zf, cconj(zn)), 0.5);
        const double2 SRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
        const double2 SLc = cscale(cadd(zc, cconj(zcn)), 0.5);
        const double2 SRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
        double2 *sL = spec + (2 * ((size_t)q * npairs + j0 + it)) * (size_t)(h + 1);
        double2 *sR = sL + (h + 1);
        sL[f] = SLf;
        sR[f] = SRf;
        if (f == 0) { sL[h] = SLc; sR[h] = SRc; }
        if (spectra_only) continue;
        const double2 Cf = cmul(SLf, SRf), Cc = cmul(SLc, SRc);
        double2 E = cadd(Cf, cconj(Cc)), D = csub(Cf, cconj(Cc));
        if (f == 0) { E.y = 0.0; D.y = 0.0; }
        const double2 O = cmulc(D, __ldg(&tw[(long)f << (logTW - logN)]));
        U[(size_t)it * h + bitrev(f, logN - 1)] = cadd(E, cmul_pi(O));
    }
    if (spectra_only) return;
    __syncthreads();
    smem_fft_dit<+1>(U, logN - 1, cnt, tw, logTW);
    // 3. product coefficients (endpoints from the children directly)
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < cnt * pst_p; e += blockDim.x) {
        const int it = e / pst_p, t = e - it * pst_p;
        double *out = Pp + q * Pp_q + (size_t)(j0 + it) * pst_p;
        double v = 0.0;
        if (t < lp) {
            const double *L = base + (size_t)(2 * (j0 + it)) * pst_c;
            if (t == 0) v = L[0] * L[pst_c];
            else if (t == N) v = L[lc - 1] * L[pst_c + lc - 1];
            else if (t < N) {
                const double2 uv = U[(size_t)it * h + (t >> 1)];
                v = ((t & 1) ? uv.y : uv.x) * inv;
            }
        }
        out[t] = v;
    }
}

__device__ void fused_prop_body(const FusedPropArgs &A, int bx, int q) {
    const auto gp = A.gp;
    const auto gp_q = A.gp_q;
    const auto gst_p = A.gst_p;
    const auto gpl = A.gpl;
    const auto npairs = A.npairs;
    const auto logN = A.logN;
    const auto spec = A.spec;
    const auto gc = A.gc;
    const auto gc_q = A.gc_q;
    const auto gst_c = A.gst_c;
    const auto gcl = A.gcl;
    const auto hot_c = A.hot_c;
    const auto tw = A.tw;
    const auto logTW = A.logTW;

    extern __shared__ double2 sm[];
    const int N = 1 << logN, h = N >> 1;
    const int cb = fused_cb(N);
        const int j0 = bx * cb;
    const int cnt = min(cb, npairs - j0);
    double2 *Z = sm;                  // cb x N
    double2 *W = sm + (size_t)cb * N; // cb x h
    if (zp_cold(A.z, q, j0 + cnt - 1)) return;   // wholly-zero parents: no child g is read
    if (hot_c) {   // subset pruning: nothing below a cold child is ever read
        bool any = false;
        for (int c = 2 * j0; c < 2 * (j0 + cnt); ++c) any = any || hot_c[c];
        if (!any) return;
    }
    // 1. parent g as w[t] = g[2t] + i g[2t+1], bit-reversed
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e / h, s = e - it * h;
        const int t = (int)bitrev(s, logN - 1);
        const double *g = gp + q * gp_q + (size_t)(j0 + it) * gst_p;
        const int t0 = 2 * t, t1 = 2 * t + 1;
        W[e] = make_double2(t0 < gpl ? g[t0] : 0.0, t1 < gpl ? g[t1] : 0.0);
    }
    __syncthreads();
    smem_fft_dit<-1>(W, logN - 1, cnt, tw, logTW);
    // 2. G, then Z = G conj(S_R) + i G conj(S_L) over all N bins (bit-reversed)
    for (int e = threadIdx.x; e < cnt * h; e += blockDim.x) {
        const int it = e / h, f = e - it * h;
        const double2 *w = W + (size_t)it * h;
        const double2 *sL = spec + (2 * ((size_t)q * npairs + j0 + it)) * (size_t)(h + 1);
        const double2 *sR = sL + (h + 1);
        double2 *z = Z + (size_t)it * N;
        const double2 wf = w[f], wc = w[(h - f) & (h - 1)];
        const double2 Ev = cscale(cadd(wf, cconj(wc)), 0.5);
        const double2 Od = cscale(cmul_mi(csub(wf, cconj(wc))), 0.5);
        const double2 G = cadd(Ev, cmul(Od, __ldg(&tw[(long)f << (logTW - logN)])));
        const double2 YL = cmulc(G, sR[f]), YR = cmulc(G, sL[f]);
        z[bitrev(f, logN)] = cadd(YL, cmul_pi(YR));
        if (f != 0) {
            z[bitrev(N - f, logN)] = cadd(cconj(YL), cmul_pi(cconj(YR)));
        } else {
            // bin h: W[h mod h] = W[0] on both sides; e^{-i pi} = -1
            const double2 Gh = csub(Ev, Od);
            const double2 YLh = cmulc(Gh, sR[h]), YRh = cmulc(Gh, sL[h]);
            z[bitrev(h, logN)] = cadd(YLh, cmul_pi(YRh));
        }
    }
    __syncthreads();
    smem_fft_dit<+1>(Z, logN, cnt, tw, logTW);
    // 3. children's g
    const double inv = 1.0 / N;
    for (int e = threadIdx.x; e < cnt * 2 * gst_c; e += blockDim.x) {
        const int it = e / (2 * gst_c), r = e - it * 2 * gst_c;
        const int side = r / gst_c, m = r - side * gst_c;
        const int c = 2 * (j0 + it) + side;
        double *out = gc + q * gc_q + (size_t)c * gst_c;
        double v = 0.0;
        if (m < gcl && !(hot_c && !hot_c[c])) {
            const double2 zv = Z[(size_t)it * N + m];
            v = (side ? zv.y : zv.x) * inv;
        }
        out[m] = v;
    }
}

__global__ void __launch_bounds__(kFusedThreads) k_fused_build(FusedBuildArgs A) { fused_build_body(A, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(kFusedThreads) k_fused_prop(FusedPropArgs A) { fused_prop_body(A, blockIdx.x, blockIdx.y); }

size_t fused_smem_bytes(int N) { return fused_smem(N); }
__global__ void kw_fused_build(const FusedBuildArgs *__restrict__ D, const int2 *__restrict__ tab, int q0);
__global__ void kw_fused_prop(const FusedPropArgs *__restrict__ D, const int2 *__restrict__ tab, int q0);

bool fused_ok(int N) { return N >= 8 && N <= kFusedMaxN; }

void fused_set_smem_limits() {
    const int mx = (int)fused_smem(kFusedMaxN);
    cudaFuncSetAttribute(k_fused_build, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fused_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_fused_build, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(kw_fused_prop, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

static int ilog2i(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

FusedBuildArgs fused_build_args(const Level &c, const Level &p, bool spectra_only, const double2 *tw, int logTW,
                                double *fq, size_t *smem) {
    const int N = p.fftn, logN = ilog2i(N);
    const int cb = N >= 8192 ? 1 : 4096 / N;
    // transforms: forward N (5 N log N) and inverse N/2; spectra/product ~40 flops per bin
    if (fq) *fq = (5.0 * N * logN + (spectra_only ? 8.0 : 40.0 + 2.5 * logN) * (N / 2)) * p.npairs;
    if (smem) *smem = fused_smem(N);
    return FusedBuildArgs{c.P, c.P_q, c.pst, c.plen, p.npairs, logN, p.P, p.P_q, p.pst, p.plen, p.spec, tw, logTW,
                          spectra_only ? 1 : 0, (p.npairs + cb - 1) / cb, ZeroPrefix{nullptr, 0, p.deg}};
}

FusedPropArgs fused_prop_args(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p,
                              const uint8_t *hot_c, const double2 *tw, int logTW, double *fq, size_t *smem) {
    const int N = p.fftn, logN = ilog2i(N);
    const int cb = N >= 8192 ? 1 : 4096 / N;
    if (fq) *fq = (5.0 * N * logN + 2.5 * N * (logN - 1) + 40.0 * (N / 2)) * p.npairs;
    if (smem) *smem = fused_smem(N);
    return FusedPropArgs{gp, gp_q, gst_p, gpl, p.npairs, logN, p.spec, c.g, c.g_q, c.gst, c.glen, hot_c, tw, logTW,
                         (p.npairs + cb - 1) / cb, ZeroPrefix{nullptr, 0, p.deg}};
}

void launch_fused_build(const Level &c, const Level &p, int nq, bool spectra_only, const double2 *tw, int logTW,
                        cudaStream_t st, Prof *pr, const int *zp, int zq0) {
    double fq = 0.0;
    size_t sm = 0;
    FusedBuildArgs A = fused_build_args(c, p, spectra_only, tw, logTW, &fq, &sm);
    A.z.zp = zp;
    A.z.q0 = zq0;
    pr->begin(spectra_only ? "fused_spectra" : "fused_build", fq * nq, st);
    k_fused_build<<<dim3(A.nbx, nq), kFusedThreads, sm, st>>>(A);
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
    pr->begin("fused_prop", fq * nq, st);
    k_fused_prop<<<dim3(A.nbx, nq), kFusedThreads, sm, st>>>(A);
    pr->end(st);
}

// ---------------------------------------------------------------- work lists
__global__ void __launch_bounds__(kFusedThreads)
kw_fused_build(const FusedBuildArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    FusedBuildArgs A = D[t.x];
    A.z.q0 = q0;
    fused_build_body(A, t.y, blockIdx.y);
}
__global__ void __launch_bounds__(kFusedThreads)
kw_fused_prop(const FusedPropArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    FusedPropArgs A = D[t.x];
    A.z.q0 = q0;
    fused_prop_body(A, t.y, blockIdx.y);
}

void launch_worklist_fused(WOp op, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                           cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    switch (op) {
        case WOp::FusedBuild: kw_fused_build<<<g, kFusedThreads, smem, st>>>((const FusedBuildArgs *)desc, tab, q0); break;
        case WOp::FusedProp: kw_fused_prop<<<g, kFusedThreads, smem, st>>>((const FusedPropArgs *)desc, tab, q0); break;
        default: break;
    }
}

}  // namespace icmg
