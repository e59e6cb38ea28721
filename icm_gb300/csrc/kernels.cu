// kernels.cu -- device kernels of the GB300 ICM engine and their launchers.
//
// Per quadrature node q the engine evaluates (reference src/cpu/icm.c:2523-2695)
//   a_i = exp(S_i logv_q)                    (0 when S_i logv_q < -700)
//   inner_i = sum_{m<k} payout[m] [x^m] prod_{j != i} (a_j + (1-a_j) x)
//   equity_i += w_q S_i a_i / v_q * inner_i  (non-finite weight -> 0)
// through a subproduct tree over blocks of B players (sorted by stack,
// descending): leaf block products, truncated products up the tree, middle
// products of the payout down the tree, then a per-player synthetic
// division of its block product fused with the dot against the block's g.
//
// Every kernel covers a whole chunk of nodes: blockIdx.y (or the batch
// index) selects the node, so one launch per tree level serves qc trees.
#include <algorithm>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"
#include "leafdiv.cuh"

namespace icmg {

// ------------------------------------------------------------------ leaves
// Leaf factors and block products (leafdiv.cuh).  One thread per (node, block);
// the block product lives in registers.
template <int B>
__device__ __forceinline__ void leaf_body_t(const LeafArgs &A, int bx, int q) {
    const int b = bx * blockDim.x + threadIdx.x;
    if (b >= A.nblocks) return;
    const int n = A.n, nblocks = A.nblocks;
    const double logv = A.node[3 * (A.q0 + q)];
    const int start = b * B;
    const int bs = min(B, n - start);
    double P[B + 1];
    block_product<B>(A.S + start, bs, logv, A.a + (size_t)q * A.aq + start, P);
    double *bp = A.blockP + ((size_t)q * nblocks + b) * (B + 1);
#pragma unroll
    for (int m = 0; m <= B; ++m) bp[m] = P[m];
    const int pst0 = A.pst0, plen0 = A.plen0;
    double *leaf = A.P0 + ((size_t)q * nblocks + b) * pst0;
#pragma unroll
    for (int m = 0; m <= B; ++m)
        if (m < pst0) leaf[m] = (m < plen0) ? P[m] : 0.0;
    for (int m = B + 1; m < pst0; ++m) leaf[m] = 0.0;
}

// leaf factors of given arguments, as the leaves compute them (checks)
__global__ void k_leaf_factors(int n, const double *__restrict__ arg, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = leaf_factor(arg[i]);
}

int leaf_factors(int n, const double *arg, double *out, std::string &err) {
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(d, arg, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_leaf_factors<<<(n + 255) / 256, 256>>>(n, d, d + n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) { err = std::string("leaf factors: ") + cudaGetErrorString(e); return -1; }
    return 0;
}

// one kernel per block size: registers sized for that B
template <int B>
__global__ void k_leaf_t(LeafArgs A) { leaf_body_t<B>(A, blockIdx.x, blockIdx.y); }

// ------------------------------------------------------- schoolbook build
// parent j = L*R mod x^lp, children of length lc (reference icm.c:465-480);
// parents >= j0 only (the FFT path uses j0 = npairs to let this kernel copy a
// lone left child).  Output t of the full product has min(t, 2lc-2-t) + 1
// terms, a triangle: one thread per output idles half the lanes of a warp.
// Instead each thread takes a work item of two outputs whose term counts add
// up to lc -- t and lc-2-t below the middle, t and 3lc-2-t above it -- and
// walks both in one loop of uniform length.  Per output the terms are summed
// in the same order as one thread per output would.
__device__ __forceinline__ void school_item(int lc, int w, int *t1, int *t2) {
    const int h = lc >> 1;   // pairs per half: ceil((lc - 1) / 2)
    *t2 = -1;
    if (w < h) {
        *t1 = w;
        *t2 = lc - 2 - w;
    } else if (w == h) {
        *t1 = lc - 1;   // the middle output: lc terms
    } else if (w < 2 * h + 1) {
        const int u = w - h - 1;
        *t1 = lc + u;
        *t2 = 2 * lc - 2 - u;
    } else {
        *t1 = 2 * lc - 1;   // the padding slot past the full product
    }
    if (*t2 == *t1) *t2 = -1;
}
__host__ __device__ __forceinline__ int school_items(int lc) { return 2 * (lc >> 1) + 2; }

__device__ void school_build_body(const SchoolBuildArgs &A, int bx, int q) {
    const long idx = (long)bx * blockDim.x + threadIdx.x;
    const int pst_p = A.pst_p, pst_c = A.pst_c, lc = A.lc, lp = A.lp;
    const int W = school_items(lc);
    const int j = A.j0 + (int)(idx / W);
    const int w = (int)(idx % W);
    if (j >= A.nreal_p) return;
    int t1, t2;
    school_item(lc, w, &t1, &t2);
    const double *L = A.Pc + q * A.Pc_q + (size_t)(2 * j) * pst_c;
    double *out = A.Pp + q * A.Pp_q + (size_t)j * pst_p;
    double v1 = 0.0, v2 = 0.0;
    if (zp_cold(A.z, q, j)) {   // x^deg
        v1 = (t1 == A.z.span && t1 < lp) ? 1.0 : 0.0;
        v2 = (t2 == A.z.span && t2 < lp) ? 1.0 : 0.0;
    } else if (2 * j + 1 >= A.nreal_c) {   // lone child copied up
        v1 = (t1 < lc && t1 < lp) ? L[t1] : 0.0;
        v2 = (t2 >= 0 && t2 < lc && t2 < lp) ? L[t2] : 0.0;
    } else {
        const double *R = L + pst_c;
        const int F = 2 * lc - 1;
        const int lo1 = max(0, t1 - (lc - 1));
        const int c1 = (t1 < lp && t1 < F) ? min(t1, lc - 1) - lo1 + 1 : 0;
        const int lo2 = max(0, t2 - (lc - 1));
        const int c2 = (t2 >= 0 && t2 < lp) ? min(t2, lc - 1) - lo2 + 1 : 0;
        double s1 = 0.0, s2 = 0.0;
        for (int r = 0; r < c1 + c2; ++r) {
            const bool first = r < c1;
            const int t = first ? t1 : t2;
            const int i = first ? lo1 + r : lo2 + (r - c1);
            const double acc = fma(L[i], R[t - i], first ? s1 : s2);
            s1 = first ? acc : s1;
            s2 = first ? s2 : acc;
        }
        v1 = s1;
        v2 = s2;
    }
    if (t1 < pst_p) out[t1] = v1;
    if (t2 >= 0 && t2 < pst_p) out[t2] = v2;
}

__global__ void k_school_build(SchoolBuildArgs A) { school_build_body(A, blockIdx.x, blockIdx.y); }

// --------------------------------------------------- schoolbook propagate
// g_c[m] = sum_i P_sib[i] g_parent[m+i] (reference icm.c:489-507, 1667-1819).
// One thread per child coefficient, children >= c0 only.  gp_q == 0 lets the
// root's g be the payout vector shared by all nodes.
__device__ void school_prop_body(const SchoolPropArgs &A, int bx, int q) {
    const long idx = (long)bx * blockDim.x + threadIdx.x;
    const int gst_c = A.gst_c;
    const int c = A.c0 + (int)(idx / gst_c);
    const int m = (int)(idx % gst_c);
    if (c >= A.nreal_c || zp_cold(A.z, q, c)) return;
    double *out = A.gc + q * A.gc_q + (size_t)c * gst_c;
    if (m >= A.gcl || (A.hot_c && !A.hot_c[c])) { out[m] = 0.0; return; }
    const double *g = A.gp + q * A.gp_q + (size_t)(c >> 1) * A.gst_p;
    const int sib = c ^ 1;
    const int gpl = A.gpl;
    if (sib >= A.nreal_c) { out[m] = (m < gpl) ? g[m] : 0.0; return; }
    const double *P = A.Pc + q * A.Pc_q + (size_t)sib * A.pst_c;
    const int imax = min(A.lc, gpl - m);
    double s = 0.0;
    for (int i = 0; i < imax; ++i) s = fma(P[i], g[m + i], s);
    out[m] = s;
}

__global__ void k_school_prop(SchoolPropArgs A) { school_prop_body(A, blockIdx.x, blockIdx.y); }

// --------------------------------------------------------- divide + dot
// Per player: Q_i = P_block / (a_i + (1-a_i) x) by the forward recurrence
// when a_i > 0.5, the backward one when a_i > 1e-15, else a shift; then
// inner_i = sum_{m < min(bs,k)} g_block[m] Q_i[m] and the node's weight
// (reference icm.c:2230-2302 and 2584-2589).
template <int B>
__device__ __forceinline__ void divide_body_t(const DivideArgs &A, int bx, int q) {
    const int i = bx * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (i >= n) return;
    double *out = A.contrib + (size_t)q * A.aq + i;
    if (A.active && !A.active[i]) { *out = 0.0; return; }
    const double *nd = A.node + 3 * (A.q0 + q);
    if (nd[1] == 0.0) { *out = 0.0; return; }   // zero-weight node (the reference skips it)
    const int b = i / B;
    const int start = b * B;
    const int bs = min(B, n - start);
    const int pk = min(bs, A.k);
    const double a = A.a[(size_t)q * A.aq + i];
    if (a == 0.0) { *out = 0.0; return; }   // S logv < -700: zero weight (g of its block may be pruned)
    const double *P = A.blockP + ((size_t)q * A.nblocks + b) * (B + 1);
    const double *g = A.g0 + q * A.g0_q + (size_t)b * A.gst0;
    const double eq = divide_dot<B>(a, P, bs, pk, g);
    double pw = nd[1] * A.S[i] * a * nd[2];
    if (!isfinite(pw)) pw = 0.0;
    *out = pw * eq;
}

template <int B>
__global__ void k_divide_t(DivideArgs A) { divide_body_t<B>(A, blockIdx.x, blockIdx.y); }

// ordered sum over the chunk's nodes: deterministic for a fixed chunking
__global__ void k_accumulate(int n, int nq, const double *__restrict__ contrib, double *__restrict__ acc,
                             int first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = first ? 0.0 : acc[i];
    for (int q = 0; q < nq; ++q) s += contrib[(size_t)q * n + i];
    acc[i] = s;
}

__global__ void k_scatter(int n, const double *__restrict__ acc, const int *__restrict__ perm,
                          const uint8_t *__restrict__ active, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[perm[i]] = (active && !active[i]) ? 0.0 : acc[i];
}

// --------------------------------------------------------------- FFT core
// Batched complex transforms of size 2^logM, in place in `data` (natural
// order).  Sizes up to kSmemFftMax run in one kernel; larger sizes use the
// four-step split M = M1 * M2 through `scratch`.
__device__ __forceinline__ bool fft_skip(const FftSkip &k, long item) {
    if (!k.zp) return false;
    const long it = k.item0 + item;
    const long q = it / k.per_q, j = it - q * k.per_q;
    return (j + 1) * k.span <= (long)k.zp[k.q0 + q];
}

template <int SIGN, int SHIFT = 0>
__global__ void k_fft_smem(double2 *__restrict__ data, long batch, int logM, int cb,
                           const double2 *__restrict__ tw, int logTW, FftSkip skip) {
    extern __shared__ double2 sx[];
    const int M = 1 << logM;
    const long item0 = (long)blockIdx.x * cb;
    const int cnt = (int)min((long)cb, batch - item0);
    if (skip.zp) {   // every item of the block wholly zero: nothing reads them
        bool all = true;
        for (int it = 0; it < cnt; ++it) all = all && fft_skip(skip, item0 + it);
        if (all) return;
    }
    for (int e = threadIdx.x; e < cnt * M; e += blockDim.x) {
        const int it = e >> logM, s = e & (M - 1);
        sx[e] = data[(item0 + it) * M + bitrev(s, logM)];
    }
    __syncthreads();
    smem_fft_dit<SIGN, SHIFT>(sx, logM, cnt, tw, logTW);
    for (int e = threadIdx.x; e < cnt * M; e += blockDim.x) data[item0 * M + e] = sx[e];
}

// four-step, pass A: columns n2 of the M1 x M2 view x[M2 n1 + n2]; SHIFT =
// +1 / -1 makes the whole transform half-shifted (forward only): half-shifted
// column transforms and twiddles W_M^{n2 (k1 + SHIFT/2)}, plain rows
template <int SIGN, int SHIFT = 0>
__global__ void k_fft4_cols(const double2 *__restrict__ in, double2 *__restrict__ out, int logM1, int logM2,
                            int cb, const double2 *__restrict__ tw, int logTW, FftSkip skip) {
    extern __shared__ double2 sx[];
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    const long item = blockIdx.y;
    if (fft_skip(skip, item)) return;
    const int n20 = blockIdx.x * cb;
    const double2 *src = in + (item << (logM1 + logM2));
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int c = e % cb, s = e / cb;
        sx[c * M1 + s] = src[(long)bitrev(s, logM1) * M2 + n20 + c];
    }
    __syncthreads();
    smem_fft_dit<SIGN, SHIFT>(sx, logM1, cb, tw, logTW);
    const int logM = logM1 + logM2;
    double2 *dst = out + (item << logM);
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int c = e >> logM1, k1 = e & (M1 - 1);
        const int n2 = n20 + c;
        const long t = fft4_tw_index<SHIFT>(n2, k1, logM, logTW);
        double2 v = sx[e];
        if (t) v = twmul<SIGN>(v, __ldg(&tw[t]));
        dst[(long)n2 * M1 + k1] = v;
    }
}

// four-step, pass B: rows k1, FFT over n2, output X[k1 + M1 k2]
template <int SIGN>
__global__ void k_fft4_rows(const double2 *__restrict__ in, double2 *__restrict__ out, int logM1, int logM2,
                            int cb, const double2 *__restrict__ tw, int logTW, FftSkip skip) {
    extern __shared__ double2 sx[];
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    const long item = blockIdx.y;
    if (fft_skip(skip, item)) return;
    const int k10 = blockIdx.x * cb;
    const double2 *src = in + (item << (logM1 + logM2));
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int c = e % cb, s = e / cb;
        sx[c * M2 + s] = src[(long)bitrev(s, logM2) * M1 + k10 + c];
    }
    __syncthreads();
    smem_fft_dit<SIGN>(sx, logM2, cb, tw, logTW);
    double2 *dst = out + (item << (logM1 + logM2));
    for (int e = threadIdx.x; e < cb * M2; e += blockDim.x) {
        const int c = e % cb, k2 = e / cb;
        dst[(long)k2 * M1 + k10 + c] = sx[c * M2 + k2];
    }
}

int fft_batched(double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw, int logTW,
                cudaStream_t st, long *launches, Prof *pr, FftSkip skip, int shift) {
    if (batch <= 0) return 0;
    const int M = 1 << logM;
    const int threads = 256;
    if (M <= kSmemFftMax) {
        const int cb = short_grid_cb((M >= 4096) ? 1 : 4096 / M, (int)std::min(batch, 1L << 30), 1);
        const long blocks = (batch + cb - 1) / cb;
        const size_t smem = (size_t)cb * M * sizeof(double2);
        // one CTA per SM when the transform takes more than half the shared
        // memory: twice the warps to hide the butterflies' latency
        const int tpb = smem > kOneCtaSmem ? 512 : threads;
        pr->begin("fft_smem", 5.0 * M * logM * (double)batch, st);
        if (shift > 0)
            k_fft_smem<-1, +1><<<(unsigned)blocks, tpb, smem, st>>>(data, batch, logM, cb, tw, logTW, skip);
        else if (shift < 0)
            k_fft_smem<-1, -1><<<(unsigned)blocks, tpb, smem, st>>>(data, batch, logM, cb, tw, logTW, skip);
        else if (sign < 0)
            k_fft_smem<-1><<<(unsigned)blocks, tpb, smem, st>>>(data, batch, logM, cb, tw, logTW, skip);
        else
            k_fft_smem<+1><<<(unsigned)blocks, tpb, smem, st>>>(data, batch, logM, cb, tw, logTW, skip);
        pr->end(st);
        ++*launches;
        return 0;
    }
    if (batch > 65535) {   // grid.y limit of the four-step kernels
        for (long b0 = 0; b0 < batch; b0 += 65535) {
            FftSkip sk = skip;
            sk.item0 += b0;
            fft_batched(data + (b0 << logM), scratch + (b0 << logM), std::min(65535L, batch - b0), logM, sign, tw,
                        logTW, st, launches, pr, sk, shift);
        }
        return 0;
    }
    const int logM1 = (logM + 1) / 2, logM2 = logM - logM1;
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    // columns (rows) per CTA: 4096 points' worth, fewer on short grids
    const int cbA = short_grid_cb(max(1, min(M2, 4096 / M1)), M2, (int)batch);
    const int cbB = short_grid_cb(max(1, min(M1, 4096 / M2)), M1, (int)batch);
    dim3 gA(M2 / cbA, (unsigned)batch), gB(M1 / cbB, (unsigned)batch);
    const size_t smA = (size_t)cbA * M1 * sizeof(double2), smB = (size_t)cbB * M2 * sizeof(double2);
    pr->begin("fft4_cols", (5.0 * logM1 + 6.0) * M * (double)batch, st);
    if (shift > 0) k_fft4_cols<-1, +1><<<gA, threads, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else if (shift < 0) k_fft4_cols<-1, -1><<<gA, threads, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else if (sign < 0) k_fft4_cols<-1><<<gA, threads, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else k_fft4_cols<+1><<<gA, threads, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    pr->end(st);
    pr->begin("fft4_rows", 5.0 * logM2 * M * (double)batch, st);
    if (sign < 0) k_fft4_rows<-1><<<gB, threads, smB, st>>>(scratch, data, logM1, logM2, cbB, tw, logTW, skip);
    else k_fft4_rows<+1><<<gB, threads, smB, st>>>(scratch, data, logM1, logM2, cbB, tw, logTW, skip);
    pr->end(st);
    *launches += 2;
    return 0;
}

std::atomic<long> g_tma_launches{0};

void launch_fft4_cols(const double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw,
                      int logTW, cudaStream_t st, long *launches, Prof *pr, FftSkip skip, int shift) {
    if (batch <= 0) return;
    if (batch > 65535) {   // grid.y limit
        for (long b0 = 0; b0 < batch; b0 += 65535) {
            FftSkip sk = skip;
            sk.item0 += b0;
            launch_fft4_cols(data + (b0 << logM), scratch + (b0 << logM), std::min(65535L, batch - b0), logM, sign, tw,
                             logTW, st, launches, pr, sk, shift);
        }
        return;
    }
    const int logM1 = (logM + 1) / 2, logM2 = logM - logM1;
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    const int cbA = short_grid_cb(max(1, min(M2, 4096 / M1)), M2, (int)batch);
    dim3 gA(M2 / cbA, (unsigned)batch);
    const size_t smA = (size_t)cbA * M1 * sizeof(double2);
    pr->begin("fft4_cols", (5.0 * logM1 + 6.0) * (double)(1L << logM) * (double)batch, st);
    // the tile staged by TMA (measured 0.4-1% faster than the gathers below,
    // bitwise the same); the plain gathers where a tensor map cannot be made
    // or the configuration asks for them
    const bool tma = g_config.disable_tma != 1 && launch_fft4_cols_tma(data, scratch, batch, logM, sign, tw, logTW,
                                                                       cbA, st, skip, shift);
    if (tma) ++g_tma_launches;
    else if (shift > 0) k_fft4_cols<-1, +1><<<gA, 256, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else if (shift < 0) k_fft4_cols<-1, -1><<<gA, 256, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else if (sign < 0) k_fft4_cols<-1><<<gA, 256, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    else k_fft4_cols<+1><<<gA, 256, smA, st>>>(data, scratch, logM1, logM2, cbA, tw, logTW, skip);
    pr->end(st);
    ++*launches;
}

void vjp_set_smem_limits();   // vjp.cu

void fft_set_smem_limits() {
    fused_set_smem_limits();
    tma_set_smem_limits();
    specbig_set_smem_limits();
    spec_set_smem_limits();
    vjp_set_smem_limits();
    sub_set_smem_limits();
    small_set_smem_limits();
    const int mx = kSmemFftMax * (int)sizeof(double2);
    cudaFuncSetAttribute(k_fft_smem<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft_smem<+1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft_smem<-1, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft_smem<-1, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols<+1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols<-1, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols<-1, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_rows<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_rows<+1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

// ------------------------------------------------------ FFT tree levels
// Build at an FFT level: children L, R of length lc packed as z = L + iR,
// one complex transform of size N gives both spectra; the product spectrum
// goes back through a half-size complex transform (real-output packing).
// N >= 2 lc - 2, so only coefficient 0 can alias (with coefficient N); it is
// taken directly as L[0] R[0], and coefficient N (needed when lp > N) as
// L[lc-1] R[lc-1].
__global__ void k_pack_pair(const double *__restrict__ Pc, size_t Pc_q, int pst_c, int lc, int npairs, int N,
                            double2 *__restrict__ z) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int j = (int)(idx / N), t = (int)(idx % N);
    if (j >= npairs) return;
    const double *L = Pc + q * Pc_q + (size_t)(2 * j) * pst_c;
    const double *R = L + pst_c;
    z[((size_t)q * npairs + j) * N + t] = (t < lc) ? make_double2(L[t], R[t]) : make_double2(0.0, 0.0);
}

// spectra of both children from Z = FFT(L + iR); optionally the product's
// half-size inverse input U[f] = E[f] + i O[f].
__global__ void k_build_mid(const double2 *__restrict__ Z, int npairs, int N, double2 *__restrict__ spec,
                            double2 *__restrict__ U, const double2 *__restrict__ tw, int logTW, int logN) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = N >> 1;
    const int j = (int)(idx / h), f = (int)(idx % h);
    if (j >= npairs) return;
    const size_t item = (size_t)q * npairs + j;
    const double2 *z = Z + item * N;
    const int fc = h - f;                       // partner frequency for the real inverse
    const double2 zf = z[f], zn = z[(N - f) & (N - 1)];
    const double2 zc = z[fc], zcn = z[(N - fc) & (N - 1)];
    // S_L = (Z[f] + conj Z[-f]) / 2, S_R = (Z[f] - conj Z[-f]) / (2i)
    const double2 SLf = cscale(cadd(zf, cconj(zn)), 0.5);
    const double2 SRf = cscale(cmul_mi(csub(zf, cconj(zn))), 0.5);
    double2 *sL = spec + (2 * item) * (size_t)(h + 1);
    double2 *sR = sL + (h + 1);
    sL[f] = SLf;
    sR[f] = SRf;
    const double2 SLc = cscale(cadd(zc, cconj(zcn)), 0.5);
    const double2 SRc = cscale(cmul_mi(csub(zc, cconj(zcn))), 0.5);
    if (f == 0) { sL[h] = SLc; sR[h] = SRc; }
    if (!U) return;
    const double2 Cf = cmul(SLf, SRf);
    const double2 Cc = cmul(SLc, SRc);
    // E = C[f] + conj C[h-f];  O = (C[f] - conj C[h-f]) e^{+2 pi i f/N}
    double2 E = cadd(Cf, cconj(Cc));
    double2 D = csub(Cf, cconj(Cc));
    if (f == 0) { E.y = 0.0; D.y = 0.0; }
    const double2 w = __ldg(&tw[(long)f << (logTW - logN)]);
    const double2 O = cmulc(D, w);
    U[item * h + f] = cadd(E, cmul_pi(O));
}

__global__ void k_build_post(const double2 *__restrict__ u, int npairs, int N,
                             const double *__restrict__ Pc, size_t Pc_q, int pst_c, int lc,
                             double *__restrict__ Pp, size_t Pp_q, int pst_p, int lp) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int j = (int)(idx / pst_p), t = (int)(idx % pst_p);
    if (j >= npairs) return;
    double *out = Pp + q * Pp_q + (size_t)j * pst_p;
    if (t >= lp) { out[t] = 0.0; return; }
    const double *L = Pc + q * Pc_q + (size_t)(2 * j) * pst_c;
    const double *R = L + pst_c;
    double v;
    if (t == 0) v = L[0] * R[0];
    else if (t == N) v = L[lc - 1] * R[lc - 1];
    else if (t > N) v = 0.0;
    else {
        const double2 uv = u[((size_t)q * npairs + j) * (N >> 1) + (t >> 1)];
        v = ((t & 1) ? uv.y : uv.x) * (1.0 / N);
    }
    out[t] = v;
}

// Propagate at an FFT level: W = FFT_{N/2}(g[2t] + i g[2t+1]) gives the
// parent's real spectrum G; Y_L = G conj(S_R), Y_R = G conj(S_L); one size-N
// inverse of Z = Y_L + i Y_R yields both children's g (cyclic correlation,
// exact because N >= glen_child + lc - 1).
__global__ void k_prop_pack(const double *__restrict__ gp, size_t gp_q, int gst_p, int gpl, int npairs, int N,
                            const uint8_t *__restrict__ hot_c, double2 *__restrict__ w) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = N >> 1;
    const int j = (int)(idx / h), t = (int)(idx % h);
    if (j >= npairs) return;
    const double *g = gp + q * gp_q + (size_t)j * gst_p;
    const int t0 = 2 * t, t1 = 2 * t + 1;
    double2 v = make_double2(t0 < gpl ? g[t0] : 0.0, t1 < gpl ? g[t1] : 0.0);
    if (hot_c && !hot_c[2 * j] && !hot_c[2 * j + 1]) v = make_double2(0.0, 0.0);
    w[((size_t)q * npairs + j) * h + t] = v;
}

__global__ void k_prop_mid(const double2 *__restrict__ W, const double2 *__restrict__ spec, int npairs, int N,
                           double2 *__restrict__ Z, const double2 *__restrict__ tw, int logTW, int logN) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int h = N >> 1;
    const int j = (int)(idx / (h + 1)), f = (int)(idx % (h + 1));
    if (j >= npairs) return;
    const size_t item = (size_t)q * npairs + j;
    const double2 *w = W + item * h;
    const double2 wf = w[f & (h - 1)], wc = w[(h - f) & (h - 1)];
    // G[f] = (W[f] + conj W[h-f])/2 + e^{-2 pi i f/N} (W[f] - conj W[h-f]) / (2i)
    const double2 Ev = cscale(cadd(wf, cconj(wc)), 0.5);
    const double2 Od = cscale(cmul_mi(csub(wf, cconj(wc))), 0.5);
    const double2 tf = __ldg(&tw[(long)f << (logTW - logN)]);
    const double2 G = cadd(Ev, cmul(Od, tf));
    const double2 *sL = spec + (2 * item) * (size_t)(h + 1);
    const double2 *sR = sL + (h + 1);
    const double2 YL = cmulc(G, sR[f]);
    const double2 YR = cmulc(G, sL[f]);
    double2 *z = Z + item * N;
    z[f] = cadd(YL, cmul_pi(YR));
    if (f != 0 && f != h) z[N - f] = cadd(cconj(YL), cmul_pi(cconj(YR)));
}

__global__ void k_prop_post(const double2 *__restrict__ Z, int npairs, int N, double *__restrict__ gc,
                            size_t gc_q, int gst_c, int gcl, const uint8_t *__restrict__ hot_c) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    const int c = (int)(idx / gst_c), m = (int)(idx % gst_c);
    if (c >= 2 * npairs) return;
    double *out = gc + q * gc_q + (size_t)c * gst_c;
    if (m >= gcl || (hot_c && !hot_c[c])) { out[m] = 0.0; return; }
    const double2 zv = Z[((size_t)q * npairs + (c >> 1)) * N + m];
    out[m] = ((c & 1) ? zv.y : zv.x) * (1.0 / N);
}

// ------------------------------------------------------------ launchers
static inline unsigned nblk(long work, int threads) { return (unsigned)((work + threads - 1) / threads); }

LeafArgs leaf_args(int B, int n, int nblocks, const double *S, const double *node, double *a, size_t aq,
                   double *blockP, double *P0, int pst0, int plen0, double *fq) {
    LeafArgs A{};
    A.B = B; A.n = n; A.nblocks = nblocks; A.S = S; A.node = node; A.q0 = 0;
    A.a = a; A.blockP = blockP; A.P0 = P0; A.pst0 = pst0; A.plen0 = plen0;
    A.nbx = (int)nblk(nblocks, 128);
    A.aq = aq;
    if (fq) {   // reference recurrence: per player bs coefficient updates (2 mul + 1 add) and P[0] *= a
        const int r = n % B;
        *fq = (double)(n / B) * B * (3.0 * B + 1.0) + (double)r * (3.0 * r + 1.0);
    }
    return A;
}

DivideArgs divide_args(int B, int n, int k, int nblocks, const double *S, const double *node, const double *a,
                       size_t aq, const double *blockP, const double *g0, size_t g0_q, int gst0, const uint8_t *active,
                       double *contrib, double *fq) {
    DivideArgs A{};
    A.B = B; A.n = n; A.k = k; A.nblocks = nblocks; A.S = S; A.node = node; A.q0 = 0;
    A.a = a; A.blockP = blockP; A.g0 = g0; A.g0_q = g0_q; A.gst0 = gst0; A.active = active; A.contrib = contrib;
    A.nbx = (int)nblk(n, 128);
    A.aq = aq;
    if (fq) *fq = (double)n * (5.0 * std::min(B, k) + 4.0);   // divide 3 + dot 2 per term, weight 4
    return A;
}

SchoolBuildArgs school_build_args(const Level &c, const Level &p, int j0, double *fq) {
    const long work = (long)(p.nreal - j0) * school_items(c.plen);
    SchoolBuildArgs A{c.P, c.P_q, c.pst, c.plen, c.nreal, p.P, p.P_q, p.pst, p.plen, p.nreal, j0,
                      work > 0 ? (int)nblk(work, 256) : 0, ZeroPrefix{nullptr, 0, p.deg}};
    if (fq) {
        double terms = 0.0;   // multiply-adds of one full pair: sum_t (ihi - ilo + 1)
        for (int t = 0; t < p.plen; ++t) terms += std::min(t, c.plen - 1) - std::max(0, t - (c.plen - 1)) + 1;
        const long pairs = std::max(0, std::min(p.nreal, c.nreal / 2) - j0);
        *fq = 2.0 * terms * pairs;
    }
    return A;
}

SchoolPropArgs school_prop_args(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const uint8_t *hot_c,
                                int c0, double *fq) {
    const long work = (long)(c.nreal - c0) * c.gst;
    SchoolPropArgs A{gp, gp_q, gst_p, gpl, c.P, c.P_q, c.pst, c.plen, c.g, c.g_q, c.gst, c.glen, c.nreal, hot_c, c0,
                     work > 0 ? (int)nblk(work, 256) : 0, ZeroPrefix{nullptr, 0, c.deg}};
    if (fq) {
        double terms = 0.0;   // per child with a sibling: sum_m min(lc, gpl - m)
        for (int m = 0; m < c.glen; ++m) terms += std::max(0, std::min(c.plen, gpl - m));
        const long kids = std::max(0, 2 * (c.nreal / 2) - c0);
        *fq = 2.0 * terms * kids;
    }
    return A;
}

void launch_leaf(int B, int n, int nblocks, const double *S, const double *node, int q0, int nq, double *a,
                 double *blockP, double *P0, int pst0, int plen0, cudaStream_t st, Prof *pr) {
    double fq = 0.0;
    LeafArgs A = leaf_args(B, n, nblocks, S, node, a, (size_t)n, blockP, P0, pst0, plen0, &fq);
    A.q0 = q0;
    pr->begin("leaf", fq * nq, st);
    const dim3 g(A.nbx, nq);
    switch (B) {
        case 4: k_leaf_t<4><<<g, 128, 0, st>>>(A); break;
        case 8: k_leaf_t<8><<<g, 128, 0, st>>>(A); break;
        case 16: k_leaf_t<16><<<g, 128, 0, st>>>(A); break;
        default: k_leaf_t<32><<<g, 128, 0, st>>>(A); break;
    }
    pr->end(st);
}

void launch_divide(int B, int n, int k, int nblocks, const double *S, const double *node, int q0, int nq,
                   const double *a, const double *blockP, const double *g0, size_t g0_q, int gst0,
                   const uint8_t *active, double *contrib, cudaStream_t st, Prof *pr) {
    double fq = 0.0;
    DivideArgs A = divide_args(B, n, k, nblocks, S, node, a, (size_t)n, blockP, g0, g0_q, gst0, active, contrib, &fq);
    A.q0 = q0;
    pr->begin("divide", fq * nq, st);
    const dim3 g(A.nbx, nq);
    switch (B) {
        case 4: k_divide_t<4><<<g, 128, 0, st>>>(A); break;
        case 8: k_divide_t<8><<<g, 128, 0, st>>>(A); break;
        case 16: k_divide_t<16><<<g, 128, 0, st>>>(A); break;
        default: k_divide_t<32><<<g, 128, 0, st>>>(A); break;
    }
    pr->end(st);
}

void launch_school_build(const Level &c, const Level &p, int nq, int j0, cudaStream_t st, Prof *pr, const int *zp,
                         int zq0) {
    double fq = 0.0;
    SchoolBuildArgs A = school_build_args(c, p, j0, &fq);
    A.z.zp = zp;
    A.z.q0 = zq0;
    if (A.nbx <= 0) return;
    pr->begin("school_build", fq * nq, st);
    k_school_build<<<dim3(A.nbx, nq), 256, 0, st>>>(A);
    pr->end(st);
}

void launch_school_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, int nq,
                        const uint8_t *hot_c, int c0, cudaStream_t st, Prof *pr, const int *zp, int zq0) {
    double fq = 0.0;
    SchoolPropArgs A = school_prop_args(gp, gp_q, gst_p, gpl, c, hot_c, c0, &fq);
    A.z.zp = zp;
    A.z.q0 = zq0;
    if (A.nbx <= 0) return;
    pr->begin("school_prop", fq * nq, st);
    k_school_prop<<<dim3(A.nbx, nq), 256, 0, st>>>(A);
    pr->end(st);
}

// ---------------------------------------------------------------- work lists
template <int B>
__global__ void kw_leaf(const LeafArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    LeafArgs A = D[t.x];
    A.q0 = q0;
    leaf_body_t<B>(A, t.y, blockIdx.y);
}
template <int B>
__global__ void kw_divide(const DivideArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    DivideArgs A = D[t.x];
    A.q0 = q0;
    divide_body_t<B>(A, t.y, blockIdx.y);
}
__global__ void kw_school_build(const SchoolBuildArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    SchoolBuildArgs A = D[t.x];
    A.z.q0 = q0;
    school_build_body(A, t.y, blockIdx.y);
}
__global__ void kw_school_prop(const SchoolPropArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    SchoolPropArgs A = D[t.x];
    A.z.q0 = q0;
    school_prop_body(A, t.y, blockIdx.y);
}

void launch_worklist_basic(WOp op, int B, const void *desc, const int2 *tab, int nctas, int nq, int q0,
                           cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    const LeafArgs *DL = (const LeafArgs *)desc;
    const DivideArgs *DD = (const DivideArgs *)desc;
    switch (op) {
        case WOp::Leaf:
            switch (B) {
                case 4: kw_leaf<4><<<g, 128, 0, st>>>(DL, tab, q0); break;
                case 8: kw_leaf<8><<<g, 128, 0, st>>>(DL, tab, q0); break;
                case 16: kw_leaf<16><<<g, 128, 0, st>>>(DL, tab, q0); break;
                default: kw_leaf<32><<<g, 128, 0, st>>>(DL, tab, q0); break;
            }
            break;
        case WOp::Divide:
            switch (B) {
                case 4: kw_divide<4><<<g, 128, 0, st>>>(DD, tab, q0); break;
                case 8: kw_divide<8><<<g, 128, 0, st>>>(DD, tab, q0); break;
                case 16: kw_divide<16><<<g, 128, 0, st>>>(DD, tab, q0); break;
                default: kw_divide<32><<<g, 128, 0, st>>>(DD, tab, q0); break;
            }
            break;
        case WOp::SchoolBuild: kw_school_build<<<g, 256, 0, st>>>((const SchoolBuildArgs *)desc, tab, q0); break;
        case WOp::SchoolProp: kw_school_prop<<<g, 256, 0, st>>>((const SchoolPropArgs *)desc, tab, q0); break;
        default: break;
    }
}

void launch_accumulate(int n, int nq, const double *contrib, double *acc, int first, cudaStream_t st, Prof *pr) {
    pr->begin("accumulate", (double)n * nq, st);
    k_accumulate<<<nblk(n, 256), 256, 0, st>>>(n, nq, contrib, acc, first);
    pr->end(st);
}

// Items per CTA of a single-plan FFT-level launch: the default (4096 points
// per CTA) unless the launch would then have fewer than two CTAs
// per SM, in which case fewer items per CTA (halving) spread it over more SMs.
// Each item's arithmetic is the same either way.
int short_grid_cb(int cb, int nitems, int nq) {
    static const int sms = [] {   // thread-safe one-time query of the SM count
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        return v;
    }();
    while (cb > 1 && (long)((nitems + cb - 1) / cb) * nq < 2L * sms) cb >>= 1;
    return cb;
}

void launch_scatter(int n, const double *acc, const int *perm, const uint8_t *active, double *out,
                    cudaStream_t st) {
    k_scatter<<<nblk(n, 256), 256, 0, st>>>(n, acc, perm, active, out);
}

// FFT build for parents [0, npairs) of level p (children c); spectra only when
// U == nullptr (the root level, whose product is never used).
void launch_fft_build(const Level &c, const Level &p, int nq, double2 *fa, double2 *fb, double2 *fc,
                      bool spectra_only, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr,
                      const int *zp, int zq0) {
    const int N = p.fftn, npairs = p.npairs;
    if (npairs <= 0) return;
    if (fused_ok(N)) {
        launch_fused_build(c, p, nq, spectra_only, tw, logTW, st, pr, zp, zq0);
        ++*launches;
        return;
    }
    int logN = 0;
    while ((1 << logN) < N) ++logN;
    const double items = (double)nq * npairs;
    const double sc = pr->scale;   // the multi-pass path computes every parent
    pr->scale = 1.0;
    dim3 g1(nblk((long)npairs * N, 256), nq);
    pr->begin("fft_pack", 0.0, st);
    k_pack_pair<<<g1, 256, 0, st>>>(c.P, c.P_q, c.pst, c.plen, npairs, N, fa);
    pr->end(st);
    fft_batched(fa, fc, (long)nq * npairs, logN, -1, tw, logTW, st, launches, pr);
    dim3 g2(nblk((long)npairs * (N / 2), 256), nq);
    pr->begin("build_mid", items * (N / 2) * (spectra_only ? 8.0 : 40.0), st);
    k_build_mid<<<g2, 256, 0, st>>>(fa, npairs, N, p.spec, spectra_only ? nullptr : fb, tw, logTW, logN);
    pr->end(st);
    *launches += 2;
    if (spectra_only) { pr->scale = sc; return; }
    fft_batched(fb, fc, (long)nq * npairs, logN - 1, +1, tw, logTW, st, launches, pr);
    dim3 g3(nblk((long)npairs * p.pst, 256), nq);
    pr->begin("build_post", items * p.plen, st);
    k_build_post<<<g3, 256, 0, st>>>(fb, npairs, N, c.P, c.P_q, c.pst, c.plen, p.P, p.P_q, p.pst, p.plen);
    pr->end(st);
    *launches += 1;
    pr->scale = sc;
}

void launch_fft_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                     const uint8_t *hot_c, double2 *fa, double2 *fb, double2 *fc, const double2 *tw, int logTW,
                     cudaStream_t st, long *launches, Prof *pr, const int *zp, int zq0) {
    const int N = p.fftn, npairs = p.npairs;
    if (npairs <= 0) return;
    if (fused_ok(N)) {
        launch_fused_prop(gp, gp_q, gst_p, gpl, c, p, nq, hot_c, tw, logTW, st, pr, zp, zq0);
        ++*launches;
        return;
    }
    int logN = 0;
    while ((1 << logN) < N) ++logN;
    const double items = (double)nq * npairs;
    const double sc = pr->scale;   // the multi-pass path computes every parent
    pr->scale = 1.0;
    dim3 g1(nblk((long)npairs * (N / 2), 256), nq);
    pr->begin("prop_pack", 0.0, st);
    k_prop_pack<<<g1, 256, 0, st>>>(gp, gp_q, gst_p, gpl, npairs, N, hot_c, fb);
    pr->end(st);
    fft_batched(fb, fc, (long)nq * npairs, logN - 1, -1, tw, logTW, st, launches, pr);
    dim3 g2(nblk((long)npairs * (N / 2 + 1), 256), nq);
    pr->begin("prop_mid", items * (N / 2 + 1) * 40.0, st);
    k_prop_mid<<<g2, 256, 0, st>>>(fb, p.spec, npairs, N, fa, tw, logTW, logN);
    pr->end(st);
    fft_batched(fa, fc, (long)nq * npairs, logN, +1, tw, logTW, st, launches, pr);
    dim3 g3(nblk((long)2 * npairs * c.gst, 256), nq);
    pr->begin("prop_post", items * 2 * c.glen, st);
    k_prop_post<<<g3, 256, 0, st>>>(fa, npairs, N, c.g, c.g_q, c.gst, c.glen, hot_c);
    pr->end(st);
    *launches += 3;
    pr->scale = sc;
}

}  // namespace icmg
