// subtree.cu -- the bottom of the tree in one kernel per direction.
//
// The lowest tree levels are schoolbook levels (children below the FFT
// crossover degree), a few coefficients per node and many nodes.  Level by
// level they are latency-bound: every product term reloads its operands from
// L2.  Here one CTA owns kSubBlocks consecutive leaf blocks for one quadrature
// node and keeps its part of the bottom Lf levels in shared memory:
//
//   build:     leaf factors and block products (one thread per block, in
//              registers), then levels 1..Lf as truncated schoolbook products
//              from shared memory; every level's coefficients are also written
//              to HBM for the propagate of the levels above and below.
//   propagate: g of level Lf from HBM, then levels Lf..1 as middle products
//              with the siblings' coefficients staged in shared memory, then
//              the per-player division and weight; the g of levels below Lf
//              never goes to HBM (unless the caller asks for it, as the VJP
//              does).
//
// Arithmetic per coefficient is the level-by-level kernels' (same terms, same
// order), so the equities do not change.  Zero-prefix and subset pruning
// apply as in those kernels.
#include "engine.h"
#include "kernels.h"
#include "leafdiv.cuh"

namespace icmg {

constexpr int kSubThreads = kSubBlocks;

// one buffer holds a level's rows for the CTA: level l has 256 >> l nodes of
// stride <= B 2^l + 2 (coefficients rounded up to even), so 256 (B + 2) doubles
static inline size_t sub_buf_doubles(int B) { return (size_t)kSubBlocks * (B + 2); }
size_t sub_build_smem(int B) { return 2 * sub_buf_doubles(B) * sizeof(double); }
size_t sub_prop_smem(int B) { return 3 * sub_buf_doubles(B) * sizeof(double); }

template <int B>
__device__ __forceinline__ void sub_build_t(const SubArgs &A, int bx, int q, int q0) {
    extern __shared__ double sm[];
    const int SB = kSubBlocks * (B + 2);
    double *cur = sm, *nxt = sm + SB;
    const int tid = threadIdx.x;
    const int b0 = bx * kSubBlocks;
    const int b = b0 + tid;
    const int n = A.n;
    const SubLevel &L0 = A.lv[0];
    // leaf blocks
    if (b < A.nblocks) {
        const double logv = A.node[3 * (q0 + q)];
        const int start = b * B;
        const int bs = min(B, n - start);
        double P[B + 1];
        block_product<B>(A.S + start, bs, logv, A.a + (size_t)q * A.aq + start, P);
        double *bp = A.blockP + ((size_t)q * A.nblocks + b) * (B + 1);
        double *leaf = L0.P + q * L0.P_q + (size_t)b * L0.pst;
#pragma unroll
        for (int m = 0; m <= B; ++m) {
            bp[m] = P[m];
            cur[tid * (B + 1) + m] = P[m];
            if (m < L0.pst) leaf[m] = (m < L0.plen) ? P[m] : 0.0;
        }
        for (int m = B + 1; m < L0.pst; ++m) leaf[m] = 0.0;
    }
    __syncthreads();
    // levels 1..Lf: children in `cur` (level 0 with stride B+1), parents to `nxt`
    for (int l = 1; l <= A.Lf; ++l) {
        const SubLevel &P = A.lv[l], &C = A.lv[l - 1];
        const int cs = (l == 1) ? (B + 1) : C.pst;
        const int lc = C.plen, pst = P.pst, lp = P.plen;
        const int npar = kSubBlocks >> l;
        const long J0 = (long)b0 >> l;
        const ZeroPrefix zl{A.z.zp, q0, P.deg};
        // outputs t and lp-1-t together: their term counts add up to about lc, so
        // the lanes of a warp do equal work (a triangular loop idles half of them)
        const int half = (lp + 1) >> 1;
        for (int e = tid; e < npar * half; e += blockDim.x) {
            const int j = e / half, t = e - j * half;
            const long J = J0 + j;
            if (J >= P.nreal) continue;
            const int t2 = lp - 1 - t;
            double v = 0.0, v2 = 0.0;
            if (zp_cold(zl, q, J)) {
                v = (t == P.deg) ? 1.0 : 0.0;   // x^deg
                v2 = (t2 == P.deg) ? 1.0 : 0.0;
            } else {
                const double *Lc = cur + (size_t)(2 * j) * cs;
                if (2 * J + 1 >= C.nreal) {
                    v = (t < lc) ? Lc[t] : 0.0;   // lone child copied up
                    v2 = (t2 < lc) ? Lc[t2] : 0.0;
                } else {
                    const double *R = Lc + cs;
                    int ilo = max(0, t - (lc - 1)), ihi = min(t, lc - 1);
                    double s0 = 0.0;
                    for (int i = ilo; i <= ihi; ++i) s0 = fma(Lc[i], R[t - i], s0);
                    ilo = max(0, t2 - (lc - 1));
                    ihi = min(t2, lc - 1);
                    double s1 = 0.0;
                    for (int i = ilo; i <= ihi; ++i) s1 = fma(Lc[i], R[t2 - i], s1);
                    v = s0;
                    v2 = s1;
                }
            }
            double *outP = P.P + q * P.P_q + (size_t)J * pst;
            nxt[(size_t)j * pst + t] = v;
            outP[t] = v;
            if (t2 != t) {
                nxt[(size_t)j * pst + t2] = v2;
                outP[t2] = v2;
            }
        }
        for (int e = tid; e < npar * (pst - lp); e += blockDim.x) {   // padding to the row stride
            const int j = e / (pst - lp), t = lp + e % (pst - lp);
            const long J = J0 + j;
            if (J >= P.nreal) continue;
            nxt[(size_t)j * pst + t] = 0.0;
            P.P[q * P.P_q + (size_t)J * pst + t] = 0.0;
        }
        __syncthreads();
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

template <int B>
__device__ __forceinline__ void sub_prop_t(const SubArgs &A, int bx, int q, int q0) {
    extern __shared__ double sm[];
    const int SB = kSubBlocks * (B + 2);
    double *gcur = sm, *gnxt = sm + SB, *pb = sm + 2 * SB;
    const int tid = threadIdx.x;
    const int b0 = bx * kSubBlocks;
    const int n = A.n;
    {   // g of level Lf for this CTA's nodes
        const SubLevel &T = A.lv[A.Lf];
        const int npar = kSubBlocks >> A.Lf;
        const long J0 = (long)b0 >> A.Lf;
        for (int e = tid; e < npar * T.gst; e += blockDim.x) {
            const int j = e / T.gst, m = e - j * T.gst;
            const long J = J0 + j;
            gcur[e] = (J < T.nreal) ? T.g[q * T.g_q + (size_t)J * T.gst + m] : 0.0;
        }
    }
    for (int l = A.Lf; l >= 1; --l) {
        const SubLevel &P = A.lv[l], &C = A.lv[l - 1];
        const int nc = kSubBlocks >> (l - 1);
        const long Jc0 = (long)b0 >> (l - 1);
        // the children's coefficients (siblings of one another)
        for (int e = tid; e < nc * C.pst; e += blockDim.x) {
            const int c = e / C.pst, i = e - c * C.pst;
            const long Jc = Jc0 + c;
            pb[e] = (Jc < C.nreal) ? C.P[q * C.P_q + (size_t)Jc * C.pst + i] : 0.0;
        }
        __syncthreads();
        const ZeroPrefix zc{A.z.zp, q0, C.deg};
        const int gpl = P.glen;
        for (int e = tid; e < nc * C.gst; e += blockDim.x) {
            const int c = e / C.gst, m = e - c * C.gst;
            const long Jc = Jc0 + c;
            if (Jc >= C.nreal || zp_cold(zc, q, Jc)) continue;   // wholly zero: never read
            double v = 0.0;
            if (!(C.hot && !C.hot[Jc]) && m < C.glen) {
                const double *gp = gcur + (size_t)(c >> 1) * P.gst;
                if ((Jc ^ 1) >= C.nreal) {
                    v = (m < gpl) ? gp[m] : 0.0;                     // lone child: the parent's g
                } else {
                    const double *Ps = pb + (size_t)(c ^ 1) * C.pst;
                    const int imax = min(C.plen, gpl - m);
                    double s = 0.0;
                    for (int i = 0; i < imax; ++i) s = fma(Ps[i], gp[m + i], s);
                    v = s;
                }
            }
            gnxt[(size_t)c * C.gst + m] = v;
            if (A.write_g) C.g[q * C.g_q + (size_t)Jc * C.gst + m] = v;
        }
        __syncthreads();
        double *tmp = gcur;
        gcur = gnxt;
        gnxt = tmp;
    }
    if (!A.do_divide) return;
    // per player: division, dot with its block's g (level 0, in gcur), weight
    const double *nd = A.node + 3 * (q0 + q);
    const int gst0 = A.lv[0].gst;
    for (int e = tid; e < kSubBlocks * B; e += blockDim.x) {
        const long i = (long)b0 * B + e;
        if (i >= n) break;
        double *out = A.contrib + (size_t)q * A.aq + i;
        if (A.active && !A.active[i]) { *out = 0.0; continue; }
        if (nd[1] == 0.0) { *out = 0.0; continue; }   // zero-weight node (the reference skips it)
        const double a = A.a[(size_t)q * A.aq + i];
        if (a == 0.0) { *out = 0.0; continue; }
        const long bb = i / B;
        const int start = (int)(bb * B);
        const int bs = min(B, n - start);
        const int pk = min(bs, A.k);
        const double *Pb = A.blockP + ((size_t)q * A.nblocks + bb) * (B + 1);
        const double eq = divide_dot<B>(a, Pb, bs, pk, gcur + (size_t)(bb - b0) * gst0);
        double pw = nd[1] * A.S[i] * a * nd[2];
        if (!isfinite(pw)) pw = 0.0;
        *out = pw * eq;
    }
}

// One kernel per block size (registers sized for that B).  q0: the chunk's
// first node (node table and zero prefixes); work-list argument blocks live
// in global memory and are read in place.
template <int B>
__global__ void __launch_bounds__(kSubThreads) k_sub_build(SubArgs A) {
    sub_build_t<B>(A, blockIdx.x, blockIdx.y, A.z.q0);
}
template <int B>
__global__ void __launch_bounds__(kSubThreads) k_sub_prop(SubArgs A) {
    sub_prop_t<B>(A, blockIdx.x, blockIdx.y, A.z.q0);
}
template <int B>
__global__ void __launch_bounds__(kSubThreads)
kw_sub_build(const SubArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    sub_build_t<B>(D[t.x], t.y, blockIdx.y, q0);
}
template <int B>
__global__ void __launch_bounds__(kSubThreads)
kw_sub_prop(const SubArgs *__restrict__ D, const int2 *__restrict__ tab, int q0) {
    const int2 t = tab[blockIdx.x];
    sub_prop_t<B>(D[t.x], t.y, blockIdx.y, q0);
}

template <int B>
static void sub_limits_b() {
    cudaFuncSetAttribute(k_sub_build<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_build_smem(B));
    cudaFuncSetAttribute(k_sub_prop<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_prop_smem(B));
    cudaFuncSetAttribute(kw_sub_build<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_build_smem(B));
    cudaFuncSetAttribute(kw_sub_prop<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_prop_smem(B));
}

void sub_set_smem_limits() {
    sub_limits_b<4>();
    sub_limits_b<8>();
    sub_limits_b<16>();
    sub_limits_b<32>();
}

SubArgs sub_args(const Plan *p, int Lf, const double *S, const double *node, double *a, size_t aq,
                 const uint8_t *active, double *contrib, bool write_g, bool do_divide, SubFlops *fl) {
    SubArgs A{};
    A.B = p->B;
    A.n = p->n;
    A.k = p->k;
    A.nblocks = p->nblocks;
    A.Lf = Lf;
    A.S = S;
    A.node = node;
    A.a = a;
    A.aq = aq;
    A.blockP = p->d_blockP;
    for (int l = 0; l <= Lf; ++l) {
        const Level &v = p->lv[l];
        SubLevel &s = A.lv[l];
        s.P = v.P;
        s.P_q = v.P_q;
        s.pst = v.pst;
        s.plen = v.plen;
        s.nreal = v.nreal;
        s.g = v.g;
        s.g_q = v.g_q;
        s.gst = v.gst;
        s.glen = v.glen;
        s.hot = p->subset ? p->d_hot + p->hot_off[l] : nullptr;
        s.deg = v.deg;
    }
    A.active = active;
    A.contrib = contrib;
    A.write_g = write_g ? 1 : 0;
    A.do_divide = do_divide ? 1 : 0;
    A.z = ZeroPrefix{p->zskip ? p->d_z : nullptr, 0, 0};
    A.nbx = (p->nblocks + kSubBlocks - 1) / kSubBlocks;
    if (fl) {   // per node: the leaf recurrence, each level's terms, the division
        *fl = SubFlops{};
        const int B = p->B, n = p->n, r = n % B;
        fl->leaf = (double)(n / B) * B * (3.0 * B + 1.0) + (double)r * (3.0 * r + 1.0);
        for (int l = 1; l <= Lf; ++l) {
            const Level &c = p->lv[l - 1], &v = p->lv[l];
            double tb = 0.0, tp = 0.0;
            for (int t = 0; t < v.plen; ++t) tb += std::min(t, c.plen - 1) - std::max(0, t - (c.plen - 1)) + 1;
            for (int m = 0; m < c.glen; ++m) tp += std::max(0, std::min(c.plen, v.glen - m));
            fl->build[l] = 2.0 * tb * std::min(v.nreal, c.nreal / 2);
            fl->prop[l] = 2.0 * tp * 2 * (c.nreal / 2);
        }
        fl->divide = do_divide ? (double)n * (5.0 * std::min(B, p->k) + 4.0) : 0.0;
    }
    return A;
}

void launch_sub_build(const SubArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq) {
    SubArgs a = A;
    a.z.q0 = q0;
    const dim3 g(a.nbx, nq);
    const size_t sm = sub_build_smem(a.B);
    pr->begin("sub_build", fq * nq, st);
    switch (a.B) {
        case 4: k_sub_build<4><<<g, kSubThreads, sm, st>>>(a); break;
        case 8: k_sub_build<8><<<g, kSubThreads, sm, st>>>(a); break;
        case 16: k_sub_build<16><<<g, kSubThreads, sm, st>>>(a); break;
        default: k_sub_build<32><<<g, kSubThreads, sm, st>>>(a); break;
    }
    pr->end(st);
}

void launch_sub_prop(const SubArgs &A, int nq, int q0, cudaStream_t st, Prof *pr, double fq) {
    SubArgs a = A;
    a.z.q0 = q0;
    const dim3 g(a.nbx, nq);
    const size_t sm = sub_prop_smem(a.B);
    pr->begin("sub_prop", fq * nq, st);
    switch (a.B) {
        case 4: k_sub_prop<4><<<g, kSubThreads, sm, st>>>(a); break;
        case 8: k_sub_prop<8><<<g, kSubThreads, sm, st>>>(a); break;
        case 16: k_sub_prop<16><<<g, kSubThreads, sm, st>>>(a); break;
        default: k_sub_prop<32><<<g, kSubThreads, sm, st>>>(a); break;
    }
    pr->end(st);
}

// work lists are keyed by the block size, so one launch has one B
void launch_worklist_sub(WOp op, int B, const void *desc, const int2 *tab, int nctas, int nq, int q0, size_t smem,
                         cudaStream_t st) {
    if (nctas <= 0 || nq <= 0) return;
    const dim3 g(nctas, nq);
    const SubArgs *D = (const SubArgs *)desc;
    if (op == WOp::SubBuild) {
        switch (B) {
            case 4: kw_sub_build<4><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            case 8: kw_sub_build<8><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            case 16: kw_sub_build<16><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            default: kw_sub_build<32><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
        }
    } else {
        switch (B) {
            case 4: kw_sub_prop<4><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            case 8: kw_sub_prop<8><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            case 16: kw_sub_prop<16><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
            default: kw_sub_prop<32><<<g, kSubThreads, smem, st>>>(D, tab, q0); break;
        }
    }
}

}  // namespace icmg
