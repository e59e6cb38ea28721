// tma_cols.cu -- the four-step column pass (fft_batched's pass A) with its
// tile staged by the tensor-memory accelerator.
//
// A CTA transforms cb columns n2 of the M1 x M2 view x[M2 n1 + n2] of one
// item.  The tile (M1 rows of cb consecutive complex values) is one box of a
// three-dimensional tensor map over the batch (doubles: 2 M2 per row, M1
// rows, items), loaded by cp.async.bulk.tensor into shared memory row by row
// as it lies in global memory; the rows are then put in bit-reversed order in
// place and the column transforms run on the tile with a stride of cb, the
// same radix-4 / radix-2 butterflies (tangent-form twiddles) as smem_fft_dit,
// so results are bit for bit those of the plain column pass.
//
// Alignment: the box's inner extent is 2 cb doubles (16 cb bytes) and its
// inner coordinate 2 n20 doubles (16 n20 bytes), multiples of 16 as TMA
// requires; the buffers come from 256-aligned arenas; boxes of at most 256
// rows land at 128-byte aligned shared-memory offsets.  The completion wait
// is bounded: a CTA that does not see its copy complete within the limit
// records the failure in g_tma_fail and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "engine.h"
#include "fft.cuh"
#include "kernels.h"

namespace icmg {

static __device__ int g_tma_fail;   // CTAs whose tile copy did not complete in the wait limit

constexpr int kTmaBoxRows = 256;    // the largest box extent

// item wholly inside its node's zero prefix (nothing reads it): as fft_batched
__device__ __forceinline__ bool tma_skip(const FftSkip &k, long item) {
    if (!k.zp) return false;
    const long it = k.item0 + item;
    const long q = it / k.per_q, j = it - q * k.per_q;
    return (j + 1) * k.span <= (long)k.zp[k.q0 + q];
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// The column transforms of `cnt` items stored with stride `cnt`: element i of
// item c at x[i cnt + c]; bit-reversed input, natural output (smem_fft_dit's
// passes, addressed through the stride, its half shifts included).
template <int SIGN, int SHIFT>
__device__ void smem_fft_dit_strided(double2 *x, int logM, int cnt, const double2 *__restrict__ tw, int logTW) {
    const TwTables T = tw_tables(tw, logTW, tw_set(SHIFT));
    const int M = 1 << logM;
    int s = 0;
    for (; s + 1 < logM; s += 2) {
        const int h = 1 << s;
        const int nb = cnt << (logM - 2);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b % cnt;   // neighbouring threads: neighbouring columns
            const int r = b / cnt;
            const int j = r & (h - 1);
            const int i = ((r >> s) << (s + 2)) + j;
            double2 *xi = x + (size_t)i * cnt + item;
            const size_t hs = (size_t)h * cnt;
            const double2 a = xi[0], bq = xi[hs], c = xi[2 * hs], d = xi[3 * hs];
            double2 x0, x1, x2, x3;
            if (SHIFT == 0 && h == 1) {
                const double2 s0 = cadd(a, bq), d0 = csub(a, bq);
                const double2 s1 = cadd(c, d), d1 = csub(c, d);
                x0 = cadd(s0, s1);
                x2 = csub(s0, s1);
                if (SIGN < 0) { x1 = cadd(d0, cmul_mi(d1)); x3 = csub(d0, cmul_mi(d1)); }
                else { x1 = cadd(d0, cmul_pi(d1)); x3 = csub(d0, cmul_pi(d1)); }
            } else {
                const GTw g = T.r4[h + j];
                const int code = __ldg(&T.r4c[h + j]);
                const double2 uc = tanmul<SIGN>(c, code & 3, g.a.x);
                const double2 ub = tanmul<SIGN>(bq, (code >> 2) & 3, g.b.x);
                const double2 ud = tanmul<SIGN>(d, (code >> 4) & 3, g.c.x);
                const double r1 = g.a.y, r2 = g.b.y, rho = g.c.y;
                const double2 s0 = make_double2(fma(r2, ub.x, a.x), fma(r2, ub.y, a.y));
                const double2 d0 = make_double2(fma(-r2, ub.x, a.x), fma(-r2, ub.y, a.y));
                const double2 e = make_double2(fma(rho, ud.x, uc.x), fma(rho, ud.y, uc.y));
                const double2 f = make_double2(fma(-rho, ud.x, uc.x), fma(-rho, ud.y, uc.y));
                x0 = make_double2(fma(r1, e.x, s0.x), fma(r1, e.y, s0.y));
                x2 = make_double2(fma(-r1, e.x, s0.x), fma(-r1, e.y, s0.y));
                if (SIGN < 0) {
                    x1 = make_double2(fma(r1, f.y, d0.x), fma(-r1, f.x, d0.y));
                    x3 = make_double2(fma(-r1, f.y, d0.x), fma(r1, f.x, d0.y));
                } else {
                    x1 = make_double2(fma(-r1, f.y, d0.x), fma(r1, f.x, d0.y));
                    x3 = make_double2(fma(r1, f.y, d0.x), fma(-r1, f.x, d0.y));
                }
            }
            xi[0] = x0;
            xi[hs] = x1;
            xi[2 * hs] = x2;
            xi[3 * hs] = x3;
        }
        __syncthreads();
    }
    if (s < logM) {   // one radix-2 stage left
        const int h = 1 << s;
        const int nb = cnt << (logM - 1);
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b % cnt;
            const int r = b / cnt;
            const int j = r & (h - 1);
            const int i = ((r >> s) << (s + 1)) + j;
            double2 *xi = x + (size_t)i * cnt + item;
            const size_t hs = (size_t)h * cnt;
            const double2 a = xi[0], bq = xi[hs];
            const double2 g = T.r2[h + j];
            const double2 u = tanmul<SIGN>(bq, __ldg(&T.r2c[h + j]), g.x);
            xi[0] = make_double2(fma(g.y, u.x, a.x), fma(g.y, u.y, a.y));
            xi[hs] = make_double2(fma(-g.y, u.x, a.x), fma(-g.y, u.y, a.y));
        }
        __syncthreads();
    }
    (void)M;
}

template <int SIGN, int SHIFT>
__global__ void __launch_bounds__(256) k_fft4_cols_tma(const __grid_constant__ CUtensorMap tmap,
                                                       double2 *__restrict__ out, int logM1, int logM2, int cb,
                                                       const double2 *__restrict__ tw, int logTW, FftSkip skip,
                                                       long item0) {
    extern __shared__ __align__(128) double2 tile[];
    __shared__ __align__(8) unsigned long long bar;
    const int M1 = 1 << logM1;
    const long item = blockIdx.y;
    if (tma_skip(skip, item)) return;
    const int n20 = blockIdx.x * cb;
    const unsigned bar_a = smem_u32(&bar);
    const int rows = min(M1, kTmaBoxRows);
    const unsigned bytes = (unsigned)(cb * M1 * sizeof(double2));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(bytes) : "memory");
        const int x = 2 * n20, z = (int)(item0 + item);
        for (int r0 = 0; r0 < M1; r0 += rows) {
            const unsigned dst = smem_u32(tile + (size_t)r0 * cb);
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                ::"r"(dst), "l"(&tmap), "r"(x), "r"(r0), "r"(z), "r"(bar_a) : "memory");
        }
    }
    // bounded wait for the copy (phase 0)
    int done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it) {
        unsigned ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(bar_a) : "memory");
        done = (int)ok;
    }
    if (__syncthreads_or(!done)) {
        if (threadIdx.x == 0) atomicAdd(&g_tma_fail, 1);
        return;
    }
    // rows into bit-reversed order, in place
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int c = e % cb, r = e / cb;
        const int rr = (int)bitrev(r, logM1);
        if (rr <= r) continue;
        const double2 va = tile[(size_t)r * cb + c], vb = tile[(size_t)rr * cb + c];
        tile[(size_t)r * cb + c] = vb;
        tile[(size_t)rr * cb + c] = va;
    }
    __syncthreads();
    smem_fft_dit_strided<SIGN, SHIFT>(tile, logM1, cb, tw, logTW);
    const int logM = logM1 + logM2;
    double2 *dst = out + (item << logM);
    for (int e = threadIdx.x; e < cb * M1; e += blockDim.x) {
        const int c = e >> logM1, k1 = e & (M1 - 1);
        const int n2 = n20 + c;
        const long t = fft4_tw_index<SHIFT>(n2, k1, logM, logTW);
        double2 v = tile[(size_t)k1 * cb + c];
        if (t) v = twmul<SIGN>(v, __ldg(&tw[t]));
        dst[(long)n2 * M1 + k1] = v;
    }
}

// ---------------------------------------------------------------- host
namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    });
    return g_encode;
}

void tma_set_smem_limits() {
    const int mx = 4096 * (int)sizeof(double2);
    cudaFuncSetAttribute(k_fft4_cols_tma<-1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols_tma<+1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols_tma<-1, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fft4_cols_tma<-1, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

// The column pass of a four-step transform of `batch` items (batch <= 65535)
// through a tensor map; false (nothing launched) where the map cannot be
// made, so that the caller runs the plain pass.
bool launch_fft4_cols_tma(const double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw,
                          int logTW, int cbA, cudaStream_t st, FftSkip skip, int shift) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || batch > 65535) return false;
    const int logM1 = (logM + 1) / 2, logM2 = logM - logM1;
    const int M1 = 1 << logM1, M2 = 1 << logM2;
    if (2 * cbA > 256 || (M1 > kTmaBoxRows && M1 % kTmaBoxRows)) return false;
    CUtensorMap tmap;
    const cuuint64_t dims[3] = {(cuuint64_t)2 * M2, (cuuint64_t)M1, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)M2 * sizeof(double2), ((cuuint64_t)M1 * M2) * sizeof(double2)};
    const cuuint32_t box[3] = {(cuuint32_t)(2 * cbA), (cuuint32_t)std::min(M1, kTmaBoxRows), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double2 *>(data), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const dim3 g(M2 / cbA, (unsigned)batch);
    const size_t sm = (size_t)cbA * M1 * sizeof(double2);
    if (shift > 0) k_fft4_cols_tma<-1, +1><<<g, 256, sm, st>>>(tmap, scratch, logM1, logM2, cbA, tw, logTW, skip, 0);
    else if (shift < 0) k_fft4_cols_tma<-1, -1><<<g, 256, sm, st>>>(tmap, scratch, logM1, logM2, cbA, tw, logTW, skip, 0);
    else if (sign < 0) k_fft4_cols_tma<-1, 0><<<g, 256, sm, st>>>(tmap, scratch, logM1, logM2, cbA, tw, logTW, skip, 0);
    else k_fft4_cols_tma<+1, 0><<<g, 256, sm, st>>>(tmap, scratch, logM1, logM2, cbA, tw, logTW, skip, 0);
    return true;
}

// CTAs of the TMA column pass that gave up waiting for their tile (read and
// cleared; 0 when none)
int tma_take_failures() {
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_fail, sizeof v) != cudaSuccess) return -1;
    if (v) cudaMemcpyToSymbol(g_tma_fail, &z, sizeof z);
    return v;
}

}  // namespace icmg
