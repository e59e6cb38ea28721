// fft.cuh -- FP64 complex FFT building blocks for sm_103a (device side).
//
// Transforms run in shared memory as in-place radix-4 decimation-in-time
// passes over bit-reversed input (two radix-2 stages fused per pass, so the
// output is in natural order), with one radix-2 pass when log2(M) is odd.
// Per fused pass a butterfly costs 3 complex twiddle products and 8 complex
// additions: 28 FP64 instructions for 4 points and 2 stages.  Twiddles come
// from one device table tw[t] = exp(-2 pi i t / 2^logTW).
#pragma once

#include <cuda_runtime.h>

namespace icmg {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
// multiply by -i and +i
__device__ __forceinline__ double2 cmul_mi(double2 a) { return make_double2(a.y, -a.x); }
__device__ __forceinline__ double2 cmul_pi(double2 a) { return make_double2(-a.y, a.x); }

__device__ __forceinline__ unsigned bitrev(unsigned v, int logM) {
    return logM == 0 ? 0u : (__brev(v) >> (32 - logM));
}

// SIGN = -1: forward (e^{-...}); SIGN = +1: backward (e^{+...}), unnormalised.
template <int SIGN>
__device__ __forceinline__ double2 twmul(double2 a, double2 w) {
    return SIGN < 0 ? cmul(a, w) : cmulc(a, w);
}

// `cnt` transforms of size 2^logM stored back to back in x (shared memory),
// each already in bit-reversed order.  All threads of the block take part;
// the caller synchronises before (after filling x) and this function ends
// with a barrier.
template <int SIGN>
__device__ void smem_fft_dit(double2 *x, int logM, int cnt, const double2 *__restrict__ tw, int logTW) {
    const int M = 1 << logM;
    int s = 0;
    for (; s + 1 < logM; s += 2) {
        const int h = 1 << s;
        const int nb = cnt << (logM - 2);
        const int sh = logTW - s - 2;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 2);
            const int r = b & ((M >> 2) - 1);
            const int j = r & (h - 1);
            const int i = item * M + ((r >> s) << (s + 2)) + j;
            double2 a = x[i], bq = x[i + h], c = x[i + 2 * h], d = x[i + 3 * h];
            if (j != 0) {
                const double2 t1 = __ldg(&tw[j << sh]);
                const double2 t2 = __ldg(&tw[(2 * j) << sh]);
                const double2 t3 = __ldg(&tw[(3 * j) << sh]);
                c = twmul<SIGN>(c, t1);
                bq = twmul<SIGN>(bq, t2);
                d = twmul<SIGN>(d, t3);
            }
            const double2 s0 = cadd(a, bq), d0 = csub(a, bq);
            const double2 s1 = cadd(c, d), d1 = csub(c, d);
            x[i] = cadd(s0, s1);
            x[i + 2 * h] = csub(s0, s1);
            if (SIGN < 0) {
                x[i + h] = cadd(d0, cmul_mi(d1));
                x[i + 3 * h] = csub(d0, cmul_mi(d1));
            } else {
                x[i + h] = cadd(d0, cmul_pi(d1));
                x[i + 3 * h] = csub(d0, cmul_pi(d1));
            }
        }
        __syncthreads();
    }
    if (s < logM) {  // one radix-2 stage left, half size h = M/2
        const int h = 1 << s;
        const int nb = cnt << (logM - 1);
        const int sh = logTW - s - 1;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 1);
            const int r = b & ((M >> 1) - 1);
            const int j = r & (h - 1);
            const int i = item * M + ((r >> s) << (s + 1)) + j;
            double2 a = x[i], bq = x[i + h];
            if (j != 0) bq = twmul<SIGN>(bq, __ldg(&tw[j << sh]));
            x[i] = cadd(a, bq);
            x[i + h] = csub(a, bq);
        }
        __syncthreads();
    }
}

// Decimation in frequency: natural-order input, bit-reversed output.  Two
// radix-2 stages (half sizes 2h and h) per pass, largest first; with
// t = w_{4h}^j the fused pass is
//   x0 = (a + c) + (b + d)            x1 = ((a + c) - (b + d)) t^2
//   x2 = ((a - c) -+ i (b - d)) t     x3 = ((a - c) +- i (b - d)) t^3
// (upper signs forward).  A leading radix-2 stage handles odd log2(M).
// Pairing a DIF inverse with a DIT forward transform lets a pointwise step
// between them run in bit-reversed order with no permutation.
template <int SIGN>
__device__ void smem_fft_dif(double2 *x, int logM, int cnt, const double2 *__restrict__ tw, int logTW) {
    const int M = 1 << logM;
    int s = logM;   // stages left
    if (logM & 1) {  // radix-2 stage with half size M/2
        const int h = M >> 1;
        const int nb = cnt << (logM - 1);
        const int sh = logTW - logM;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 1);
            const int j = b & (h - 1);
            const int i = item * M + j;
            const double2 a = x[i], bq = x[i + h];
            x[i] = cadd(a, bq);
            const double2 d = csub(a, bq);
            x[i + h] = (j != 0) ? twmul<SIGN>(d, __ldg(&tw[j << sh])) : d;
        }
        __syncthreads();
        s -= 1;
    }
    for (; s >= 2; s -= 2) {
        const int hs = s - 2;         // log2 of h
        const int h = 1 << hs;        // pass covers half sizes 2h and h; groups of 4h
        const int nb = cnt << (logM - 2);
        const int sh = logTW - hs - 2;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int item = b >> (logM - 2);
            const int r = b & ((M >> 2) - 1);
            const int j = r & (h - 1);
            const int i = item * M + ((r >> hs) << (hs + 2)) + j;
            const double2 a = x[i], bq = x[i + h], c = x[i + 2 * h], d = x[i + 3 * h];
            const double2 s0 = cadd(a, c), d0 = csub(a, c);
            const double2 s1 = cadd(bq, d), d1 = csub(bq, d);
            double2 y1 = csub(s0, s1), y2, y3;
            if (SIGN < 0) { y2 = cadd(d0, cmul_mi(d1)); y3 = csub(d0, cmul_mi(d1)); }
            else { y2 = cadd(d0, cmul_pi(d1)); y3 = csub(d0, cmul_pi(d1)); }
            x[i] = cadd(s0, s1);
            if (j != 0) {
                y1 = twmul<SIGN>(y1, __ldg(&tw[(2 * j) << sh]));
                y2 = twmul<SIGN>(y2, __ldg(&tw[j << sh]));
                y3 = twmul<SIGN>(y3, __ldg(&tw[(3 * j) << sh]));
            }
            x[i + h] = y1;
            x[i + 2 * h] = y2;
            x[i + 3 * h] = y3;
        }
        __syncthreads();
    }
}

}  // namespace icmg
