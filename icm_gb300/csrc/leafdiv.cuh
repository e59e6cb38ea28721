// leafdiv.cuh -- per-block leaf products and the per-player division, shared
// by the level-by-level kernels (kernels.cu) and the fused bottom-subtree
// kernels (subtree.cu).
#pragma once

#include <cuda_runtime.h>

namespace icmg {

// Leaf factors and block product (reference src/cpu/icm.c:2199-2224,
// src/gpu/gpu_kernels.cu:909-936,1030-1091): a_j = exp(S_j logv), 0 when the
// argument is below -700; P = prod_j (a_j + (1 - a_j) x), all B+1
// coefficients updated for every player (exact zeros above the running
// degree), which is the reference's recurrence bit for bit.
template <int B>
__device__ __forceinline__ void block_product(const double *__restrict__ S, int bs, double logv,
                                              double *__restrict__ arow, double (&P)[B + 1]) {
    P[0] = 1.0;
#pragma unroll
    for (int m = 1; m <= B; ++m) P[m] = 0.0;
    // after j players only P[0..j] can be nonzero: updating P[m] for m > j+1
    // would add exact zeros, and P[j+1] = a 0 + (1-a) P[j] = (1-a) P[j]
    // exactly, so the partial update below gives the full recurrence's bits
#pragma unroll
    for (int j = 0; j < B; ++j) {
        if (j >= bs) break;
        const double arg = S[j] * logv;
        const double a = (arg < -700.0) ? 0.0 : exp(arg);
        arow[j] = a;
        const double bb = 1.0 - a;
        P[j + 1] = bb * P[j];
#pragma unroll
        for (int m = j; m >= 1; --m) P[m] = a * P[m] + bb * P[m - 1];
        P[0] *= a;
    }
}

// inner_i = sum_{m < pk} g[m] Q_i[m] with Q_i = P / (a + (1 - a) x) by the
// forward recurrence when a > 0.5, the backward one when a > 1e-15, else a
// shift (reference icm.c:2230-2302).  P holds the full block product.
template <int B>
__device__ __forceinline__ double divide_dot(double a, const double *__restrict__ P, int bs, int pk,
                                             const double *__restrict__ g) {
    const double bb = 1.0 - a;
    double eq = 0.0;
    if (a > 0.5) {
        const double ia = 1.0 / a, c = -bb * ia;
        double Qv = P[0] * ia;
        eq = g[0] * Qv;
        for (int m = 1; m < pk; ++m) {
            Qv = c * Qv + P[m] * ia;
            eq += g[m] * Qv;
        }
    } else if (a > 1e-15) {
        // Q[bs-1] = P[bs] / (1-a), Q[m] = (P[m+1] - a Q[m+1]) / (1-a) downwards;
        // constant indices keep Q in registers
        const double ib = 1.0 / bb, c = -a * ib;
        double Qa[B];
        double Qp = 0.0;
#pragma unroll
        for (int m = B - 1; m >= 0; --m) {
            if (m == bs - 1) Qp = P[bs] * ib;
            else if (m < bs - 1) Qp = c * Qp + P[m + 1] * ib;
            Qa[m] = Qp;
        }
#pragma unroll
        for (int m = 0; m < B; ++m)
            if (m < pk) eq += g[m] * Qa[m];
    } else {
        for (int m = 0; m < pk; ++m) eq += g[m] * P[m + 1];
    }
    return eq;
}

}  // namespace icmg
