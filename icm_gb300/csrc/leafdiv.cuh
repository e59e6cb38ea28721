// leafdiv.cuh -- per-block leaf products and the per-player division, shared
// by the level-by-level kernels (kernels.cu) and the fused bottom-subtree
// kernels (subtree.cu).
#pragma once

#include <cuda_runtime.h>

#include "exp2_table.cuh"

namespace icmg {

// exp(x) for -700 <= x <= 0 (the leaf factor's domain) by Tang's
// table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989) with a 128-entry table: x = (128 m + j) ln2/128 + r, |r| <= ln2/256,
// and exp(x) = 2^m 2^(j/128) (1 + p(r)), p the degree-5 Taylor polynomial of
// e^r - 1 (its truncation is below 6e-19 relative at |r| <= ln2/256).
// 2^(j/128) is a double-double (exp2_table.cuh), ln2/128 a two-part constant
// (the reduction's error is below 1e-18 relative), and the scaling by 2^m
// (m >= -1010, so every result is a normal number) adds m to the exponent
// field.  Error about 0.5 ulp; 11 FP64 instructions.
__device__ __forceinline__ double exp_nonpos(double x) {
    constexpr double kShift = 0x1.8p52;                // 1.5 2^52: rint into the low bits
    constexpr double kInvLn2x128 = 0x1.71547652b82fep+7;
    constexpr double kLn2hi = 0x1.62e42fefa39efp-8;    // ln2/128 = kLn2hi + kLn2lo
    constexpr double kLn2lo = 0x1.abc9e3b39803fp-63;
    const double t = fma(x, kInvLn2x128, kShift);
    const int k = __double2loint(t);                    // rint(x 128/ln2)
    const double kd = t - kShift;
    double r = fma(kd, -kLn2hi, x);
    r = fma(kd, -kLn2lo, r);
    double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    q = fma(q, r, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    const double p = fma(q, r * r, r);
    const int j = k & 127, m = k >> 7;                  // floor division: k < 0
    const double thi = __ldg(&kExp2Tab[j][0]), tlo = __ldg(&kExp2Tab[j][1]);
    const double y = thi + fma(thi, p, tlo);
    return __hiloint2double(__double2hiint(y) + (m << 20), __double2loint(y));
}

// the leaf factor a = exp(S logv), 0 below -700 (reference src/cpu/icm.c:2575-2581)
__device__ __forceinline__ double leaf_factor(double arg) {
    if (arg < -700.0) return 0.0;
    return arg <= 0.0 ? exp_nonpos(arg) : exp(arg);   // arg > 0 only for nodes v > 1 (none)
}

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
        const double a = leaf_factor(S[j] * logv);
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
