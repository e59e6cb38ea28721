/*
 * offt.h -- small FP64 FFT used by the CPU oracle (test infrastructure only).
 *
 * It backs two things under oracle/:
 *   - fftw_shim.c, an FFTW3-API stand-in so the reference's unmodified
 *     src/cpu/icm.c links here (FFTW 3.x is not installed in this image);
 *   - icm_oracle.c's FFT levels, used when the oracle is timed as the CPU
 *     baseline.
 *
 * Conventions follow FFTW's published definitions: forward transform
 * X[f] = sum_t x[t] e^{-2 pi i f t / n}, backward uses e^{+...}, neither is
 * normalised.  Sizes: any n whose prime factors are 2, 3, 5, 7 (the 7-smooth
 * sizes icm.c asks for); other primes fall back to an O(p^2) butterfly.
 *
 * Nothing in the product library links this file.
 */
#ifndef ICM_ORACLE_OFFT_H
#define ICM_ORACLE_OFFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct offt_plan offt_plan;

/* complex transform of length n; sign = -1 forward, +1 backward */
offt_plan *offt_plan_c2c(int n);
void offt_exec_c2c(const offt_plan *p, const double *in, double *out, int sign,
                   double *scratch);
/* scratch needs 4*n doubles (c2c) */

/* real transforms of length n: r2c writes n/2+1 complex values,
 * c2r reads n/2+1 complex values (Hermitian half) and writes n reals. */
offt_plan *offt_plan_real(int n);
void offt_exec_r2c(const offt_plan *p, const double *in, double *out,
                   double *scratch);
void offt_exec_c2r(const offt_plan *p, const double *in, double *out,
                   double *scratch);
/* scratch needs offt_real_scratch(n) doubles */
int offt_real_scratch(int n);

int offt_size(const offt_plan *p);
void offt_destroy(offt_plan *p);

#ifdef __cplusplus
}
#endif
#endif
