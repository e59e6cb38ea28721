/*
 * fftw3.h -- FFTW3 API stand-in, test infrastructure only.
 *
 * The reference CPU library (src/cpu/icm.c:14 includes <fftw3.h>) needs FFTW 3,
 * which is not installed in this image and cannot be fetched.  This header
 * declares the subset of FFTW 3's public interface that icm.c calls (plan
 * creation for 1-D r2c/c2r transforms, execution, wisdom, allocation), with
 * FFTW's documented semantics: unnormalised transforms, r2c output of n/2+1
 * complex values, c2r reading the Hermitian half.  The implementation
 * (fftw_shim.c) is this project's own FFT (../offt.c); only the names and
 * argument meanings are FFTW's, so that the reference source compiles
 * unmodified.  It is linked only into oracle/_ref, never into the product.
 */
#ifndef ICM_ORACLE_FFTW3_SHIM_H
#define ICM_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_import_wisdom_from_filename(const char *filename);
int fftw_export_wisdom_to_filename(const char *filename);
void fftw_make_planner_thread_safe(void);

#ifdef __cplusplus
}
#endif
#endif
