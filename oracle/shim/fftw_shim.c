/*
 * fftw_shim.c -- FFTW3 API stand-in over this project's oracle FFT (offt.c).
 * Test infrastructure only: linked into oracle/_ref/libicm_ref*.so so the
 * reference's unmodified src/cpu/icm.c can run here as a parity oracle.
 *
 * Plans own their scratch; icm.c gives each OpenMP thread its own plans
 * (icm.c:1524-1575 clones the FFT cache per thread), so a plan is never
 * executed by two threads at once.  Wisdom calls are accepted and ignored.
 */
#include "fftw3.h"
#include "../offt.h"

#include <stdlib.h>

struct fftw_plan_s {
    int n;
    int kind;            /* 0 = r2c, 1 = c2r */
    double *in;          /* buffers bound at plan time (fftw_execute) */
    double *out;
    offt_plan *p;
    double *scratch;
};

static fftw_plan make(int n, int kind, double *in, double *out) {
    if (n < 1) return NULL;
    struct fftw_plan_s *pl = (struct fftw_plan_s *)calloc(1, sizeof(*pl));
    pl->n = n;
    pl->kind = kind;
    pl->in = in;
    pl->out = out;
    pl->p = offt_plan_real(n);
    pl->scratch = (double *)malloc(sizeof(double) * (size_t)offt_real_scratch(n));
    return pl;
}

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags) {
    (void)flags;
    return make(n, 0, in, (double *)out);
}

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags) {
    (void)flags;
    return make(n, 1, (double *)in, out);
}

void fftw_execute(const fftw_plan p) {
    if (!p) return;
    if (p->kind == 0) offt_exec_r2c(p->p, p->in, p->out, p->scratch);
    else offt_exec_c2r(p->p, p->in, p->out, p->scratch);
}

void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out) {
    if (p) offt_exec_r2c(p->p, in, (double *)out, p->scratch);
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out) {
    if (p) offt_exec_c2r(p->p, (double *)in, out, p->scratch);
}

void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    offt_destroy(p->p);
    free(p->scratch);
    free(p);
}

void *fftw_malloc(size_t n) {
    void *ptr = NULL;
    if (posix_memalign(&ptr, 64, n ? n : 64) != 0) return NULL;
    return ptr;
}

void fftw_free(void *p) { free(p); }
int fftw_import_wisdom_from_filename(const char *filename) { (void)filename; return 0; }
int fftw_export_wisdom_to_filename(const char *filename) { (void)filename; return 1; }
void fftw_make_planner_thread_safe(void) {}
