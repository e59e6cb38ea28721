// kernels.h -- host-side launchers of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace icmg {

struct Level;

void fft_set_smem_limits();
int fft_batched(double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw, int logTW,
                cudaStream_t st, long *launches);

void launch_leaf(int B, int n, int nblocks, const double *S, const double *node, int q0, int nq, double *a,
                 double *blockP, double *P0, int pst0, int plen0, cudaStream_t st);
void launch_divide(int B, int n, int k, int nblocks, const double *S, const double *node, int q0, int nq,
                   const double *a, const double *blockP, const double *g0, size_t g0_q, int gst0,
                   const uint8_t *active, double *contrib, cudaStream_t st);
void launch_school_build(const Level &c, const Level &p, int nq, int j0, cudaStream_t st);
void launch_school_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, int nq,
                        const uint8_t *hot_c, int c0, cudaStream_t st);
void launch_accumulate(int n, int nq, const double *contrib, double *acc, int first, cudaStream_t st);
void launch_scatter(int n, const double *acc, const int *perm, const uint8_t *active, double *out,
                    cudaStream_t st);
void launch_fft_build(const Level &c, const Level &p, int nq, double2 *fa, double2 *fb, double2 *fc,
                      bool spectra_only, const double2 *tw, int logTW, cudaStream_t st, long *launches);
void launch_fft_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                     const uint8_t *hot_c, double2 *fa, double2 *fb, double2 *fc, const double2 *tw, int logTW,
                     cudaStream_t st, long *launches);

}  // namespace icmg
