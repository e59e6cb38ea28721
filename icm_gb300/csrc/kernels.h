// kernels.h -- host-side launchers of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace icmg {

struct Level;

// Optional per-launch timing: when `on`, every launcher brackets its kernel
// with CUDA events on the launch stream and records the kernel's algorithmic
// FP64 flop count (the plan aggregates them by name after the run).
struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
    double flops;
};
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<ProfRec> recs;
    cudaEvent_t get() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(const char *name, double flops, cudaStream_t st) {
        if (!on) return;
        ProfRec r{name, get(), get(), flops};
        cudaEventRecord(r.a, st);
        recs.push_back(r);
    }
    void end(cudaStream_t st) {
        if (on) cudaEventRecord(recs.back().b, st);
    }
};

void fft_set_smem_limits();

// one-kernel FFT levels (fused.cu), used when the level's real FFT size fits
bool fused_ok(int N);
void fused_set_smem_limits();
void launch_fused_build(const Level &c, const Level &p, int nq, bool spectra_only, const double2 *tw, int logTW,
                        cudaStream_t st, Prof *pr);
// spectral levels (spectral.cu)
constexpr int kSpecMaxD = 8192;   // largest child degree of a spectral level
void spec_set_smem_limits();
void launch_spec_init(const Level &v, int nq, const double2 *tw, int logTW, cudaStream_t st, Prof *pr);
void launch_spec_build(const Level &c, const Level &p, bool write_coeffs, int nq, const double2 *tw, int logTW,
                       cudaStream_t st, Prof *pr);
void launch_gspec_init(const double *g, size_t g_q, int gst, int glen, int nreal, const Level &v, double2 *G,
                       size_t G_q, int nq, const uint8_t *hot, const double2 *tw, int logTW, cudaStream_t st,
                       Prof *pr);
void launch_spec_prop(const double2 *Gp, size_t Gp_q, const Level &c, const Level &p, bool children_spectral, int nq,
                      const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr);

// spectral levels with transforms beyond one CTA (spectral_big.cu)
void launch_specbig_build(const Level &c, const Level &p, bool write_coeffs, int nq, double2 *buf, double2 *scratch,
                          const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr);
void launch_specbig_prop(const double2 *Gp, size_t Gp_q, const Level &c, int nq, const uint8_t *hot_c, double2 *buf,
                         double2 *scratch, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr);
void launch_gspecbig_init(const double *g, size_t g_q, int gst, int glen, int nreal, int logd, double2 *G, size_t G_q,
                          int nq, const uint8_t *hot, double2 *buf, double2 *scratch, const double2 *tw, int logTW,
                          cudaStream_t st, long *launches, Prof *pr);

void launch_fused_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                       const uint8_t *hot_c, const double2 *tw, int logTW, cudaStream_t st, Prof *pr);
int fft_batched(double2 *data, double2 *scratch, long batch, int logM, int sign, const double2 *tw, int logTW,
                cudaStream_t st, long *launches, Prof *pr);

void launch_leaf(int B, int n, int nblocks, const double *S, const double *node, int q0, int nq, double *a,
                 double *blockP, double *P0, int pst0, int plen0, cudaStream_t st, Prof *pr);
void launch_divide(int B, int n, int k, int nblocks, const double *S, const double *node, int q0, int nq,
                   const double *a, const double *blockP, const double *g0, size_t g0_q, int gst0,
                   const uint8_t *active, double *contrib, cudaStream_t st, Prof *pr);
void launch_school_build(const Level &c, const Level &p, int nq, int j0, cudaStream_t st, Prof *pr);
void launch_school_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, int nq,
                        const uint8_t *hot_c, int c0, cudaStream_t st, Prof *pr);
void launch_accumulate(int n, int nq, const double *contrib, double *acc, int first, cudaStream_t st, Prof *pr);
void launch_scatter(int n, const double *acc, const int *perm, const uint8_t *active, double *out,
                    cudaStream_t st);
void launch_fft_build(const Level &c, const Level &p, int nq, double2 *fa, double2 *fb, double2 *fc,
                      bool spectra_only, const double2 *tw, int logTW, cudaStream_t st, long *launches, Prof *pr);
void launch_fft_prop(const double *gp, size_t gp_q, int gst_p, int gpl, const Level &c, const Level &p, int nq,
                     const uint8_t *hot_c, double2 *fa, double2 *fb, double2 *fc, const double2 *tw, int logTW,
                     cudaStream_t st, long *launches, Prof *pr);

}  // namespace icmg
