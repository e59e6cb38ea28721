// probes.cu -- measured peaks (FP64 pipe, HBM copy) and per-level kernel
// timing used by the calibration entry points.
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/icm_gpu.h"
#include "engine.h"
#include "kernels.h"

namespace icmg {

// Register-resident DFMA chains: 8 independent chains per thread so the
// FP64 pipe, not the dependency latency, sets the rate.
__global__ void k_dfma_peak(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-7, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;   // keeps the chains live
}

int measure_fp64_gflops(double *out, std::string &err) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) { err = "alloc"; return -1; }
    const int threads = 256, blocks = sms * 8, iters = 1 << 14;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dfma_peak<<<blocks, threads>>>(d, 256, 0.999999, 1e-9);   // warm-up
    double best = 0.0;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_dfma_peak<<<blocks, threads>>>(d, iters, 0.999999, 1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
        best = std::max(best, flops / (ms * 1e-3) / 1e9);
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return -1; }
    *out = best;
    return 0;
}

__global__ void k_copy(const double2 *__restrict__ a, double2 *__restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

int measure_hbm_gbps(double *out, std::string &err) {
    const size_t bytes = (size_t)1 << 31;
    void *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, bytes) != cudaSuccess) { err = "alloc"; return -1; }
    if (cudaMalloc(&b, bytes) != cudaSuccess) { cudaFree(a); err = "alloc"; return -1; }
    cudaMemset(a, 1, bytes);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t n4 = bytes / sizeof(double2);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int r = 0; r < 6; ++r) {
        cudaEventRecord(e0);
        k_copy<<<sms * 16, 256>>>((const double2 *)a, (double2 *)b, n4);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r) best = std::max(best, 2.0 * bytes / (ms * 1e-3) / 1e9);
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return -1; }
    *out = best;
    return 0;
}

}  // namespace icmg

using namespace icmg;

// ns per parent of one FFT build level and one FFT propagate level, FFT size
// fft_n (children of degree fft_n/2), `batch` parents.
extern "C" int icm_gpu_measure_fused_pair_ns(int fft_n, int batch, int quick, double *build_ns_out,
                                             double *corr_ns_out) {
    if (!build_ns_out || !corr_ns_out || fft_n < 8 || (fft_n & (fft_n - 1)) || batch < 1) return 0;
    if (g_device < 0 && icm_gpu_init(0) != 1) return 0;
    *build_ns_out = *corr_ns_out = 0.0;
    std::string err;
    Level c, p;
    c.nreal = 2 * batch;
    c.deg = fft_n / 2;
    c.plen = c.pst = fft_n / 2 + 1;
    c.pst = (c.plen + 1) & ~1;
    c.glen = fft_n / 2;
    c.gst = c.glen;
    p.nreal = batch;
    p.npairs = batch;
    p.fft = 1;
    p.fftn = fft_n;
    p.plen = p.pst = fft_n + 1;
    p.pst = (p.plen + 1) & ~1;
    p.glen = p.gst = fft_n;
    c.P_q = (size_t)c.nreal * c.pst;
    c.g_q = (size_t)c.nreal * c.gst;
    p.P_q = (size_t)p.nreal * p.pst;
    p.g_q = (size_t)p.nreal * p.gst;
    p.spec_q = (size_t)2 * batch * (fft_n / 2 + 1);
    const size_t work = (size_t)batch * fft_n;
    std::vector<void *> bufs;
    auto alloc = [&](size_t bytes) {
        void *q = nullptr;
        if (cudaMalloc(&q, bytes) != cudaSuccess) return (void *)nullptr;
        cudaMemset(q, 0, bytes);
        bufs.push_back(q);
        return q;
    };
    c.P = (double *)alloc(c.P_q * 8);
    c.g = (double *)alloc(c.g_q * 8);
    p.P = (double *)alloc(p.P_q * 8);
    p.g = (double *)alloc(p.g_q * 8);
    p.spec = (double2 *)alloc(p.spec_q * 16);
    double2 *fa = (double2 *)alloc(work * 16), *fb = (double2 *)alloc(work * 16), *fc = (double2 *)alloc(work * 16);
    int ok = c.P && c.g && p.P && p.g && p.spec && fa && fb && fc;
    int logN = 0;
    while ((1 << logN) < fft_n) ++logN;
    int logTW = 0;
    const double2 *tw = ok ? twiddles(logN, 0, err, &logTW) : nullptr;
    if (ok && tw) {
        long launches = 0;
        Prof prof;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int reps = quick ? 3 : 10;
        std::vector<double> tb, tp;
        for (int r = 0; r < reps + 1; ++r) {
            cudaEventRecord(e0);
            launch_fft_build(c, p, 1, fa, fb, fc, false, tw, logTW, 0, &launches, &prof);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r) tb.push_back(ms * 1e6 / batch);
            cudaEventRecord(e0);
            launch_fft_prop(p.g, 0, p.gst, p.glen, c, p, 1, nullptr, fa, fb, fc, tw, logTW, 0, &launches, &prof);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            if (r) tp.push_back(ms * 1e6 / batch);
        }
        std::sort(tb.begin(), tb.end());
        std::sort(tp.begin(), tp.end());
        *build_ns_out = tb[tb.size() / 2];
        *corr_ns_out = tp[tp.size() / 2];
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ok = cudaGetLastError() == cudaSuccess;
    } else {
        ok = 0;
    }
    for (void *q : bufs) cudaFree(q);
    return ok ? 1 : 0;
}
