// Measurement helpers for the benchmark: kernel-launch counting and the
// FP64 / FP32 FMA throughput of the device (the denominators of the
// compute rooflines; the HBM denominator is a measured copy bandwidth).
#include <atomic>

#include "psba_internal.h"

namespace psba {

static std::atomic<long long> g_launches{0};

void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// Eight independent FMA chains per thread; FLOPs = 2 * 8 * iters * threads.
template <typename R>
__global__ void __launch_bounds__(256) k_fma_peak(R *out, int iters, R m, R c)
{
    R a0 = (R)threadIdx.x * (R)1e-3, a1 = a0 + (R)1, a2 = a0 + (R)2, a3 = a0 + (R)3;
    R a4 = a0 + (R)4, a5 = a0 + (R)5, a6 = a0 + (R)6, a7 = a0 + (R)7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const R s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (R)-1.2345) out[blockIdx.x] = s;  // never true; keeps the chains live
}

template <typename R>
static int peak_one(double *tflops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    const int iters = sizeof(R) == 8 ? 1 << 12 : 1 << 16;
    R *out = nullptr;
    if (cudaMalloc(&out, sizeof(R) * blocks) != cudaSuccess) return PSBA_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fma_peak<R><<<blocks, threads>>>(out, iters / 8, (R)0.999999, (R)1e-7);  // warm up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a);
        k_fma_peak<R><<<blocks, threads>>>(out, iters, (R)0.999999, (R)1e-7);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return set_error(cudaGetErrorString(e)), PSBA_ERR_CUDA;
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return PSBA_OK;
}

}  // namespace psba

extern "C" {

long long psba_kernel_launches(void) { return psba::launch_count(); }

int psba_measure_peak(int which, double *tflops)
{
    if (!tflops) return psba::set_error("null output"), PSBA_ERR_ARG;
    if (which == 0) return psba::peak_one<double>(tflops);
    if (which == 1) return psba::peak_one<float>(tflops);
    return psba::set_error("which must be 0 (FP64) or 1 (FP32)"), PSBA_ERR_ARG;
}

}  // extern "C"
