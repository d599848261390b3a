// Measurement helpers for the benchmark: kernel-launch counting and the
// FP64 / FP32 FMA and FP64 tensor-core (DMMA) throughput of the device (the
// denominators of the compute rooflines, and the figures that decide whether
// a tile product belongs on the FP64 tensor cores; the HBM denominator is a
// measured copy bandwidth).
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

// FP64 tensor-core throughput: eight independent accumulator chains per warp
// of mma.sync m8n8k4 (512 flops per warp instruction) or m16n8k16 (4,096).
template <int SHAPE>
__global__ void __launch_bounds__(256) k_dmma_peak(double *out, int iters)
{
    const int lane = threadIdx.x & 31;
    const double a = 1e-3 * (lane + 1), b = 1e-4;
    if (SHAPE == 0) {
        double c[8][2];
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = (double)k;
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                             : "+d"(c[k][0]), "+d"(c[k][1])
                             : "d"(a), "d"(b));
        }
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
        if (s == -1.2345) out[blockIdx.x] = s;
    } else {
        double c[8][4];
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = c[k][2] = c[k][3] = (double)k;
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 "
                             "{%0,%1,%2,%3}, {%4,%4,%4,%4,%4,%4,%4,%4}, {%5,%5,%5,%5}, {%0,%1,%2,%3};"
                             : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
                             : "d"(a), "d"(b));
        }
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1] + c[k][2] + c[k][3];
        if (s == -1.2345) out[blockIdx.x] = s;
    }
}

// DMMA and DFMA side by side: even warps run the m8n8k4 chains above, odd
// warps eight DFMA chains, with eight times the iterations (the same flops
// per warp).  Whether the two share one FP64 datapath decides if tile
// products could run on both at once.
__global__ void __launch_bounds__(256) k_dmma_dfma_peak(double *out, int iters)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    if (((threadIdx.x >> 5) & 1) == 0) {
        const double a = 1e-3 * (lane + 1), b = 1e-4;
        double c[8][2];
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = (double)k;
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                             : "+d"(c[k][0]), "+d"(c[k][1])
                             : "d"(a), "d"(b));
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
    } else {
        double a0 = (double)threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
        double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
        const double m = 0.999999, c = 1e-7;
        for (int i = 0; i < 8 * iters; ++i) {
            a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
            a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
        }
        s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    }
    if (s == -1.2345) out[blockIdx.x] = s;
}

static int dmma_dfma_peak(double *tflops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4, threads = 256, iters = 1 << 10;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess) return PSBA_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_dmma_dfma_peak<<<blocks, threads>>>(out, iters / 8);  // warm up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a);
        k_dmma_dfma_peak<<<blocks, threads>>>(out, iters);
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
    // per warp: 8 chains x iters x 512 flops (DMMA) or x 8 iters x 32 lanes x 2 (DFMA): equal
    const double flops = 2.0 * 8 * 8 * 4 * 8.0 * (double)iters * blocks * (threads / 32);
    *tflops = flops / (best * 1e-3) / 1e12;
    return PSBA_OK;
}

template <int SHAPE>
static int dmma_peak(double *tflops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4, threads = 256;
    const int iters = SHAPE == 0 ? 1 << 10 : 1 << 7;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess) return PSBA_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_dmma_peak<SHAPE><<<blocks, threads>>>(out, iters / 8);  // warm up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a);
        k_dmma_peak<SHAPE><<<blocks, threads>>>(out, iters);
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
    const double per_mma = SHAPE == 0 ? 2.0 * 8 * 8 * 4 : 2.0 * 16 * 8 * 16;
    const double flops = per_mma * 8.0 * (double)iters * blocks * (threads / 32);
    *tflops = flops / (best * 1e-3) / 1e12;
    return PSBA_OK;
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
    if (which == 2) return psba::dmma_peak<0>(tflops);
    if (which == 3) return psba::dmma_peak<1>(tflops);
    if (which == 4) return psba::dmma_dfma_peak(tflops);
    return psba::set_error("which must be 0 (FP64 FMA), 1 (FP32 FMA), 2 (FP64 mma m8n8k4), 3 (FP64 mma m16n8k16) "
                           "or 4 (m8n8k4 and FP64 FMA side by side)"),
           PSBA_ERR_ARG;
}

}  // extern "C"
