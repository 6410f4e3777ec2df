// FP32 / FP64 FMA throughput microbenchmark.
//
// The geodesic kernels are bound by the FP32 and FP64 arithmetic pipes, not by memory,
// so their roofline denominators are the chip's measured FMA rates. Each thread runs
// ILP independent FMA chains; the grid fills every SM several times over. The result is
// reported in TFLOP/s with one FMA counted as two floating-point operations.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/foort_gpu.h"

namespace {

template <typename T, int ILP>
__global__ void __launch_bounds__(256) fma_chains(T* sink, int iters, T seed) {
    T a[ILP];
#pragma unroll
    for (int k = 0; k < ILP; ++k) a[k] = seed + static_cast<T>(k) * static_cast<T>(threadIdx.x & 7);
    const T b = static_cast<T>(0.9999995);
    const T c = static_cast<T>(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < ILP; ++k) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < ILP; ++k) s += a[k];
    if (s == static_cast<T>(-1.2345)) sink[blockIdx.x] = s;  // never true; keeps the chains live
}

template <typename T, int ILP>
double measure(int iters, int blocks_per_sm) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * blocks_per_sm, threads = 256;
    T* sink = nullptr;
    if (cudaMalloc(&sink, blocks * sizeof(T)) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T, ILP><<<blocks, threads>>>(sink, iters / 8, static_cast<T>(1));  // warm-up
    double best = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        fma_chains<T, ILP><<<blocks, threads>>>(sink, iters, static_cast<T>(1));
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        double flops = 2.0 * ILP * static_cast<double>(iters) * blocks * threads;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return cudaGetLastError() == cudaSuccess ? best : -1.0;
}

}  // namespace

extern "C" {

// Measured FMA throughput of this GPU in TFLOP/s (FMA = 2 flops). Returns FOORT_OK or
// FOORT_E_CUDA.
int foort_measure_peaks(double* fp32_tflops, double* fp64_tflops) {
    double f32 = measure<float, 8>(1 << 16, 8);
    double f64 = measure<double, 4>(1 << 11, 4);
    if (fp32_tflops) *fp32_tflops = f32;
    if (fp64_tflops) *fp64_tflops = f64;
    return (f32 > 0 && f64 > 0) ? FOORT_OK : FOORT_E_CUDA;
}

}  // extern "C"
