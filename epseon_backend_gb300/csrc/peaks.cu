// peaks.cu -- FP32 / FP64 FMA throughput burst, the denominators of the
// solver's ALU rooflines (the measured peaks cover only HBM and bf16).
#include <cuda_runtime.h>

#include "launch.h"

namespace epscu {

namespace {

template <typename T>
__global__ void fma_burst(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            x0 = fma(x0, a, b);
            x1 = fma(x1, a, b);
            x2 = fma(x2, a, b);
            x3 = fma(x3, a, b);
            x4 = fma(x4, a, b);
            x5 = fma(x5, a, b);
            x6 = fma(x6, a, b);
            x7 = fma(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double burst_tflops(int sm_count, int iters) {
    const int blocks = sm_count * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_burst<T><<<blocks, threads>>>(out, 4, (T)0.999, (T)0.001);
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        fma_burst<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms > 0.f && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double fmas = (double)blocks * threads * iters * 64.0;
    return 2.0 * fmas / (best * 1e-3) / 1e12;
}

}  // namespace

void measure_fma_peaks(int sm_count, double* fp32_tflops, double* fp64_tflops) {
    if (fp32_tflops) *fp32_tflops = burst_tflops<float>(sm_count, 4000);
    if (fp64_tflops) *fp64_tflops = burst_tflops<double>(sm_count, 200);
}

}  // namespace epscu
