// diag.cu -- measured FP32 CUDA-core throughput, the denominator of the
// gravity kernel's roofline (the pair interactions are FP32 FMA/MUFU work,
// not tensor-core work).  Every thread runs 8 independent FMA chains so the
// pipes, not dependencies, bound the rate.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

__global__ void __launch_bounds__(256) fmaPeakKernel(float* out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1.0e-7f;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 123.456f) out[blockIdx.x] = s;   // keeps the chains live; never true in practice
}

}  // namespace

cudaError_t measureFp32Tflops(int sms, float* tflops, cudaStream_t st) {
    float* dummy = nullptr;
    cudaError_t e = cudaMalloc(&dummy, 4096 * sizeof(float));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, iters = 2048;
    fmaPeakKernel<<<blocks, 256, 0, st>>>(dummy, 64, 1.0f);   // warm-up
    cudaEventRecord(a, st);
    fmaPeakKernel<<<blocks, 256, 0, st>>>(dummy, iters, 1.0f);
    cudaEventRecord(b, st);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(dummy);
    const double flops = 2.0 * 8.0 * 16.0 * iters * static_cast<double>(blocks) * 256.0;
    *tflops = static_cast<float>(flops / (ms * 1.0e-3) / 1.0e12);
    return e;
}

}  // namespace astraea_gb300
