// diag.cu -- measured FP32 CUDA-core throughput, the denominator of the
// gravity kernel's roofline (the pair interactions are FP32 FMA/MUFU work,
// not tensor-core work).  Two forms are timed: scalar fmaf chains and packed
// fma.rn.f32x2 chains (two FP32 FMAs per instruction, the form the gravity
// pair evaluation issues); the larger rate is the peak.  Every thread runs 8
// independent chains so the pipes, not dependencies, bound the rate.
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

__global__ void __launch_bounds__(256) fma2PeakKernel(float* out, int iters, float seed) {
    const float b0 = seed + threadIdx.x;
    f2 a0 = pack2(b0, b0 + 0.5f), a1 = pack2(b0 + 1.f, b0 + 1.5f), a2 = pack2(b0 + 2.f, b0 + 2.5f),
       a3 = pack2(b0 + 3.f, b0 + 3.5f), a4 = pack2(b0 + 4.f, b0 + 4.5f), a5 = pack2(b0 + 5.f, b0 + 5.5f),
       a6 = pack2(b0 + 6.f, b0 + 6.5f), a7 = pack2(b0 + 7.f, b0 + 7.5f);
    const f2 m = pack2(0.999999f, 0.999999f), c = pack2(1.0e-7f, 1.0e-7f);
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fma2(a0, m, c); a1 = fma2(a1, m, c); a2 = fma2(a2, m, c); a3 = fma2(a3, m, c);
            a4 = fma2(a4, m, c); a5 = fma2(a5, m, c); a6 = fma2(a6, m, c); a7 = fma2(a7, m, c);
        }
    }
    f2 s2 = add2(add2(add2(a0, a1), add2(a2, a3)), add2(add2(a4, a5), add2(a6, a7)));
    float lo, hi;
    unpack2(s2, lo, hi);
    if (lo + hi == 123.456f) out[blockIdx.x] = lo;   // keeps the chains live; never true in practice
}

template <typename K>
float timeFmaKernel(K kernel, int blocks, int iters, float* dummy, double fmaPerThreadIter, cudaStream_t st,
                    cudaError_t* err) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    kernel<<<blocks, 256, 0, st>>>(dummy, 64, 1.0f);   // warm-up
    cudaEventRecord(a, st);
    kernel<<<blocks, 256, 0, st>>>(dummy, iters, 1.0f);
    cudaEventRecord(b, st);
    *err = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double flops = 2.0 * fmaPerThreadIter * iters * static_cast<double>(blocks) * 256.0;
    return (*err == cudaSuccess && ms > 0.f) ? static_cast<float>(flops / (ms * 1.0e-3) / 1.0e12) : 0.f;
}

}  // namespace

cudaError_t measureFp32Tflops(int sms, float* tflops, cudaStream_t st) {
    float scalar = 0.f, packed = 0.f;
    return measureFp32TflopsBoth(sms, &scalar, &packed, tflops, st);
}

cudaError_t measureFp32TflopsBoth(int sms, float* scalarOut, float* packedOut, float* peakOut, cudaStream_t st) {
    float* dummy = nullptr;
    cudaError_t e = cudaMalloc(&dummy, 4096 * sizeof(float));
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, iters = 2048;
    cudaError_t e1 = cudaSuccess, e2 = cudaSuccess;
    *scalarOut = timeFmaKernel(fmaPeakKernel, blocks, iters, dummy, 8.0 * 16.0, st, &e1);
    *packedOut = timeFmaKernel(fma2PeakKernel, blocks, iters, dummy, 2.0 * 8.0 * 16.0, st, &e2);
    *peakOut = *scalarOut > *packedOut ? *scalarOut : *packedOut;
    cudaFree(dummy);
    return e1 != cudaSuccess ? e1 : e2;
}

}  // namespace astraea_gb300

// ---------------------------------------------------------------------------
// FP64 direct-sum gravity at listed targets: the truth the Barnes-Hut and
// far-field accuracies are measured against (the N^2 check of the engine's
// tests/cpp/test_gravity_sph.cpp:366-378, eps_ij = (eps_i + eps_j) / 2 with
// eps = 0.8 max(h0, 1e-6), G_PSU).  One thread per target; sources staged
// through shared memory in tiles; every operation in FP64.
namespace astraea_gb300 {
namespace {
constexpr int kDirectThreads = 128;
constexpr double kGPsuDirect = 6.67430e-11 * 1.0e24 * 1.0e3 * 1.0e3 / (1.0e6 * 1.0e6 * 1.0e6);
struct Src4 { double x, y, z, w; };   // one staged source: position, mass

__global__ void __launch_bounds__(kDirectThreads) directGravityF64Kernel(AstraeaParticles p, uint32_t n,
                                                                        const uint32_t* targets, uint32_t nt,
                                                                        double* acc3, double* phiOut) {
    __shared__ Src4 src[kDirectThreads];      // x, y, z, m
    __shared__ double srcEps[kDirectThreads];
    const uint32_t t = blockIdx.x * kDirectThreads + threadIdx.x;
    const bool live = t < nt;
    const uint32_t i = live ? targets[t] : 0u;
    const bool valid = live && i < n;
    double xi = 0.0, yi = 0.0, zi = 0.0, ei = 0.0;
    if (valid) {
        xi = p.posX[i]; yi = p.posY[i]; zi = p.posZ[i];
        ei = 0.8 * static_cast<double>(fmaxf(p.h0[i], 1.0e-6f));
    }
    double ax = 0.0, ay = 0.0, az = 0.0, phi = 0.0;
    for (uint32_t base = 0; base < n; base += kDirectThreads) {
        const uint32_t j = base + threadIdx.x;
        __syncthreads();
        if (j < n) {
            src[threadIdx.x] = Src4{p.posX[j], p.posY[j], p.posZ[j], p.mass[j]};
            srcEps[threadIdx.x] = 0.8 * static_cast<double>(fmaxf(p.h0[j], 1.0e-6f));
        } else {
            src[threadIdx.x] = Src4{0.0, 0.0, 0.0, 0.0};
            srcEps[threadIdx.x] = 1.0;
        }
        __syncthreads();
        const int cnt = static_cast<int>(min(static_cast<uint32_t>(kDirectThreads), n - base));
        for (int k = 0; k < cnt; ++k) {
            if (base + static_cast<uint32_t>(k) == i) continue;
            const Src4 s = src[k];
            const double dx = xi - s.x, dy = yi - s.y, dz = zi - s.z;
            const double e = 0.5 * (ei + srcEps[k]);
            const double r2 = dx * dx + dy * dy + dz * dz + e * e;
            const double inv = 1.0 / sqrt(r2);
            const double f = -kGPsuDirect * s.w * inv * inv * inv;
            ax += f * dx; ay += f * dy; az += f * dz;
            phi -= kGPsuDirect * s.w * inv;
        }
    }
    if (live) {
        acc3[3 * static_cast<size_t>(t)] = valid ? ax : 0.0;
        acc3[3 * static_cast<size_t>(t) + 1] = valid ? ay : 0.0;
        acc3[3 * static_cast<size_t>(t) + 2] = valid ? az : 0.0;
        phiOut[t] = valid ? phi : 0.0;
    }
}
}  // namespace

cudaError_t launchDirectGravityF64(const AstraeaParticles& p, uint32_t n, const uint32_t* targets, uint32_t nt,
                                   double* acc3, double* phi, cudaStream_t st) {
    if (nt == 0) return cudaSuccess;
    directGravityF64Kernel<<<(nt + kDirectThreads - 1) / kDirectThreads, kDirectThreads, 0, st>>>(p, n, targets, nt,
                                                                                                  acc3, phi);
    return cudaGetLastError();
}
}  // namespace astraea_gb300
