// relax.cu -- the single-body relaxation loop of the engine, on the device.
//
// Restates the per-iteration host work of Simulation::Impl::
// relaxLoadedSingleBody (engine/simulation.cpp:585-781): after every
// damped step the engine copies ten particle arrays to the host, removes the
// COM position and velocity (FP64 sums), damps the velocities by 0.85,
// re-anchors u to the cold energy plus c_v T_anchor(originalId), uploads the
// arrays again and zeroes the stresses and damage.  Here those are two
// device passes (an FP64 moment reduction and an apply pass) with nothing
// crossing to the host; the step kernels between them are the library's
// stage calls (capi.cu).  The closing diagnostics (v_rms / v_esc, :753-767)
// and the final re-anchoring (:769-780) are device passes too.
//
// Reductions: fixed grid, fixed-order block sums, per-block partials, a
// last-block finalisation (atomic ticket, no waits), so results do not
// depend on scheduling.  Scratch is file-scope device memory.
#include <math_constants.h>

#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kRelaxThreads = 256;
constexpr int kRelaxMaxBlocks = 512;
constexpr int kRelaxSlots = 8;
constexpr double kGPsuD = 6.67430e-11 * 1.0e24 * 1.0e3 * 1.0e3 / (1.0e6 * 1.0e6 * 1.0e6);   // engine/units.hpp:27

struct RelaxState {
    uint32_t ticket;
    double com[3], vcom[3];
    double vrmsOverVesc;
};
__device__ double g_relPart[kRelaxMaxBlocks * kRelaxSlots];
__device__ double g_relMax[kRelaxMaxBlocks];
__device__ RelaxState g_rel;

__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int kCnt>
__device__ __forceinline__ void blockSums(const double (&v)[kCnt]) {
    __shared__ double red[kRelaxThreads / 32][kRelaxSlots];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kCnt; ++k) {
        const double s = warpSumD(v[k]);
        if (lane == 0) red[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < kCnt) {
        double s = 0.0;
        for (int w = 0; w < kRelaxThreads / 32; ++w) s += red[w][threadIdx.x];
        g_relPart[blockIdx.x * kRelaxSlots + threadIdx.x] = s;
    }
}

__device__ __forceinline__ bool lastBlockRelax() {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&g_rel.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) {
        __threadfence();
        if (threadIdx.x == 0) g_rel.ticket = 0u;
    }
    return last;
}

__device__ __forceinline__ double sumRelax(int slot) {
    double s = 0.0;
    for (int b = 0; b < static_cast<int>(gridDim.x); ++b) s += __ldcg(&g_relPart[b * kRelaxSlots + slot]);
    return s;
}

// COM position and velocity, simulation.cpp:640-660.
__global__ void __launch_bounds__(kRelaxThreads) relaxMomentsKernel(AstraeaParticles p, uint32_t n) {
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * kRelaxThreads + threadIdx.x; i < n; i += gridDim.x * kRelaxThreads) {
        const double m = p.mass[i];
        v[0] += m;
        v[1] += m * static_cast<double>(p.posX[i]);
        v[2] += m * static_cast<double>(p.posY[i]);
        v[3] += m * static_cast<double>(p.posZ[i]);
        v[4] += m * static_cast<double>(p.velX[i]);
        v[5] += m * static_cast<double>(p.velY[i]);
        v[6] += m * static_cast<double>(p.velZ[i]);
    }
    blockSums<7>(v);
    if (!lastBlockRelax()) return;
    if (threadIdx.x != 0) return;
    double t[7];
    for (int k = 0; k < 7; ++k) t[k] = sumRelax(k);
    for (int k = 0; k < 3; ++k) {
        g_rel.com[k] = t[0] > 0.0 ? t[1 + k] / t[0] : t[1 + k];
        g_rel.vcom[k] = t[0] > 0.0 ? t[4 + k] / t[0] : t[4 + k];
    }
}

__device__ __forceinline__ float anchoredU(const AstraeaParticles& p, uint32_t i, const double* anchorT,
                                           uint32_t anchorCount) {
    const uint32_t oid = p.originalId[i];
    const double tAnchor = (anchorT != nullptr && oid < anchorCount) ? anchorT[oid] : 288.0;
    const uint8_t m8 = p.materialId[i];
    const int mat = m8 <= 4u ? static_cast<int>(m8) : 1;
    return static_cast<float>(coldEnergyF64(mat, static_cast<double>(p.rho[i])) + c_matD[mat].cv * tAnchor);
}

__device__ __forceinline__ void zeroStrength(const AstraeaParticles& p, uint32_t i) {
    p.sXX[i] = 0.f; p.sYY[i] = 0.f; p.sZZ[i] = 0.f; p.sXY[i] = 0.f; p.sXZ[i] = 0.f; p.sYZ[i] = 0.f;
    p.damage[i] = 0.f; p.damageCbrt[i] = 0.f;
    p.dSXX[i] = 0.f; p.dSYY[i] = 0.f; p.dSZZ[i] = 0.f; p.dSXY[i] = 0.f; p.dSXZ[i] = 0.f; p.dSYZ[i] = 0.f;
    p.dDamageCbrtDt[i] = 0.f;
}

// Recentre, damp, re-anchor, clear strength (simulation.cpp:662-705).
__global__ void __launch_bounds__(kRelaxThreads) relaxApplyKernel(AstraeaParticles p, uint32_t n,
                                                                  const double* anchorT, uint32_t anchorCount) {
    const uint32_t i = blockIdx.x * kRelaxThreads + threadIdx.x;
    if (i >= n) return;
    const double cx = g_rel.com[0], cy = g_rel.com[1], cz = g_rel.com[2];
    const double vx = g_rel.vcom[0], vy = g_rel.vcom[1], vz = g_rel.vcom[2];
    p.posX[i] = static_cast<float>(static_cast<double>(p.posX[i]) - cx);
    p.posY[i] = static_cast<float>(static_cast<double>(p.posY[i]) - cy);
    p.posZ[i] = static_cast<float>(static_cast<double>(p.posZ[i]) - cz);
    const float nvx = static_cast<float>(0.85 * (static_cast<double>(p.velX[i]) - vx));
    const float nvy = static_cast<float>(0.85 * (static_cast<double>(p.velY[i]) - vy));
    const float nvz = static_cast<float>(0.85 * (static_cast<double>(p.velZ[i]) - vz));
    p.velX[i] = nvx; p.velY[i] = nvy; p.velZ[i] = nvz;
    p.velHalfX[i] = nvx; p.velHalfY[i] = nvy; p.velHalfZ[i] = nvz;
    p.u[i] = anchoredU(p, i, anchorT, anchorCount);
    zeroStrength(p, i);
}

// v_rms / v_esc of the relaxed body (simulation.cpp:747-767).
__global__ void __launch_bounds__(kRelaxThreads) relaxDiagnosticKernel(AstraeaParticles p, uint32_t n,
                                                                       double nominalRadius) {
    double v[2] = {0.0, 0.0};
    double rMax = nominalRadius;
    for (uint32_t i = blockIdx.x * kRelaxThreads + threadIdx.x; i < n; i += gridDim.x * kRelaxThreads) {
        const double m = p.mass[i];
        const double vx = p.velX[i], vy = p.velY[i], vz = p.velZ[i];
        const double rx = p.posX[i], ry = p.posY[i], rz = p.posZ[i];
        v[0] += m;
        v[1] += m * (vx * vx + vy * vy + vz * vz);
        rMax = fmax(rMax, sqrt(rx * rx + ry * ry + rz * rz));
    }
    blockSums<2>(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rMax = fmax(rMax, __shfl_xor_sync(0xffffffffu, rMax, o));
    __shared__ double wmax[kRelaxThreads / 32];
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = rMax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = wmax[0];
        for (int k = 1; k < kRelaxThreads / 32; ++k) r = fmax(r, wmax[k]);
        g_relMax[blockIdx.x] = r;
    }
    if (!lastBlockRelax()) return;
    if (threadIdx.x != 0) return;
    const double mTot = sumRelax(0), sumMv2 = sumRelax(1);
    double r = nominalRadius;
    for (int b = 0; b < static_cast<int>(gridDim.x); ++b) r = fmax(r, __ldcg(&g_relMax[b]));
    const double vRms = mTot > 0.0 ? sqrt(sumMv2 / mTot) : 0.0;
    const double rScale = fmax(r, 1.0e-3);
    const double vEsc = sqrt((2.0 * kGPsuD * mTot) / rScale);
    g_rel.vrmsOverVesc = vEsc > 0.0 ? vRms / vEsc : 0.0;
}

// Final thermal re-anchoring and strength reset (simulation.cpp:769-780).
__global__ void __launch_bounds__(kRelaxThreads) relaxAnchorKernel(AstraeaParticles p, uint32_t n,
                                                                   const double* anchorT, uint32_t anchorCount) {
    const uint32_t i = blockIdx.x * kRelaxThreads + threadIdx.x;
    if (i >= n) return;
    p.u[i] = anchoredU(p, i, anchorT, anchorCount);
    zeroStrength(p, i);
}

uint32_t reduceBlocks(uint32_t n, int sms) {
    return std::max<uint32_t>(1u, std::min<uint32_t>(static_cast<uint32_t>(std::min(2 * sms, kRelaxMaxBlocks)),
                                                     (n + kRelaxThreads - 1) / kRelaxThreads));
}

cudaError_t resetTicket(cudaStream_t st) {
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_rel);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(addr, 0, sizeof(uint32_t), st);
}

}  // namespace

cudaError_t launchRelaxRecentre(const AstraeaParticles& p, uint32_t n, const double* anchorT, uint32_t anchorCount,
                                int sms, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = resetTicket(st);
    if (e != cudaSuccess) return e;
    relaxMomentsKernel<<<reduceBlocks(n, sms), kRelaxThreads, 0, st>>>(p, n);
    relaxApplyKernel<<<(n + kRelaxThreads - 1) / kRelaxThreads, kRelaxThreads, 0, st>>>(p, n, anchorT, anchorCount);
    return cudaGetLastError();
}

cudaError_t launchRelaxDiagnostic(const AstraeaParticles& p, uint32_t n, double nominalRadius, int sms,
                                  double* hostOut, cudaStream_t st) {
    *hostOut = 0.0;
    if (n == 0) return cudaSuccess;
    cudaError_t e = resetTicket(st);
    if (e != cudaSuccess) return e;
    relaxDiagnosticKernel<<<reduceBlocks(n, sms), kRelaxThreads, 0, st>>>(p, n, nominalRadius);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyFromSymbolAsync(hostOut, g_rel, sizeof(double), offsetof(RelaxState, vrmsOverVesc),
                                  cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

cudaError_t launchRelaxAnchor(const AstraeaParticles& p, uint32_t n, const double* anchorT, uint32_t anchorCount,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    relaxAnchorKernel<<<(n + kRelaxThreads - 1) / kRelaxThreads, kRelaxThreads, 0, st>>>(p, n, anchorT, anchorCount);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
