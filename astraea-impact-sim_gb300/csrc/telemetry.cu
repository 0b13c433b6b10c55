// telemetry.cu -- the O(N) loops of the engine's per-frame telemetry on the GPU.
//
// Replaces the host loops of Simulation::Impl::computeTelemetryFromDevice
// (engine/simulation.cpp:948-1285) and sumDeviceRadPowerW (:567-582), which
// copy 17 particle arrays to the host and walk them seven times.  Here every
// loop is a device pass in FP64 (the engine's arithmetic), and the scalar
// state between passes (COMs, the remnant estimate) stays on the device:
//
//   pass A   totals: mass, COMs and mean velocities per body (body 0 vs the
//            rest), kinetic / potential / internal energy, momentum, angular
//            momentum, max T, max P, max damage, radiated power, and the
//            particle of lowest potential (the remnant seed)      :982-1047, 1183
//   pass B   living-body spin sums (lSpinY, I_yy)                  :1092-1111
//            + remnant iteration 0                                 :1131-1174
//   pass C   remnant iterations 1..4 (skipped once one finds nothing bound)
//   pass D   bound-planet / disk / ejecta / bound-impactor masses  :1176-1230
//
// Determinism: each pass is a grid-stride loop over a fixed grid, a block
// reduction in a fixed order, per-block partials in global memory, and a
// final sum over the blocks in block order by the last block to finish (an
// atomic ticket; nothing waits).  Results are identical run to run; against
// the engine's serial loops they differ only by FP64 summation order.
//
// Scratch (partials, pass state, result) is file-scope device memory: the
// call allocates nothing, and calls must not overlap on the GPU.
#include <math_constants.h>

#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kTelThreads = 256;
constexpr int kTelMaxBlocks = 512;
constexpr int kTelSlots = 32;
constexpr double kGPsu = 6.67430e-11 * 1.0e24 * 1.0e3 * 1.0e3 / (1.0e6 * 1.0e6 * 1.0e6);   // engine/units.hpp:27

// Pass A slot layout.
enum SlotA {
    kMass = 0, kSysX, kSysY, kSysZ,
    kM0, kX0, kY0, kZ0, kVx0, kVy0, kVz0,
    kM1, kX1, kY1, kZ1, kVx1, kVy1, kVz1,
    kKe, kPe, kIe, kPx, kPy, kPz, kLx, kLy, kLz, kRad,
    kSlotsA
};
// Remnant-pass slot layout (passes B and C); B adds two spin slots at the end.
enum SlotR { kRM = 0, kRX, kRY, kRZ, kRVx, kRVy, kRVz, kRMR2, kSpinL, kSpinI, kSlotsB };
enum SlotD { kBound = 0, kDisk, kEjecta, kImpBound, kSlotsD };

struct TelState {
    uint32_t ticket;            // last-block detection, reset by the last block
    uint32_t stop;              // a remnant iteration found nothing bound
    double remX, remY, remZ, remVx, remVy, remVz, remMass, remRadius;
    double x0, y0, z0, vx0, vy0, vz0;   // body-0 COM and mean velocity
};

__device__ double g_partials[kTelMaxBlocks * kTelSlots];
__device__ double g_maxA[kTelMaxBlocks * 3];        // max T, max P [GPa], max damage per block
__device__ double g_minPhi[kTelMaxBlocks];
__device__ uint32_t g_minIdx[kTelMaxBlocks];
__device__ TelState g_state;
__device__ AstraeaTelemetry g_out;

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums `cnt` per-thread values over the block (fixed order) and stores them
// as this block's partials.
template <int kCnt>
__device__ __forceinline__ void blockPartials(const double (&v)[kCnt]) {
    __shared__ double red[kTelThreads / 32][kTelSlots];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kCnt; ++k) {
        const double s = warpSum(v[k]);
        if (lane == 0) red[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < kCnt) {
        double s = 0.0;
        for (int w = 0; w < kTelThreads / 32; ++w) s += red[w][threadIdx.x];
        g_partials[blockIdx.x * kTelSlots + threadIdx.x] = s;
    }
}

// True in every thread of the block that finished last (after its partials
// are visible); that block then resets the ticket.
__device__ __forceinline__ bool lastBlock() {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&g_state.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) {
        __threadfence();
        if (threadIdx.x == 0) g_state.ticket = 0u;
    }
    return last;
}

__device__ __forceinline__ double sumPartials(int slot) {
    double s = 0.0;
    for (int b = 0; b < static_cast<int>(gridDim.x); ++b) s += __ldcg(&g_partials[b * kTelSlots + slot]);
    return s;
}

__global__ void __launch_bounds__(kTelThreads) passA(AstraeaParticles p, uint32_t n, double targetRadius) {
    double v[kSlotsA];
#pragma unroll
    for (int k = 0; k < kSlotsA; ++k) v[k] = 0.0;
    double maxT = 0.0, maxP = 0.0, maxD = 0.0, minPhi = CUDART_INF;
    uint32_t minIdx = 0u;
    bool found = false;
    for (uint32_t i = blockIdx.x * kTelThreads + threadIdx.x; i < n; i += gridDim.x * kTelThreads) {
        const double m = p.mass[i];
        const double x = p.posX[i], y = p.posY[i], z = p.posZ[i];
        const double vx = p.velX[i], vy = p.velY[i], vz = p.velZ[i];
        const double phi = p.phiGrav[i];
        const double uVal = p.u[i];
        const double temp = p.tempK[i];
        const double presGPa = static_cast<double>(p.pressure[i]) * 1000.0;
        v[kMass] += m;
        v[kSysX] += m * x; v[kSysY] += m * y; v[kSysZ] += m * z;
        if (p.bodyId[i] == 0u) {
            v[kM0] += m;
            v[kX0] += m * x; v[kY0] += m * y; v[kZ0] += m * z;
            v[kVx0] += m * vx; v[kVy0] += m * vy; v[kVz0] += m * vz;
        } else {
            v[kM1] += m;
            v[kX1] += m * x; v[kY1] += m * y; v[kZ1] += m * z;
            v[kVx1] += m * vx; v[kVy1] += m * vy; v[kVz1] += m * vz;
        }
        v[kKe] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        v[kPe] += 0.5 * m * phi;
        v[kIe] += m * uVal;
        v[kPx] += m * vx; v[kPy] += m * vy; v[kPz] += m * vz;
        v[kLx] += m * (y * vz - z * vy);
        v[kLy] += m * (z * vx - x * vz);
        v[kLz] += m * (x * vy - y * vx);
        const double w = p.radPowerW[i];
        if (isfinite(w) && w > 0.0) v[kRad] += w;
        if (isfinite(temp)) maxT = fmax(maxT, temp);
        if (isfinite(presGPa)) maxP = fmax(maxP, presGPa);
        maxD = fmax(maxD, static_cast<double>(p.damage[i]));
        if (isfinite(phi) && (!found || phi < minPhi)) { minPhi = phi; minIdx = i; found = true; }
    }
    blockPartials<kSlotsA>(v);
    // maxima and the first index of the lowest potential, by warp then block
    __shared__ double smax[3][kTelThreads / 32];
    __shared__ double sphi[kTelThreads / 32];
    __shared__ uint32_t sidx[kTelThreads / 32];
    if (!found) minIdx = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        maxT = fmax(maxT, __shfl_xor_sync(0xffffffffu, maxT, o));
        maxP = fmax(maxP, __shfl_xor_sync(0xffffffffu, maxP, o));
        maxD = fmax(maxD, __shfl_xor_sync(0xffffffffu, maxD, o));
        const double oPhi = __shfl_xor_sync(0xffffffffu, minPhi, o);
        const uint32_t oIdx = __shfl_xor_sync(0xffffffffu, minIdx, o);
        if (oIdx != 0xffffffffu && (minIdx == 0xffffffffu || oPhi < minPhi || (oPhi == minPhi && oIdx < minIdx))) {
            minPhi = oPhi;
            minIdx = oIdx;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { smax[0][warp] = maxT; smax[1][warp] = maxP; smax[2][warp] = maxD; sphi[warp] = minPhi; sidx[warp] = minIdx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, bP = 0.0, d = 0.0, ph = CUDART_INF;
        uint32_t ix = 0xffffffffu;
        for (int k = 0; k < kTelThreads / 32; ++k) {
            a = fmax(a, smax[0][k]); bP = fmax(bP, smax[1][k]); d = fmax(d, smax[2][k]);
            if (sidx[k] != 0xffffffffu && (ix == 0xffffffffu || sphi[k] < ph || (sphi[k] == ph && sidx[k] < ix))) {
                ph = sphi[k];
                ix = sidx[k];
            }
        }
        g_maxA[3 * blockIdx.x + 0] = a; g_maxA[3 * blockIdx.x + 1] = bP; g_maxA[3 * blockIdx.x + 2] = d;
        g_minPhi[blockIdx.x] = ph;
        g_minIdx[blockIdx.x] = ix;
    }
    if (!lastBlock()) return;
    __shared__ double tot[kSlotsA];
    if (threadIdx.x < kSlotsA) tot[threadIdx.x] = sumPartials(threadIdx.x);
    __syncthreads();
    if (threadIdx.x != 0) return;
    AstraeaTelemetry& o = g_out;
    TelState& s = g_state;
    double a = 0.0, bP = 0.0, d = 0.0, ph = CUDART_INF;
    uint32_t seed = 0xffffffffu;
    for (int k = 0; k < static_cast<int>(gridDim.x); ++k) {
        a = fmax(a, __ldcg(&g_maxA[3 * k])); bP = fmax(bP, __ldcg(&g_maxA[3 * k + 1]));
        d = fmax(d, __ldcg(&g_maxA[3 * k + 2]));
        const uint32_t ix = __ldcg(&g_minIdx[k]);
        const double pk = __ldcg(&g_minPhi[k]);
        if (ix != 0xffffffffu && (seed == 0xffffffffu || pk < ph || (pk == ph && ix < seed))) { ph = pk; seed = ix; }
    }
    if (seed == 0xffffffffu) seed = 0u;                          // :999 (no finite potential)
    o.totalMassPsu = tot[kMass];
    o.kineticPsu = tot[kKe]; o.potentialPsu = tot[kPe]; o.internalPsu = tot[kIe];
    o.momentumPsu[0] = tot[kPx]; o.momentumPsu[1] = tot[kPy]; o.momentumPsu[2] = tot[kPz];
    o.angularMomentumPsu[0] = tot[kLx]; o.angularMomentumPsu[1] = tot[kLy]; o.angularMomentumPsu[2] = tot[kLz];
    o.maxTempK = a; o.maxPressureGPa = bP; o.maxDamage = d;
    o.radiatedPowerW = tot[kRad];
    o.remnantSeedIndex = seed;
    if (tot[kMass] > 0.0) {                                      // :1049-1056
        o.sysComPsu[0] = tot[kSysX] / tot[kMass];
        o.sysComPsu[1] = tot[kSysY] / tot[kMass];
        o.sysComPsu[2] = tot[kSysZ] / tot[kMass];
    } else {
        o.sysComPsu[0] = o.sysComPsu[1] = o.sysComPsu[2] = 0.0;
    }
    const double m0 = tot[kM0], m1 = tot[kM1];
    o.massBody0Psu = m0;
    o.massOtherPsu = m1;
    double c0[6], c1[6];
    for (int k = 0; k < 6; ++k) {
        c0[k] = tot[kX0 + k];
        c1[k] = tot[kX1 + k];
    }
    if (m0 > 0.0)                                                // :1058-1069
        for (int k = 0; k < 6; ++k) c0[k] /= m0;
    if (m1 > 0.0)                                                // :1071-1074
        for (int k = 0; k < 6; ++k) c1[k] /= m1;
    for (int k = 0; k < 3; ++k) {
        o.comBody0Psu[k] = c0[k]; o.velBody0Psu[k] = c0[3 + k];
        o.comOtherPsu[k] = c1[k]; o.velOtherPsu[k] = c1[3 + k];
        o.livingComPsu[k] = m0 > 0.0 ? c0[k] : o.sysComPsu[k];
    }
    s.x0 = c0[0]; s.y0 = c0[1]; s.z0 = c0[2]; s.vx0 = c0[3]; s.vy0 = c0[4]; s.vz0 = c0[5];
    // remnant seed, :1121-1128
    s.remX = p.posX[seed]; s.remY = p.posY[seed]; s.remZ = p.posZ[seed];
    s.remVx = p.velX[seed]; s.remVy = p.velY[seed]; s.remVz = p.velZ[seed];
    s.remMass = fmax(m0, tot[kMass] * 0.5);
    s.remRadius = fmax(targetRadius, 0.25);
    s.stop = 0u;
    o.spinLPsu = 0.0;
    o.spinIPsu = 0.0;
    o.remnantIterations = 0;
}

// Remnant iteration (:1131-1174), plus the living-body spin sums in pass B.
template <bool kWithSpin>
__global__ void __launch_bounds__(kTelThreads) passRemnant(AstraeaParticles p, uint32_t n, double targetRadius,
                                                           int living) {
    const TelState s = g_state;                                  // written by the previous launch
    if (s.stop) return;
    constexpr int kCnt = kWithSpin ? kSlotsB : kRMR2 + 1;
    double v[kCnt];
#pragma unroll
    for (int k = 0; k < kCnt; ++k) v[k] = 0.0;
    const double rSoft = fmax(0.5 * s.remRadius, 0.1);
    const double rLimSq = (1.5 * targetRadius) * (1.5 * targetRadius);
    for (uint32_t i = blockIdx.x * kTelThreads + threadIdx.x; i < n; i += gridDim.x * kTelThreads) {
        const double x = p.posX[i], y = p.posY[i], z = p.posZ[i];
        const double vx = p.velX[i], vy = p.velY[i], vz = p.velZ[i];
        const double m = p.mass[i];
        const double dx = x - s.remX, dy = y - s.remY, dz = z - s.remZ;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double r = sqrt(r2);
        const double dvx = vx - s.remVx, dvy = vy - s.remVy, dvz = vz - s.remVz;
        const double v2 = dvx * dvx + dvy * dvy + dvz * dvz;
        const double phiRem = -kGPsu * s.remMass / fmax(r, rSoft);
        const double eSpec = 0.5 * v2 + phiRem;
        if (eSpec < 0.0) {
            v[kRM] += m;
            v[kRX] += m * x; v[kRY] += m * y; v[kRZ] += m * z;
            v[kRVx] += m * vx; v[kRVy] += m * vy; v[kRVz] += m * vz;
            v[kRMR2] += m * r2;
        }
        if constexpr (kWithSpin) {
            if (living && p.bodyId[i] == 0u) {                   // :1097-1111
                const double ex = x - s.x0, ey = y - s.y0, ez = z - s.z0;
                if (ex * ex + ey * ey + ez * ez <= rLimSq) {
                    const double evx = vx - s.vx0, evz = vz - s.vz0;
                    v[kSpinL] += m * (ez * evx - ex * evz);
                    v[kSpinI] += m * (ex * ex + ez * ez);
                }
            }
        }
    }
    blockPartials<kCnt>(v);
    if (!lastBlock()) return;
    __shared__ double tot[kCnt];
    if (threadIdx.x < kCnt) tot[threadIdx.x] = sumPartials(threadIdx.x);
    __syncthreads();
    if (threadIdx.x != 0) return;
    if constexpr (kWithSpin) {
        g_out.spinLPsu = tot[kSpinL];
        g_out.spinIPsu = tot[kSpinI];
    }
    const double nm = tot[kRM];
    if (nm > 0.0) {                                              // :1162-1173
        TelState& w = g_state;
        w.remMass = nm;
        w.remX = tot[kRX] / nm; w.remY = tot[kRY] / nm; w.remZ = tot[kRZ] / nm;
        w.remVx = tot[kRVx] / nm; w.remVy = tot[kRVy] / nm; w.remVz = tot[kRVz] / nm;
        const double rmsR = sqrt(tot[kRMR2] / nm);
        w.remRadius = fmax(0.5 * targetRadius, sqrt(5.0 / 3.0) * rmsR);
        g_out.remnantIterations += 1;
    } else {
        g_state.stop = 1u;
    }
}

// Final classification (:1176-1230).
__global__ void __launch_bounds__(kTelThreads) passClassify(AstraeaParticles p, uint32_t n) {
    const TelState s = g_state;
    double v[kSlotsD] = {0.0, 0.0, 0.0, 0.0};
    const double rSoft = fmax(0.5 * s.remRadius, 0.1);
    const double mu = kGPsu * s.remMass;
    for (uint32_t i = blockIdx.x * kTelThreads + threadIdx.x; i < n; i += gridDim.x * kTelThreads) {
        const double m = p.mass[i];
        const double dx = static_cast<double>(p.posX[i]) - s.remX;
        const double dy = static_cast<double>(p.posY[i]) - s.remY;
        const double dz = static_cast<double>(p.posZ[i]) - s.remZ;
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double dvx = static_cast<double>(p.velX[i]) - s.remVx;
        const double dvy = static_cast<double>(p.velY[i]) - s.remVy;
        const double dvz = static_cast<double>(p.velZ[i]) - s.remVz;
        const double v2 = dvx * dvx + dvy * dvy + dvz * dvz;
        const double eSpec = 0.5 * v2 + (-mu / fmax(r, rSoft));
        if (eSpec >= 0.0) {
            v[kEjecta] += m;
        } else {
            if (p.bodyId[i] != 0u) v[kImpBound] += m;
            bool disk = false;
            if (r > s.remRadius && mu > 0.0) {
                const double jx = dy * dvz - dz * dvy;
                const double jy = dz * dvx - dx * dvz;
                const double jz = dx * dvy - dy * dvx;
                const double j2 = jx * jx + jy * jy + jz * jz;
                const double ecc = sqrt(fmax(0.0, 1.0 + (2.0 * eSpec * j2) / (mu * mu)));
                const double rPeri = j2 / (mu * (1.0 + ecc));
                disk = rPeri > s.remRadius;
            }
            v[disk ? kDisk : kBound] += m;
        }
    }
    blockPartials<kSlotsD>(v);
    if (!lastBlock()) return;
    __shared__ double tot[kSlotsD];
    if (threadIdx.x < kSlotsD) tot[threadIdx.x] = sumPartials(threadIdx.x);
    __syncthreads();
    if (threadIdx.x != 0) return;
    AstraeaTelemetry& o = g_out;
    o.boundPlanetMassPsu = tot[kBound];
    o.diskMassPsu = tot[kDisk];
    o.ejectaMassPsu = tot[kEjecta];
    o.impactorBoundMassPsu = tot[kImpBound];
    o.remnantPsu[0] = s.remX; o.remnantPsu[1] = s.remY; o.remnantPsu[2] = s.remZ;
    o.remnantVelPsu[0] = s.remVx; o.remnantVelPsu[1] = s.remVy; o.remnantVelPsu[2] = s.remVz;
    o.remnantMassPsu = s.remMass;
    o.remnantRadiusPsu = s.remRadius;
}

}  // namespace

cudaError_t launchTelemetry(const AstraeaParticles& p, uint32_t n, double targetRadiusPsu, int livingBodyPresent,
                            int sms, AstraeaTelemetry* hostOut, cudaStream_t st) {
    void* state = nullptr;                     // a ticket left by an aborted call must not survive
    cudaError_t e = cudaGetSymbolAddress(&state, g_state);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(state, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = std::max<uint32_t>(
        1u, std::min<uint32_t>(static_cast<uint32_t>(std::min(2 * sms, kTelMaxBlocks)),
                               (n + kTelThreads - 1) / kTelThreads));
    passA<<<blocks, kTelThreads, 0, st>>>(p, n, targetRadiusPsu);
    passRemnant<true><<<blocks, kTelThreads, 0, st>>>(p, n, targetRadiusPsu, livingBodyPresent);
    for (int it = 1; it < 5; ++it) passRemnant<false><<<blocks, kTelThreads, 0, st>>>(p, n, targetRadiusPsu, 0);
    passClassify<<<blocks, kTelThreads, 0, st>>>(p, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyFromSymbolAsync(hostOut, g_out, sizeof(AstraeaTelemetry), 0, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace astraea_gb300
