// integrate.cu -- EOS, KDK half kick, adaptive dt reduction and stat reset.
//
// Restates evaluateEosKernel (engine/sph_gravity.cu:792-806, EOS of
// engine/eos.cu:320-388 evaluated in FP32 here), leapfrogKickHalfKernel
// (:1291-1374), reduceDtMinKernel + launchReduceDtPsu (:1493-1550,
// 2136-2161) and clearStatsKernel (:624-641).  Fusions used by the step:
//   * the EOS kernel that follows SPH pass 1 also writes the packed pass-2
//     neighbour record of its particle;
//   * the closing half kick evaluates the EOS of its kicked state (the
//     engine's separate EOS launch) and reduces the next step's dt candidate
//     in the same pass over the particles;
//   * the opening half kick resolves dt on the device (the engine clamps it
//     on the host after a blocking copy) and writes the drift's velocity
//     records.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

// Per-particle dt candidate (sph_gravity.cu:1504-1527), each operation an
// explicit IEEE op rounded as the engine's compiled kernel rounds it (its
// multiply-adds contracted: |v|^2 as len2Engine, 2.2 cs + |v| and
// u + 0.01 u_scale as one fma each), so the minimum is bit-identical to the
// engine's and the oracle's.
__device__ __forceinline__ float dtCandidate(float h, float cs, float vx, float vy, float vz, float ax, float ay,
                                             float az, float u, float duDt, uint8_t mat) {
    const float hi = fmaxf(h, 1.0e-6f);
    const float csI = fmaxf(cs, 0.05f);
    const float vMag = __fsqrt_rn(len2Engine(vx, vy, vz));
    const float dtCfl = __fdiv_rn(__fmul_rn(0.25f, hi), __fadd_rn(__fmaf_rn(2.2f, csI, vMag), 1.0e-6f));
    const float aMag = __fsqrt_rn(len2Engine(ax, ay, az));
    const float dtAcc = __fmul_rn(0.25f, __fsqrt_rn(__fdiv_rn(hi, __fadd_rn(aMag, 1.0e-8f))));
    const float uI = fmaxf(u, 0.0f);
    const float uScale = fmaxf(uI, c_mat[matIndex(mat)].u0Ref);
    const float dtTherm = __fdiv_rn(__fmul_rn(0.20f, __fmaf_rn(0.01f, uScale, uI)), __fadd_rn(fabsf(duDt), 1.0e-8f));
    return fminf(dtCfl, fminf(dtAcc, dtTherm));
}

// Block minimum of valid candidates, merged with atomicMin on the float bits
// (positive floats order like their bit patterns), sph_gravity.cu:1533-1549.
__device__ __forceinline__ void blockMinToWord(float v, uint32_t* word) {
    __shared__ float sMin[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warpMinF(v);
    if (lane == 0) sMin[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        float m = (lane < nw) ? sMin[lane] : 1.0e30f;
        m = warpMinF(m);
        if (lane == 0 && isfinite(m) && m > 0.0f) atomicMin(word, __float_as_uint(m));
    }
}

// Host clamp of launchReduceDtPsu (sph_gravity.cu:2137-2160) on the device.
__device__ __forceinline__ float resolveDt(uint32_t rawBits, float prevDt, float maxDt) {
    const float floorDt = fminf(1.0e-5f, maxDt);
    const float upper = (prevDt > 0.0f) ? fminf(prevDt * 1.15f, maxDt) : maxDt;
    float raw = __uint_as_float(rawBits);
    if (rawBits == 0x7f7f7f7fu || !isfinite(raw) || raw <= 0.0f) raw = upper;
    return fminf(upper, fmaxf(floorDt, raw));
}

// Pass-2 record of particle i (6 float4, read by pass 2 for i and for every
// neighbour j):
//   q0 {x, y, z, h}  q1 {vx, vy, vz, m}  q2 {rho, P_eff / rho^2, cs, f_Balsara}
//   q3 {sXX, sYY, sZZ, sXY} / rho^2   q4 {sXZ / rho^2, sYZ / rho^2, material, R_tensile}
//   q5 {m / rho, 210 / (pi H^5), 1 / rho^2, 1 / H}    (H = 2h)
// with h, rho and cs clamped as the engine clamps them on load.  Every
// derived value but 1 / H is the IEEE operation the engine's pair loop
// performs on the same inputs (sph_gravity.cu:1076-1142), done once per
// particle; 1 / H replaces the pair loop's quotient r / H by a product.
__device__ __forceinline__ void writePass2Record(float4* R, float x, float y, float z, float hRaw, float vx, float vy,
                                                 float vz, float m, float rhoRaw, float pEff, float csRaw, float fBalIn,
                                                 float sxx, float syy, float szz, float sxy, float sxz, float syz,
                                                 int mat) {
    const float h = fmaxf(hRaw, 1.0e-6f);
    const float rho = fmaxf(rhoRaw, 1.0e-9f);
    const float invRho2 = 1.0f / (rho * rho);
    const float H = 2.0f * h;
    const float H2 = H * H;
    const float H5 = H2 * H2 * H;
    const float gradNorm = 210.0f / (kPiF * H5);
    const float rTens = (pEff < 0.0f) ? (0.3f * (-pEff) * invRho2) : 0.0f;
    R[0] = make_float4(x, y, z, h);
    R[1] = make_float4(vx, vy, vz, m);
    R[2] = make_float4(rho, pEff * invRho2, csRaw, fBalIn);
    R[3] = make_float4(sxx * invRho2, syy * invRho2, szz * invRho2, sxy * invRho2);
    R[4] = make_float4(sxz * invRho2, syz * invRho2, __int_as_float(mat), rTens);
    R[5] = make_float4(m / rho, gradNorm, invRho2, 1.0f / H);
}

__global__ void __launch_bounds__(256) eosKernel(AstraeaParticles p, Work w, bool withRecords, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t mat = __ldg(&p.materialId[i]);
    const float rho = __ldg(&p.rho[i]);
    const EosOut e = evaluateEosF32(mat, rho, __ldg(&p.u[i]), __ldg(&p.damage[i]));
    p.pressure[i] = e.P;
    p.soundSpeed[i] = e.cs;
    p.tempK[i] = e.T;
    p.phaseId[i] = e.phase;
    if (withRecords) {
        const float h = fmaxf(__ldg(&p.h[i]), 1.0e-6f);
        const float cs = fmaxf(e.cs, 0.05f);
        const float fBal = balsaraSwitch(__ldg(&p.divV[i]), __ldg(&p.curlVX[i]), __ldg(&p.curlVY[i]),
                                         __ldg(&p.curlVZ[i]), cs, h);
        writePass2Record(w.rec2 + kRec2Width * static_cast<size_t>(i), __ldg(&p.posX[i]), __ldg(&p.posY[i]),
                         __ldg(&p.posZ[i]), h, __ldg(&p.velX[i]), __ldg(&p.velY[i]), __ldg(&p.velZ[i]),
                         __ldg(&p.mass[i]), rho, effectivePressure(e.P, e.phase), cs, fBal, __ldg(&p.sXX[i]),
                         __ldg(&p.sYY[i]), __ldg(&p.sZZ[i]), __ldg(&p.sXY[i]), __ldg(&p.sXZ[i]), __ldg(&p.sYZ[i]),
                         static_cast<int>(mat));
    }
}

__global__ void __launch_bounds__(256) kickKernel(AstraeaParticles p, uint32_t n, KickArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float halfDt = a.halfDtHost;
    if (a.dtMode == 1) {
        const float dt = resolveDt(*a.rawMinIn, a.dtSlots[a.parity], a.maxDt);
        halfDt = 0.5f * dt;
        if (blockIdx.x == 0 && threadIdx.x == 0) a.dtSlots[a.parity ^ 1] = dt;
    } else if (a.dtMode == 2) {
        halfDt = 0.5f * a.dtSlots[a.parity ^ 1];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.resetWord != nullptr) *a.resetWord = 0x7f7f7f7fu;
        if (a.boundsWordsInit != nullptr) {
            const uint32_t hi = orderedFromFloat(1.0e30f), lo = orderedFromFloat(-1.0e30f);
            uint32_t* wds = a.boundsWordsInit;
            wds[kWBounds + 0] = hi; wds[kWBounds + 1] = hi; wds[kWBounds + 2] = hi;
            wds[kWBounds + 3] = lo; wds[kWBounds + 4] = lo; wds[kWBounds + 5] = lo;
            wds[kWLiving + 0] = 0u; wds[kWLiving + 1] = 0u; wds[kWMassMax] = 0u;
        }
    }
    float dtCand = 1.0e30f;
    if (i < n) {
        // every input first (the fields are plain pointers, so loads after a
        // store could not be moved ahead of it): all reads in flight at once
        const float ax0 = p.accX[i], ay0 = p.accY[i], az0 = p.accZ[i];
        const float vx0 = p.velX[i], vy0 = p.velY[i], vz0 = p.velZ[i];
        const float rho0 = p.rho[i], drho = p.drhoDt[i], u0 = p.u[i], du = p.duDt[i];
        const float dOld = p.damageCbrt[i], dDam = p.dDamageCbrtDt[i];
        const float temp0 = p.tempK[i], pres0 = p.pressure[i], cs0 = p.soundSpeed[i];
        const float s0xx = p.sXX[i], s0yy = p.sYY[i], s0zz = p.sZZ[i], s0xy = p.sXY[i], s0xz = p.sXZ[i], s0yz = p.sYZ[i];
        const float dsxx = p.dSXX[i], dsyy = p.dSYY[i], dszz = p.dSZZ[i], dsxy = p.dSXY[i], dsxz = p.dSXZ[i], dsyz = p.dSYZ[i];
        const float hI = (a.rawMinOut != nullptr) ? p.h[i] : 0.0f;
        const float vx = vx0 + halfDt * ax0;
        const float vy = vy0 + halfDt * ay0;
        const float vz = vz0 + halfDt * az0;
        p.velX[i] = vx; p.velY[i] = vy; p.velZ[i] = vz;
        p.velHalfX[i] = vx; p.velHalfY[i] = vy; p.velHalfZ[i] = vz;
        const float rhoNew = fmaxf(rho0 + halfDt * drho, 1.0e-9f);
        p.rho[i] = rhoNew;
        const uint8_t matRaw = p.materialId[i];
        const int mi = matIndex(matRaw);
        const MatConst& st = c_mat[mi];
        float uNew = u0 + halfDt * du;
        if (a.clampThermal) {
            uNew = fmaxf(uNew, coldEnergyF32(mi, rhoNew) + 3.0f * st.cv);
        } else {
            uNew = fmaxf(uNew, 0.0f);
        }
        p.u[i] = uNew;
        float dCbrt = dOld + halfDt * dDam;
        dCbrt = fminf(1.0f, fmaxf(dOld, dCbrt));
        const float D = dCbrt * dCbrt * dCbrt;
        p.damageCbrt[i] = dCbrt;
        p.damage[i] = D;
        float tempK = temp0;
        float pres = pres0;
        EosOut e{};
        if (a.clampThermal || a.withEos) e = evaluateEosF32(static_cast<uint8_t>(mi), rhoNew, uNew, D);
        if (a.clampThermal) {                      // EOS before the strength update (:1334-1340)
            tempK = e.T; pres = e.P;
            p.pressure[i] = e.P; p.soundSpeed[i] = e.cs; p.tempK[i] = e.T; p.phaseId[i] = e.phase;
        }
        float sXX = 0.f, sYY = 0.f, sZZ = 0.f, sXY = 0.f, sXZ = 0.f, sYZ = 0.f;
        if (!(st.muShear <= 0.0f || st.tMelt <= 0.0f || tempK >= st.tMelt)) {   // :1342-1373
            sXX = s0xx + halfDt * dsxx;
            sYY = s0yy + halfDt * dsyy;
            sZZ = s0zz + halfDt * dszz;
            sXY = s0xy + halfDt * dsxy;
            sXZ = s0xz + halfDt * dsxz;
            sYZ = s0yz + halfDt * dsyz;
            const float tr3 = (sXX + sYY + sZZ) * (1.0f / 3.0f);
            sXX -= tr3; sYY -= tr3; sZZ -= tr3;
            const float tRatio = tempK / st.tMelt;
            const float yIntact = (1.0f - D) * st.yieldY0 * fmaxf(0.0f, 1.0f - tRatio);
            const float yFriction = D * fminf(st.yieldY0, 0.6f * fmaxf(0.0f, pres));
            const float Y = fmaxf(yIntact, yFriction);
            const float j2 = 0.5f * (sXX * sXX + sYY * sYY + sZZ * sZZ + 2.0f * (sXY * sXY + sXZ * sXZ + sYZ * sYZ));
            const float eq = sqrtf(3.0f * j2 + 1.0e-30f);
            const float scale = (Y <= 0.0f) ? 0.0f : fminf(1.0f, Y / eq);
            sXX *= scale; sYY *= scale; sZZ *= scale; sXY *= scale; sXZ *= scale; sYZ *= scale;
        }
        p.sXX[i] = sXX; p.sYY[i] = sYY; p.sZZ[i] = sZZ; p.sXY[i] = sXY; p.sXZ[i] = sXZ; p.sYZ[i] = sYZ;
        float cs = a.clampThermal ? e.cs : cs0;
        if (a.withEos && !a.clampThermal) {        // the engine's EOS launch after the kick
            p.pressure[i] = e.P; p.soundSpeed[i] = e.cs; p.tempK[i] = e.T; p.phaseId[i] = e.phase;
            cs = e.cs;
        }
        if (a.driftOut != nullptr) a.driftOut[i].b = make_float4(vx, vy, vz, rhoNew);
        if (a.rawMinOut != nullptr) {
            const float d = dtCandidate(hI, cs, vx, vy, vz, ax0, ay0, az0, uNew, du, matRaw);
            if (isfinite(d) && d > 0.0f) dtCand = d;
        }
    }
    if (a.rawMinOut != nullptr) blockMinToWord(dtCand, a.rawMinOut);
}

__global__ void __launch_bounds__(256) packPass2Kernel(AstraeaParticles p, Work w, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float h = fmaxf(__ldg(&p.h[i]), 1.0e-6f);
    const float cs = fmaxf(__ldg(&p.soundSpeed[i]), 0.05f);
    const float fBal = balsaraSwitch(__ldg(&p.divV[i]), __ldg(&p.curlVX[i]), __ldg(&p.curlVY[i]),
                                     __ldg(&p.curlVZ[i]), cs, h);
    writePass2Record(w.rec2 + kRec2Width * static_cast<size_t>(i), __ldg(&p.posX[i]), __ldg(&p.posY[i]),
                     __ldg(&p.posZ[i]), h, __ldg(&p.velX[i]), __ldg(&p.velY[i]), __ldg(&p.velZ[i]),
                     __ldg(&p.mass[i]), __ldg(&p.rho[i]),
                     effectivePressure(__ldg(&p.pressure[i]), __ldg(&p.phaseId[i])), cs, fBal, __ldg(&p.sXX[i]),
                     __ldg(&p.sYY[i]), __ldg(&p.sZZ[i]), __ldg(&p.sXY[i]), __ldg(&p.sXZ[i]), __ldg(&p.sYZ[i]),
                     static_cast<int>(__ldg(&p.materialId[i])));
}

__global__ void __launch_bounds__(256) driftPlainKernel(AstraeaParticles p, uint32_t n, float dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = static_cast<double>(dt);
    p.posX[i] = static_cast<float>(static_cast<double>(p.posX[i]) + d * static_cast<double>(p.velX[i]));
    p.posY[i] = static_cast<float>(static_cast<double>(p.posY[i]) + d * static_cast<double>(p.velY[i]));
    p.posZ[i] = static_cast<float>(static_cast<double>(p.posZ[i]) + d * static_cast<double>(p.velZ[i]));
}

__global__ void setDtSlotsKernel(float* slots, int parity, float prevDt, uint32_t* rawMin) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        slots[parity] = prevDt;
        slots[parity ^ 1] = 0.0f;
        rawMin[parity] = 0x7f7f7f7fu;
    }
}

__global__ void __launch_bounds__(256) reduceDtKernel(AstraeaParticles p, uint32_t n, uint32_t* out) {
    float m = 1.0e30f;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float d = dtCandidate(__ldg(&p.h[i]), __ldg(&p.soundSpeed[i]), __ldg(&p.velX[i]), __ldg(&p.velY[i]),
                                    __ldg(&p.velZ[i]), __ldg(&p.accX[i]), __ldg(&p.accY[i]), __ldg(&p.accZ[i]),
                                    __ldg(&p.u[i]), __ldg(&p.duDt[i]), __ldg(&p.materialId[i]));
        if (isfinite(d) && d > 0.0f) m = fminf(m, d);
    }
    blockMinToWord(m, out);
}

__global__ void __launch_bounds__(256) clearStatsKernel(AstraeaParticles p, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    p.accX[i] = 0.f; p.accY[i] = 0.f; p.accZ[i] = 0.f;
    p.drhoDt[i] = 0.f; p.duDt[i] = 0.f; p.radPowerW[i] = 0.f;
    p.dSXX[i] = 0.f; p.dSYY[i] = 0.f; p.dSZZ[i] = 0.f; p.dSXY[i] = 0.f; p.dSXZ[i] = 0.f; p.dSYZ[i] = 0.f;
    p.dDamageCbrtDt[i] = 0.f; p.divV[i] = 0.f;
    p.curlVX[i] = 0.f; p.curlVY[i] = 0.f; p.curlVZ[i] = 0.f;
    p.shepardC[i] = 1.0f; p.surfFactor[i] = 0.0f; p.phiGrav[i] = 0.0f;
}

inline unsigned gridFor(uint32_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

cudaError_t launchClearStats(const AstraeaParticles& p, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    clearStatsKernel<<<gridFor(n, 256), 256, 0, st>>>(p, n);
    return cudaGetLastError();
}

cudaError_t launchEos(const AstraeaParticles& p, const Work* w, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    Work none{};
    eosKernel<<<gridFor(n, 256), 256, 0, st>>>(p, w ? *w : none, w != nullptr, n);
    return cudaGetLastError();
}

cudaError_t launchKick(const AstraeaParticles& p, uint32_t n, const KickArgs& a, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    kickKernel<<<gridFor(n, 256), 256, 0, st>>>(p, n, a);
    return cudaGetLastError();
}

cudaError_t launchPackPass2Records(const AstraeaParticles& p, const Work& w, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    packPass2Kernel<<<gridFor(n, 256), 256, 0, st>>>(p, w, n);
    return cudaGetLastError();
}

cudaError_t launchDriftPlain(const AstraeaParticles& p, uint32_t n, float dt, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    driftPlainKernel<<<gridFor(n, 256), 256, 0, st>>>(p, n, dt);
    return cudaGetLastError();
}

cudaError_t launchSetDtSlots(float* slots, int parity, float prevDt, uint32_t* rawMin, cudaStream_t st) {
    setDtSlotsKernel<<<1, 32, 0, st>>>(slots, parity, prevDt, rawMin);
    return cudaGetLastError();
}

cudaError_t launchReduceDt(const AstraeaParticles& p, uint32_t n, uint32_t* rawMinOut, int sms, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const unsigned blocks = std::min(gridFor(n, 256), static_cast<unsigned>(sms) * 4u);
    reduceDtKernel<<<blocks, 256, 0, st>>>(p, n, rawMinOut);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
