// render.cu -- render-record and crust-tracer packing, and the PCLS frame.
//
// Restates packRenderRecordsKernel and extractTracersKernel
// (engine/sph_gravity.cu:1554-1743) with the same per-particle arithmetic
// (same expressions, same CUDA math functions, so the bytes match the
// engine's), and adds a device-side builder of the uncompressed PCLS frame of
// server/binary_protocol.cpp:155-217 (40-byte header, particle records,
// tracer records, speed bytes) so one device-to-host copy ships a frame.
//
// GB300 layout choices: these are HBM-bound byte-packing passes (about 47 B
// read and 21 B written per particle), so each block builds its 256 records
// in shared memory and writes them out with the widest stores the
// destination's alignment allows (16, 8 or 4 bytes; bytes as a last resort),
// instead of five scattered 4-byte stores per thread.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kPackThreads = 256;

// Wire-format quantisation scales of the engine (sph_gravity.cu:1675-1677):
// temperature log range 10 K .. 200 kK, pressure 1 kPa .. 10 TPa (in GPa
// x 1000), particle radius 1 .. 2000 km.
constexpr float kInvLnTempRange = 1.0f / 9.9034875525361280f;    // 1 / ln(2e4)
constexpr float kInvLnPresRange = 1.0f / 16.118095650958320f;    // 1 / ln(1e7)
constexpr float kInvLnRadRange = 1.0f / 7.6009024595420823f;     // 1 / ln(2e3)
constexpr float kPiF = 3.14159265358979323846f;

__device__ __forceinline__ float finite0(float v) { return isfinite(v) ? v : 0.0f; }

// Copy `words` 32-bit words from shared memory to an arbitrary byte address
// with the widest aligned stores; all threads of the block take part.
__device__ __forceinline__ void storeWords(uint8_t* dst, const uint32_t* tile, int words) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
    if ((a & 15u) == 0u) {
        const int q = words >> 2;
        for (int k = threadIdx.x; k < q; k += blockDim.x)
            reinterpret_cast<uint4*>(dst)[k] =
                make_uint4(tile[4 * k], tile[4 * k + 1], tile[4 * k + 2], tile[4 * k + 3]);
        for (int k = 4 * q + threadIdx.x; k < words; k += blockDim.x) reinterpret_cast<uint32_t*>(dst)[k] = tile[k];
    } else if ((a & 7u) == 0u) {
        const int q = words >> 1;
        for (int k = threadIdx.x; k < q; k += blockDim.x)
            reinterpret_cast<uint2*>(dst)[k] = make_uint2(tile[2 * k], tile[2 * k + 1]);
        for (int k = 2 * q + threadIdx.x; k < words; k += blockDim.x) reinterpret_cast<uint32_t*>(dst)[k] = tile[k];
    } else if ((a & 3u) == 0u) {
        for (int k = threadIdx.x; k < words; k += blockDim.x) reinterpret_cast<uint32_t*>(dst)[k] = tile[k];
    } else {
        for (int k = threadIdx.x; k < 4 * words; k += blockDim.x) dst[k] = static_cast<uint8_t>(tile[k >> 2] >> (8 * (k & 3)));
    }
}

// One 20-byte particle record (ParticleRecordPacked, sph_gravity.cu:1570-1581)
// as five little-endian words, and the speed byte (:1730-1736).
__device__ __forceinline__ void renderRecord(const AstraeaParticles& p, uint32_t i, float sx, float sy, float sz,
                                             uint32_t rec[5], uint8_t& speedByte, bool withSpeed) {
    const float xKm = finite0((__ldg(&p.posX[i]) - sx) * 1000.0f);
    const float yKm = finite0((__ldg(&p.posY[i]) - sy) * 1000.0f);
    const float zKm = finite0((__ldg(&p.posZ[i]) - sz) * 1000.0f);

    const float T = fmaxf(10.0f, finite0(__ldg(&p.tempK[i])));
    const float tNorm = fminf(1.0f, fmaxf(0.0f, logf(T * 0.1f) * kInvLnTempRange));
    const uint32_t tempU16 = static_cast<uint16_t>(lrintf(65535.0f * tNorm));

    const float pGPa = finite0(__ldg(&p.pressure[i])) * 1000.0f;
    uint32_t presU16 = 0u;
    if (pGPa > 1.0e-3f) {
        const float pNorm = fminf(1.0f, fmaxf(0.0f, logf(pGPa * 1000.0f) * kInvLnPresRange));
        presU16 = static_cast<uint16_t>(lrintf(1.0f + 65534.0f * pNorm));
    }

    const uint32_t mat = __ldg(&p.materialId[i]);
    const uint32_t phaseBody = static_cast<uint8_t>(((__ldg(&p.bodyId[i]) & 0x0Fu) << 4) | (__ldg(&p.phaseId[i]) & 0x0Fu));
    const float dam = fminf(1.0f, fmaxf(0.0f, finite0(__ldg(&p.damage[i]))));
    const uint32_t damU8 = static_cast<uint8_t>(lrintf(dam * 255.0f));

    const float volPsu = fmaxf(__ldg(&p.mass[i]), 0.0f) / fmaxf(__ldg(&p.rho[i]), 1.0e-9f);
    const float rKm = cbrtf((3.0f * volPsu) / (4.0f * kPiF)) * 1000.0f;
    const float rNorm = fminf(1.0f, fmaxf(0.0f, logf(fmaxf(rKm, 1.0f)) * kInvLnRadRange));
    const uint32_t radU8 = static_cast<uint8_t>(lrintf(255.0f * rNorm));

    rec[0] = __float_as_uint(xKm);
    rec[1] = __float_as_uint(yKm);
    rec[2] = __float_as_uint(zKm);
    rec[3] = tempU16 | (presU16 << 16);
    rec[4] = mat | (phaseBody << 8) | (damU8 << 16) | (radU8 << 24);

    speedByte = 0;
    if (withSpeed) {
        const float vx = __ldg(&p.velX[i]);
        const float vy = __ldg(&p.velY[i]);
        const float vz = __ldg(&p.velZ[i]);
        const float speedKmS = finite0(sqrtf(vx * vx + vy * vy + vz * vz));
        const float vNorm = fminf(1.0f, fmaxf(0.0f, logf(fmaxf(speedKmS, 0.05f) * 20.0f) * kInvLnRadRange));
        speedByte = static_cast<uint8_t>(lrintf(255.0f * vNorm));
    }
}

__global__ void __launch_bounds__(kPackThreads) packRenderKernel(AstraeaParticles p, uint32_t n, uint8_t* records,
                                                                 uint8_t* speed, float sx, float sy, float sz) {
    __shared__ uint32_t tile[5 * kPackThreads];   // stride 5 words: conflict-free
    const uint32_t base = blockIdx.x * kPackThreads;
    const uint32_t i = base + threadIdx.x;
    if (i < n) {
        uint32_t rec[5];
        uint8_t sb;
        renderRecord(p, i, sx, sy, sz, rec, sb, speed != nullptr);
#pragma unroll
        for (int k = 0; k < 5; ++k) tile[5 * threadIdx.x + k] = rec[k];
        if (speed != nullptr) speed[i] = sb;
    }
    __syncthreads();
    const int cnt = static_cast<int>(min(static_cast<uint32_t>(kPackThreads), n - base));
    storeWords(records + static_cast<size_t>(base) * 20u, tile, 5 * cnt);
}

// One 40-byte crust-tracer record (CrustTracerRecordPacked,
// sph_gravity.cu:1554-1567, values of :1586-1668) as ten words.
__device__ __forceinline__ void tracerRecord(const AstraeaParticles& p, uint32_t i, int32_t tIdx, float lx, float ly,
                                             float lz, float sx, float sy, float sz, uint32_t w[10]) {
    const float px = __ldg(&p.posX[i]);
    const float py = __ldg(&p.posY[i]);
    const float pz = __ldg(&p.posZ[i]);
    const float dx = px - lx;
    const float dy = py - ly;
    const float dz = pz - lz;
    const float rPsu = sqrtf(dx * dx + dy * dy + dz * dz);
    const float rRest = __ldg(&p.tracerRestRadiusPsu[i]);
    const float dispKm = (rPsu - rRest) * 1000.0f;

    float normalDelta = 0.0f;
    if (rPsu > 1.0e-9f) {
        const float invR = 1.0f / rPsu;
        const float nx = dx * invR;
        const float ny = dy * invR;
        const float nz = dz * invR;
        const float dotVal = fminf(1.0f, fmaxf(-1.0f, nx * __ldg(&p.tracerRestNormalX[i]) +
                                                          ny * __ldg(&p.tracerRestNormalY[i]) +
                                                          nz * __ldg(&p.tracerRestNormalZ[i])));
        normalDelta = acosf(dotVal);
    }

    const float dam = fminf(1.0f, fmaxf(0.0f, finite0(__ldg(&p.damage[i]))));
    const float tempK = fmaxf(3.0f, finite0(__ldg(&p.tempK[i])));
    const uint8_t phase = __ldg(&p.phaseId[i]);
    const bool isOcean = __ldg(&p.tracerIsOcean[i]) != 0u;
    // phases 2 and 3 are Vapor and Plasma (engine/types.hpp PhaseId)
    const bool isDisrupted = (dam >= 0.85f) || (phase == 2u) || (phase == 3u) ||
                             (fabsf(rPsu - rRest) > 0.5f * fmaxf(rRest, 1.0e-3f));

    const float dvShockMs = fmaxf(0.0f, -finite0(__ldg(&p.divV[i]))) * fmaxf(__ldg(&p.h[i]), 0.0f) * 1000.0f;
    const float overpressureKpa = fmaxf(0.0f, 1.225f * 340.0f * dvShockMs * 1.0e-3f);
    const float tsunamiHeightM = isOcean ? fmaxf(0.0f, finite0(dispKm) * 1000.0f) : 0.0f;

    const uint32_t flags = (isOcean ? 1u : 0u) | (isDisrupted ? 2u : 0u);
    w[0] = static_cast<uint32_t>(static_cast<uint16_t>(tIdx)) | (flags << 16);
    w[1] = __float_as_uint(finite0((px - sx) * 1000.0f));
    w[2] = __float_as_uint(finite0((py - sy) * 1000.0f));
    w[3] = __float_as_uint(finite0((pz - sz) * 1000.0f));
    w[4] = __float_as_uint(finite0(dispKm));
    w[5] = __float_as_uint(finite0(normalDelta));
    w[6] = __float_as_uint(tempK);
    w[7] = __float_as_uint(dam);
    w[8] = __float_as_uint(finite0(overpressureKpa));
    w[9] = __float_as_uint(finite0(tsunamiHeightM));
}

__global__ void __launch_bounds__(kPackThreads) extractTracersKernel(AstraeaParticles p, uint32_t n, uint8_t* records,
                                                                     uint32_t tracerCount, float lx, float ly,
                                                                     float lz, float sx, float sy, float sz) {
    const uint32_t i = blockIdx.x * kPackThreads + threadIdx.x;
    if (i >= n) return;
    const int32_t tIdx = __ldg(&p.tracerIndex[i]);
    if (tIdx < 0 || static_cast<uint32_t>(tIdx) >= tracerCount) return;
    uint32_t w[10];
    tracerRecord(p, i, tIdx, lx, ly, lz, sx, sy, sz, w);
    uint8_t* dst = records + static_cast<size_t>(tIdx) * 40u;
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
    if ((a & 7u) == 0u) {
#pragma unroll
        for (int k = 0; k < 5; ++k) reinterpret_cast<uint2*>(dst)[k] = make_uint2(w[2 * k], w[2 * k + 1]);
    } else if ((a & 3u) == 0u) {
#pragma unroll
        for (int k = 0; k < 10; ++k) reinterpret_cast<uint32_t*>(dst)[k] = w[k];
    } else {
        for (int k = 0; k < 40; ++k) dst[k] = static_cast<uint8_t>(w[k >> 2] >> (8 * (k & 3)));
    }
}

__global__ void writeHeaderKernel(uint8_t* frame, PclsHeaderWords h) {
    const int k = threadIdx.x;
    if (k < 10) {
        const uint32_t v = h.w[k];
        frame[4 * k + 0] = static_cast<uint8_t>(v);
        frame[4 * k + 1] = static_cast<uint8_t>(v >> 8);
        frame[4 * k + 2] = static_cast<uint8_t>(v >> 16);
        frame[4 * k + 3] = static_cast<uint8_t>(v >> 24);
    }
}

}  // namespace

cudaError_t launchPackRender(const AstraeaParticles& p, uint32_t n, uint8_t* records, uint8_t* speed, float sx, float sy,
                             float sz, cudaStream_t st) {
    if (n == 0 || records == nullptr) return cudaSuccess;
    packRenderKernel<<<(n + kPackThreads - 1) / kPackThreads, kPackThreads, 0, st>>>(p, n, records, speed, sx, sy, sz);
    return cudaGetLastError();
}

cudaError_t launchExtractTracers(const AstraeaParticles& p, uint32_t n, uint8_t* records, uint32_t tracerCount,
                                 float lx, float ly, float lz, float sx, float sy, float sz, cudaStream_t st) {
    if (tracerCount == 0 || records == nullptr) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(records, 0, static_cast<size_t>(tracerCount) * 40u, st);
    if (e != cudaSuccess || n == 0) return e;
    extractTracersKernel<<<(n + kPackThreads - 1) / kPackThreads, kPackThreads, 0, st>>>(p, n, records, tracerCount,
                                                                                         lx, ly, lz, sx, sy, sz);
    return cudaGetLastError();
}

cudaError_t launchWriteHeader(uint8_t* frame, const PclsHeaderWords& h, cudaStream_t st) {
    writeHeaderKernel<<<1, 32, 0, st>>>(frame, h);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
