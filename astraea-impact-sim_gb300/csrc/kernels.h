// kernels.h -- launchers of every kernel of the library (host side) and the
// small device helpers more than one translation unit inlines.
#pragma once

#include <string>
#include <vector>

#include "internal.h"

namespace astraea_gb300 {

// ------------------------------------------------------ device helpers ---
__device__ __forceinline__ float warpMinF(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warpMaxF(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Reduce each thread's partial AABB over the block and merge it into the
// ordered-uint bound words with atomics (engine/sph_gravity.cu:300-324).
// Every thread of the block must call it.
__device__ __forceinline__ void blockBoundsToWords(const float* mn, const float* mx, uint32_t* words) {
    __shared__ float sMin[3][32], sMax[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = warpMinF(mn[k]), b = warpMaxF(mx[k]);
        if (lane == 0) { sMin[k][warp] = a; sMax[k][warp] = b; }
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float a = (lane < nw) ? sMin[k][lane] : 1.0e30f;
            float b = (lane < nw) ? sMax[k][lane] : -1.0e30f;
            a = warpMinF(a);
            b = warpMaxF(b);
            if (lane == 0) {
                atomicMin(&words[kWBounds + k], orderedFromFloat(a));
                atomicMax(&words[kWBounds + 3 + k], orderedFromFloat(b));
            }
        }
    }
}

// ------------------------------------------------------------ build.cu ---
cudaError_t launchInitBounds(uint32_t* words, cudaStream_t st);
cudaError_t launchBounds(const AstraeaParticles& p, uint32_t n, uint32_t* words, int sms, cudaStream_t st);
cudaError_t launchPermuteLeavesKarras(const AstraeaParticles& p, const AstraeaParticles& alt,
                                      const AstraeaRadixBvh& bvh, const float4* posSrc, const Work& w, uint32_t n,
                                      uint32_t* livingFlags, bool allFields, cudaStream_t st);
cudaError_t launchRefreshLeaves(const AstraeaParticles& p, const Work& w, uint32_t n, bool withVelRho,
                                cudaStream_t st);
cudaError_t launchRefit(const AstraeaRadixBvh& bvh, const Work& w, uint32_t n, bool moments, cudaStream_t st);
// node masses and COMs in the engine's FP32 bottom-up rounding (after launchRefit)
cudaError_t launchEngineNodeMoments(const AstraeaParticles& p, const AstraeaRadixBvh& bvh, const Work& w, uint32_t n,
                                    cudaStream_t st);
// Scratch geometry of the range refit: blocks of 256 leaves, sparse-table levels.
uint32_t refitBlocks(uint32_t n);
uint32_t refitLevels(uint32_t nb);

// ----------------------------------------------------------- render.cu ---
// PCLS frame header as ten little-endian words (server/binary_protocol.cpp:76-87).
struct PclsHeaderWords {
    uint32_t w[10];
};
cudaError_t launchPackRender(const AstraeaParticles& p, uint32_t n, uint8_t* records, uint8_t* speed, float sx, float sy,
                             float sz, cudaStream_t st);
cudaError_t launchExtractTracers(const AstraeaParticles& p, uint32_t n, uint8_t* records, uint32_t tracerCount,
                                 float lx, float ly, float lz, float sx, float sy, float sz, cudaStream_t st);
cudaError_t launchWriteHeader(uint8_t* frame, const PclsHeaderWords& h, cudaStream_t st);

// -------------------------------------------------------- telemetry.cu ---
cudaError_t launchTelemetry(const AstraeaParticles& p, uint32_t n, double targetRadiusPsu, int livingBodyPresent,
                            int sms, AstraeaTelemetry* hostOut, cudaStream_t st);

// ------------------------------------------------------------ relax.cu ---
cudaError_t launchRelaxRecentre(const AstraeaParticles& p, uint32_t n, const double* anchorT, uint32_t anchorCount,
                                int sms, cudaStream_t st);
cudaError_t launchRelaxDiagnostic(const AstraeaParticles& p, uint32_t n, double nominalRadius, int sms,
                                  double* hostOut, cudaStream_t st);
cudaError_t launchRelaxAnchor(const AstraeaParticles& p, uint32_t n, const double* anchorT, uint32_t anchorCount,
                              cudaStream_t st);

// ------------------------------------------------------------- diag.cu ---
cudaError_t launchDirectGravityF64(const AstraeaParticles& p, uint32_t n, const uint32_t* targets, uint32_t nt,
                                   double* acc3, double* phi, cudaStream_t st);

// ---------------------------------------------------------- gravity.cu ---
// Far-field mode 2: the walk also takes a node the theta test opens when
// every member passes theta_far (sound bound) and L1 group extent <=
// gamma r; it records the (group, node) pair and each group's centre.
struct FarCapture {
    uint2* pairs;          // {group, node}
    uint32_t cap;
    uint32_t* count;       // device word, zeroed by the caller
    float4* groups;        // per group {centre x, y, z, L1 extent}
    float thetaFar2;
    float gamma2;
    uint32_t groupStride;  // only groups g % stride == 0 apply the far test
};
// warps: 2, 4 or 8 warps per block for the plain and quadrupole walks (the
// autotuner's choice; the learned far-field walk uses 4); results do not
// depend on it.
// expansion: far-field mode 3 (quadrupole walk with w.leafBucket leaf
// buckets and the group expansion of nodes far against the group,
// w.expandGamma2); needs quadrupole.
cudaError_t launchGravity(const AstraeaParticles& p, const Work& w, uint32_t n, float theta, bool quadrupole, int sms,
                          cudaStream_t st, const FarCapture* far = nullptr, int warps = 4, bool expansion = false);

// ---------------------------------------------------------------- ff.cu ---
namespace ff {
constexpr int kIn = 16, kHid = 64, kOut = 16, kUsedOut = 12;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid;
constexpr int kB3 = kW3 + kHid * kOut, kParams = kB3 + kOut;   // 6,288 FP32 parameters
struct Net {
    float* params;     // FP32 master weights (W row-major in x out, then bias), layout above
    float* grads;
    float* adamM;
    float* adamV;
    float* outScale;   // kOut
    float* loss;       // one word
};
cudaError_t prepareKernels();
cudaError_t launchLabels(const Work& w, uint32_t n, const uint2* pairs, uint32_t count, const float4* groups,
                         float* feat, float* label, cudaStream_t st);
cudaError_t launchTrain(const Net& net, const float* feat, const float* label, uint32_t count, int sms,
                        cudaStream_t st);
cudaError_t launchAdam(const Net& net, float lr, int step, cudaStream_t st);
cudaError_t launchPredict(const Net& net, const float* feat, uint32_t count, float* out, int sms, cudaStream_t st);
cudaError_t launchApply(const Net& net, const Work& w, const uint2* pairs, const uint32_t* countWord, uint32_t cap,
                        const float4* groups, float* groupCorr, int sms, cudaStream_t st);
cudaError_t launchCorrect(const AstraeaParticles& p, const float4* groups, const float* groupCorr, uint32_t n,
                          cudaStream_t st);
// Device state of the learned mode's gate (one per device).
constexpr uint32_t kGateMaxTargets = 1024;   // sampled particles of one gate, at most
struct GateDev {
    unsigned long long fallbacks;  // gated calls that fell back to the plain walk
    uint32_t runFallback;          // 1: the plain walk after the gate runs, 0: it returns at once
    uint32_t lastPairs;            // (group, node) pairs of the last gated call
    float lastRms;                 // RMS relative error of the last gate
    uint32_t reserved;
    double acc[3 * kGateMaxTargets];  // direct-sum accelerations of the targets (cleared by the decision)
};
// Direct-sum spot check of K <= kGateMaxTargets sampled particles (FP64 pair
// terms, or FP32 pair terms with FP64 sums) and the decision (gate->runFallback).
cudaError_t launchGate(const AstraeaParticles& p, const Work& w, uint32_t n, uint32_t K, float tolerance,
                       const uint32_t* pairCount, uint32_t pairCap, GateDev* gate, bool fp32Pairs, cudaStream_t st);
}  // namespace ff

// -------------------------------------------------------------- sph.cu ---
// warps: 2, 4 or 8 warps per block (the autotuner's choice; results do not depend on it)
cudaError_t launchBuildNeighbors(const Work& w, uint32_t n, int sms, cudaStream_t st, int warps = 4);
cudaError_t launchPass1(const AstraeaParticles& p, const Work& w, uint32_t n, cudaStream_t st);
cudaError_t launchPass2(const AstraeaParticles& p, const Work& w, uint32_t n, const uint32_t* livingFlags,
                        cudaStream_t st);
// XSPH drift; new positions go to w.driftPos when toScratch, else back into
// p.pos (after all neighbours were read).  Also merges the new positions'
// AABB into the bound words when boundsWords != nullptr.
cudaError_t launchDrift(const AstraeaParticles& p, const Work& w, uint32_t n, const float* dtDev, float dtHost,
                        bool useList, bool toScratch, uint32_t* boundsWords, cudaStream_t st);

// -------------------------------------------------------- integrate.cu ---
cudaError_t launchClearStats(const AstraeaParticles& p, uint32_t n, cudaStream_t st);
// EOS; when w != nullptr also writes the pass-2 neighbour records.
cudaError_t launchEos(const AstraeaParticles& p, const Work* w, uint32_t n, cudaStream_t st);
// Half kick.  dtMode 0: halfDt = halfDtHost.  dtMode 1 (opening kick of a
// fused step): dt = clamp of the raw minimum *rawMinIn against the previous
// dt dtSlots[parity] (the host clamp of launchReduceDtPsu), written to
// dtSlots[parity ^ 1].  dtMode 2 (closing kick): dt = dtSlots[parity ^ 1].
struct KickArgs {
    float halfDtHost;
    int dtMode;
    bool clampThermal;
    bool withEos;              // evaluate the EOS on the kicked state (fused)
    const uint32_t* rawMinIn;  // raw dt minimum bits (device), dtMode 1
    float* dtSlots;            // 2 floats indexed by step parity
    int parity;
    float maxDt;
    uint32_t* rawMinOut;       // when non-null: reduce the next dt minimum into it
    uint32_t* resetWord;       // when non-null: block 0 writes 0x7f7f7f7f here
    uint32_t* boundsWordsInit; // when non-null: block 0 re-arms bounds + living flags
    Rec32* driftOut;           // when non-null: write the {v, rho} half of the drift records
};
cudaError_t launchKick(const AstraeaParticles& p, uint32_t n, const KickArgs& a, cudaStream_t st);
cudaError_t launchReduceDt(const AstraeaParticles& p, uint32_t n, uint32_t* rawMinOut, int sms, cudaStream_t st);
// Arm the fused step's device dt state: slots[parity] = prevDt, raw minimum
// word of this parity reset for a fresh reduction.
cudaError_t launchSetDtSlots(float* slots, int parity, float prevDt, uint32_t* rawMin, cudaStream_t st);
// Pass-2 records from the current SoA, without evaluating the EOS.
cudaError_t launchPackPass2Records(const AstraeaParticles& p, const Work& w, uint32_t n, cudaStream_t st);
// x += dt v without XSPH (drift without a tree, sph_gravity.cu:1484-1488).
cudaError_t launchDriftPlain(const AstraeaParticles& p, uint32_t n, float dt, cudaStream_t st);

// -------------------------------------------------------------- diag.cu ---
cudaError_t measureFp32Tflops(int sms, float* tflops, cudaStream_t st);
// Scalar fmaf and packed fma.rn.f32x2 throughput, and the larger of the two.
cudaError_t measureFp32TflopsBoth(int sms, float* scalarOut, float* packedOut, float* peakOut, cudaStream_t st);

// ------------------------------------------------------------ planet.cu ---
namespace planet {
struct BodySpec {
    int archetype;            // PlanetArchetype, 0..5
    double massKg, surfaceTempK, coreTempK, spinOmegaRadS;
};
struct Sample {               // RadialProfileSample (engine/planet_builder.hpp:10-17)
    double r, rho, P, M, T;
    int mat;
};
struct BuildResult {
    double radiusM, massKg, pcPa;
    uint32_t tracerCount, profileCount, shellCount;
};
bool validSpec(const BodySpec& spec, std::string* err);
// Host only: PlanetBuilder::solveHydrostatic1D.
bool solveHydrostatic(const BodySpec& spec, std::vector<Sample>& profile, double& radiusM, double& pcPa,
                      std::string* err);
// PlanetBuilder::buildPlanet into particles [offset, offset + n) of p;
// blocks until the body is on the device.
cudaError_t buildOnDevice(const BodySpec& spec, uint32_t n, uint8_t bodyId, uint32_t gridRes, uint64_t seed,
                          const AstraeaParticles& p, uint32_t offset, DevStatus* status, uint32_t spinLimit,
                          cudaStream_t st, BuildResult* out, std::string* err);
}  // namespace planet

}  // namespace astraea_gb300
