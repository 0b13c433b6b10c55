// ref_sim_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference engine's own host code -- Simulation
// (engine/simulation.cpp) with its scenario loading, body relaxation
// (relaxLoadedSingleBody, :585-781), telemetry (computeTelemetryFromDevice,
// :948-1285, and sumDeviceRadPowerW, :567-582) and step driver (:1711-1753)
// -- on the CPU, so the library's device versions of those host loops can be
// checked against the engine's own code and golden outputs can be generated.
//
// Two stand-ins make that possible without a GPU:
//   * the handful of CUDA runtime calls the engine's host code makes
//     (cudaMalloc/cudaFree/cudaMemcpy/cudaMemset and their async and pinned
//     variants, device synchronisation, events) are defined here over host
//     memory: "device" arrays are host arrays, a copy is a memcpy, an event
//     holds a wall-clock time;
//   * the kernel interface astraea::cuda::* (engine/sph_gravity.cuh:57-92) is
//     served by the oracle (oracle/oracle.cpp), the CPU restatement of the
//     engine's kernels, through the C descriptors whose layout equals the
//     engine's structs (checked below).
// simulation.cpp is compiled from the reference checkout where it lies (the
// build recipe passes its directory as an include path); its private members
// are made reachable for the harness by the define around the class header.
// Built by oracle/build_oracle.py into oracle/_ref/ (never committed); the
// result links the oracle library and no CUDA library.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <limits>
#include <memory>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "astraea_gb300.h"

#define private public
#include "simulation.hpp"
#undef private
#include "simulation.cpp"

// ----------------------------------------------------------- oracle kernels
extern "C" {
void oracle_clear_stats(AstraeaParticles* p);
void oracle_sort_and_build(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* b, float* bounds6Out);
void oracle_sph_pass1(AstraeaParticles* p, const AstraeaRadixBvh* b);
void oracle_evaluate_eos(AstraeaParticles* p);
void oracle_gravity(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, uint64_t* interactionsOut);
void oracle_sph_pass2(AstraeaParticles* p, const AstraeaRadixBvh* b);
void oracle_kick_half(AstraeaParticles* p, float hdt, int clampThermal);
void oracle_drift(AstraeaParticles* p, float dt, const AstraeaRadixBvh* b, int useBvh);
float oracle_reduce_dt(const AstraeaParticles* p, float prevDt, float maxDt, float* rawMinOut);
void oracle_pack_render_records(const AstraeaParticles* p, uint8_t* rec20, uint8_t* speed, float sx, float sy,
                                float sz);
void oracle_extract_tracers(const AstraeaParticles* p, uint8_t* rec40, uint32_t tracerCount, float lx, float ly,
                            float lz, float sx, float sy, float sz);
}

// --------------------------------------------- CUDA runtime over host memory
struct CUevent_st {
    double seconds = 0.0;
};

namespace {
double wallSeconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

extern "C" {
cudaError_t cudaMalloc(void** p, size_t bytes) {
    *p = std::calloc(std::max<size_t>(bytes, 1), 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMallocHost(void** p, size_t bytes) { return cudaMalloc(p, bytes); }
cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned int) { return cudaMalloc(p, bytes); }
cudaError_t cudaFreeHost(void* p) { return cudaFree(p); }
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind) {
    if (bytes) std::memmove(dst, src, bytes);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, enum cudaMemcpyKind kind, cudaStream_t) {
    return cudaMemcpy(dst, src, bytes, kind);
}
cudaError_t cudaMemset(void* p, int value, size_t bytes) {
    if (bytes) std::memset(p, value, bytes);
    return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* p, int value, size_t bytes, cudaStream_t) { return cudaMemset(p, value, bytes); }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "host stand-in error"; }
cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = new CUevent_st();
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    delete e;
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
    e->seconds = wallSeconds();
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = static_cast<float>((b->seconds - a->seconds) * 1.0e3);
    return cudaSuccess;
}
}  // extern "C"

// ------------------------------------------ kernel interface on the oracle
namespace astraea::cuda {
namespace {

static_assert(sizeof(ParticleBuffersDevice) == sizeof(AstraeaParticles), "particle descriptor layout");
static_assert(offsetof(ParticleBuffersDevice, tracerIsOcean) == offsetof(AstraeaParticles, tracerIsOcean),
              "particle descriptor layout");
static_assert(sizeof(RadixBvhDevice) == sizeof(AstraeaRadixBvh), "BVH descriptor layout");
static_assert(offsetof(RadixBvhDevice, nodeMaxHPacked) == offsetof(AstraeaRadixBvh, nodeMaxHPacked),
              "BVH descriptor layout");

AstraeaParticles* P(ParticleBuffersDevice& p) { return reinterpret_cast<AstraeaParticles*>(&p); }
const AstraeaParticles* P(const ParticleBuffersDevice& p) { return reinterpret_cast<const AstraeaParticles*>(&p); }
AstraeaRadixBvh* B(RadixBvhDevice& b) { return reinterpret_cast<AstraeaRadixBvh*>(&b); }
const AstraeaRadixBvh* B(const RadixBvhDevice& b) { return reinterpret_cast<const AstraeaRadixBvh*>(&b); }

template <class T>
void alloc(T*& p, size_t n) {
    std::free(p);
    p = static_cast<T*>(std::calloc(std::max<size_t>(n, 1), sizeof(T)));
    if (p == nullptr) throw std::runtime_error("host stand-in: out of memory");
}
template <class T>
void release(T*& p) {
    std::free(p);
    p = nullptr;
}

}  // namespace

void RadixBvhDevice::allocate(uint32_t maxCapacity) {
    free();
    const size_t n = std::max<uint32_t>(maxCapacity, 1u), nodes = 2 * n - 1;
    capacity = static_cast<uint32_t>(n);
    alloc(mortonCodes, n); alloc(mortonCodesSorted, n); alloc(indicesIn, n); alloc(indicesSorted, n);
    alloc(leftChild, n); alloc(rightChild, n); alloc(parent, nodes); alloc(atomicVisited, n);
    alloc(aabbMinX, nodes); alloc(aabbMinY, nodes); alloc(aabbMinZ, nodes);
    alloc(aabbMaxX, nodes); alloc(aabbMaxY, nodes); alloc(aabbMaxZ, nodes);
    alloc(nodeMass, nodes); alloc(comX, nodes); alloc(comY, nodes); alloc(comZ, nodes); alloc(nodeMaxH, nodes);
    alloc(sceneBoundsOrdered, 6); alloc(sceneBoundsFloat, 6); alloc(livingFlags, 2);
    alloc(nodeComMass, nodes); alloc(nodeMinExtent, nodes); alloc(nodeMaxHPacked, nodes);
}
void RadixBvhDevice::free() {
    release(mortonCodes); release(mortonCodesSorted); release(indicesIn); release(indicesSorted);
    release(leftChild); release(rightChild); release(parent); release(atomicVisited);
    release(aabbMinX); release(aabbMinY); release(aabbMinZ); release(aabbMaxX); release(aabbMaxY); release(aabbMaxZ);
    release(nodeMass); release(comX); release(comY); release(comZ); release(nodeMaxH);
    release(sceneBoundsOrdered); release(sceneBoundsFloat); release(livingFlags);
    release(nodeComMass); release(nodeMinExtent); release(nodeMaxHPacked);
    capacity = 0;
}
void allocateRadixBvh(RadixBvhDevice& bvh, uint32_t capacity) { bvh.allocate(capacity); }
void freeRadixBvh(RadixBvhDevice& bvh) { bvh.free(); }

// Every array member of the particle descriptor, with its element size: the
// members after {capacity, count} are all pointers; the four u8 arrays have
// 1-byte elements, every other array 4-byte ones.
template <class F>
void forEachArray(AstraeaParticles& p, F&& f) {
    char* base = reinterpret_cast<char*>(&p);
    for (size_t off = offsetof(AstraeaParticles, posX); off + sizeof(void*) <= sizeof(AstraeaParticles);
         off += sizeof(void*)) {
        const bool bytes = off == offsetof(AstraeaParticles, materialId) || off == offsetof(AstraeaParticles, phaseId) ||
                           off == offsetof(AstraeaParticles, bodyId) ||
                           off == offsetof(AstraeaParticles, tracerIsOcean);
        f(*reinterpret_cast<void**>(base + off), bytes ? size_t{1} : size_t{4}, off);
    }
}

void allocateParticleBuffers(ParticleBuffersDevice& b, uint32_t capacity) {
    freeParticleBuffers(b);
    const size_t n = std::max<uint32_t>(capacity, 1u);
    forEachArray(*P(b), [&](void*& a, size_t elem, size_t) {
        a = std::calloc(n, elem);
        if (a == nullptr) throw std::runtime_error("host stand-in: out of memory");
    });
    for (size_t i = 0; i < n; ++i) b.tracerIndex[i] = -1;
    b.capacity = static_cast<uint32_t>(n);
    b.count = 0;
}
void freeParticleBuffers(ParticleBuffersDevice& b) {
    forEachArray(*P(b), [](void*& a, size_t, size_t) {
        std::free(a);
        a = nullptr;
    });
    b.capacity = 0;
    b.count = 0;
}

void launchClearStats(ParticleBuffersDevice& p) { oracle_clear_stats(P(p)); }
void launchSortAndBuildBvh(ParticleBuffersDevice& p, ParticleBuffersDevice& alt, RadixBvhDevice& bvh) {
    if (bvh.capacity < p.count) throw std::runtime_error("launchSortAndBuildBvh: BVH capacity < particle count");
    alt.count = p.count;
    oracle_sort_and_build(P(p), P(alt), B(bvh), nullptr);
}
void launchSphPass1Neighbors(ParticleBuffersDevice& p, const RadixBvhDevice& bvh) { oracle_sph_pass1(P(p), B(bvh)); }
void launchEvaluateEos(ParticleBuffersDevice& p) { oracle_evaluate_eos(P(p)); }
void launchGravityBarnesHut(ParticleBuffersDevice& p, const RadixBvhDevice& bvh, float theta) {
    oracle_gravity(P(p), B(bvh), theta, nullptr);
}
void launchSphPass2Forces(ParticleBuffersDevice& p, const RadixBvhDevice& bvh) { oracle_sph_pass2(P(p), B(bvh)); }
void launchLeapfrogKickHalf(ParticleBuffersDevice& p, float halfDtPsu, bool, bool clampThermal) {
    oracle_kick_half(P(p), halfDtPsu, clampThermal ? 1 : 0);   // includeXsph is unused by the engine (:1297)
}
void launchLeapfrogDrift(ParticleBuffersDevice& p, float dtPsu, const RadixBvhDevice& bvh) {
    const int useBvh = (bvh.capacity >= p.count && bvh.leftChild != nullptr && p.count >= 2u) ? 1 : 0;
    oracle_drift(P(p), dtPsu, B(bvh), useBvh);
}
float launchReduceDtPsu(const ParticleBuffersDevice& p, float prevDtPsu, float maxDtPsu) {
    return oracle_reduce_dt(P(p), prevDtPsu, maxDtPsu, nullptr);
}
void launchExtractTracers(const ParticleBuffersDevice& p, uint8_t* rec40, uint32_t tracerCount, uint32_t,
                          float livingComX, float livingComY, float livingComZ, float sysComX, float sysComY,
                          float sysComZ) {
    oracle_extract_tracers(P(p), rec40, tracerCount, livingComX, livingComY, livingComZ, sysComX, sysComY, sysComZ);
}
void launchPackRenderRecords(const ParticleBuffersDevice& p, uint8_t* rec20, uint8_t* speed, float sysComX,
                             float sysComY, float sysComZ) {
    oracle_pack_render_records(P(p), rec20, speed, sysComX, sysComY, sysComZ);
}

}  // namespace astraea::cuda

// -------------------------------------------------------------- C entry points
namespace {

thread_local std::string g_err;

// TelemetrySnapshot as a flat array of doubles, in this order.
constexpr int kTelemetryValues = 34;
void flatten(const astraea::TelemetrySnapshot& s, double* o) {
    const double v[kTelemetryValues] = {
        static_cast<double>(s.frameSeq), s.simTimeSec, static_cast<double>(s.dtSec), static_cast<double>(s.outcome),
        s.kineticEnergyJ, s.potentialEnergyJ, s.internalEnergyJ, s.radiatedEnergyJ, s.totalEnergyJ,
        s.initialTotalEnergyJ, s.energyDriftRel, s.momentumKgMS[0], s.momentumKgMS[1], s.momentumKgMS[2],
        s.angularMomentumKgM2S[0], s.angularMomentumKgM2S[1], s.angularMomentumKgM2S[2], s.virialRatio,
        s.maxTempK, s.maxPressureGPa, s.boundMassFrac, s.diskMassFrac, s.ejectaMassFrac, s.qRatioQrd,
        s.livingBodyComKm[0], s.livingBodyComKm[1], s.livingBodyComKm[2], s.livingBodyRadiusKm,
        s.livingBodySpinRadS, s.impactorComKm[0], s.impactorComKm[1], s.impactorComKm[2],
        static_cast<double>(s.particleCount), static_cast<double>(s.livingBodyPresent)};
    std::memcpy(o, v, sizeof(v));
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

}  // namespace

extern "C" {

int refsim_telemetry_values(void) { return kTelemetryValues; }
const char* refsim_last_error(void) { return g_err.c_str(); }

void* refsim_create(uint32_t maxParticles) {
    try {
        return new astraea::Simulation(maxParticles);
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}
void refsim_destroy(void* s) { delete static_cast<astraea::Simulation*>(s); }

// Simulation::loadScenario of a preset (makePresetConfig), with the
// relaxation steps of both bodies overridden when relaxSteps >= 0.
int refsim_load_preset(void* s, const char* preset, uint32_t particles, int relaxSteps, uint64_t seed) {
    return guarded([&] {
        astraea::CollisionScenarioConfig cfg =
            astraea::makePresetConfig(astraea::parsePresetName(preset), particles);
        if (relaxSteps >= 0) {
            cfg.target.relaxSteps = static_cast<uint32_t>(relaxSteps);
            cfg.impactor.relaxSteps = static_cast<uint32_t>(relaxSteps);
        }
        cfg.randomSeed = seed;
        static_cast<astraea::Simulation*>(s)->loadScenario(cfg);
    });
}

int refsim_step(void* s, double maxDtSec, double* telemetry) {
    return guarded([&] { flatten(static_cast<astraea::Simulation*>(s)->step(maxDtSec), telemetry); });
}

int refsim_compute_telemetry(void* s, double* telemetry) {
    return guarded([&] { flatten(static_cast<astraea::Simulation*>(s)->computeTelemetry(), telemetry); });
}

uint32_t refsim_count(void* s) { return static_cast<astraea::Simulation*>(s)->impl_->p.count; }

// Engine state the telemetry reads besides the particles, in this order:
// targetRadiusPsu, impactorRadiusPsu, livingBodyPresent, hasImpacted,
// qRatioQrd, impactParamB, impactVelocityRatioVesc, target spinOmegaRadS,
// frameSeq, simTimeSec, radiatedEnergyJ, initialTotalEnergyJ, the sum of
// sumDeviceRadPowerW.
constexpr int kContextValues = 13;
int refsim_context_values(void) { return kContextValues; }
void refsim_context(void* s, double* out) {
    auto& im = *static_cast<astraea::Simulation*>(s)->impl_;
    const double v[kContextValues] = {im.targetRadiusPsu, im.impactorRadiusPsu, im.livingBodyPresent ? 1.0 : 0.0,
                                      im.hasImpacted ? 1.0 : 0.0, im.qRatioQrd, im.config.impactParamB,
                                      im.config.impactVelocityRatioVesc, im.config.target.spinOmegaRadS,
                                      static_cast<double>(im.frameSeq), im.simTimeSec, im.radiatedEnergyJ,
                                      im.initialTotalEnergyJ, im.sumDeviceRadPowerW()};
    std::memcpy(out, v, sizeof(v));
}

// The particle arrays of the engine's state (host arrays of the descriptor
// in `out`, capacity >= count; every field copied).
int refsim_get_particles(void* s, AstraeaParticles* out) {
    return guarded([&] {
        astraea::ParticleBuffersDevice& p = static_cast<astraea::Simulation*>(s)->impl_->p;
        if (out->capacity < p.count) throw std::runtime_error("refsim_get_particles: capacity < count");
        const char* src = reinterpret_cast<const char*>(&p);
        astraea::cuda::forEachArray(*out, [&](void*& d, size_t elem, size_t off) {
            const void* a = *reinterpret_cast<void* const*>(src + off);
            if (d != nullptr && a != nullptr) std::memcpy(d, a, elem * p.count);
        });
        out->count = p.count;
    });
}

// Overwrites the engine's particle state (the count and every field given
// non-null in `in`) -- the state a telemetry reduction then runs on.
int refsim_set_particles(void* s, AstraeaParticles* in) {
    return guarded([&] {
        auto& im = *static_cast<astraea::Simulation*>(s)->impl_;
        im.ensureCapacity(std::max(in->count, 1u));
        astraea::ParticleBuffersDevice& p = im.p;
        char* dst = reinterpret_cast<char*>(&p);
        astraea::cuda::forEachArray(*in, [&](void*& a, size_t elem, size_t off) {
            void* d = *reinterpret_cast<void**>(dst + off);
            if (d != nullptr && a != nullptr) std::memcpy(d, a, elem * in->count);
        });
        p.count = in->count;
        im.alt.count = in->count;
    });
}

// relaxLoadedSingleBody (engine/simulation.cpp:585-781) on the body given in
// `body` (uploaded as the engine's uploadHostStateToDevice leaves it), with
// the anchor temperatures indexed by originalId; `body` receives the relaxed
// state, *vrmsOverVesc the engine's diagnostic.
int refsim_relax_loaded(void* s, AstraeaParticles* body, const double* anchorTempByOrigId, double nominalRadiusPsu,
                        uint32_t steps, double* vrmsOverVesc) {
    if (refsim_set_particles(s, body) != 0) return 1;
    return guarded([&] {
        auto& im = *static_cast<astraea::Simulation*>(s)->impl_;
        std::vector<double> anchors(anchorTempByOrigId, anchorTempByOrigId + body->count);
        im.relaxLoadedSingleBody(anchors, nominalRadiusPsu, steps, *vrmsOverVesc);
        if (refsim_get_particles(s, body) != 0) throw std::runtime_error(g_err);
    });
}

// Engine context of a telemetry reduction on a state set by refsim_set_particles.
void refsim_set_context(void* s, double targetRadiusPsu, int livingBodyPresent) {
    auto& im = *static_cast<astraea::Simulation*>(s)->impl_;
    im.targetRadiusPsu = targetRadiusPsu;
    im.livingBodyPresent = livingBodyPresent != 0;
}

}  // extern "C"
