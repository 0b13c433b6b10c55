// sph_gravity_gb300.cpp -- drop-in replacement of engine/sph_gravity.cu.
//
// Built inside the ASTRAEA engine's tree in place of engine/sph_gravity.cu
// (the sim_engine target of CMakeLists.txt:18-24), with the engine's own
// headers on the include path and include/astraea_gb300.h of this
// repository.  It defines every function the engine declares in
// engine/sph_gravity.cuh:57-92, with the same C++ names and signatures, and
// forwards each one to the C-ABI of libastraea_gb300.  A non-OK status is
// thrown as std::runtime_error, as ASTRAEA_CUDA_CHECK does
// (engine/sph_gravity.cuh:12-22).  The engine's structs are passed by
// address: the C structs of the ABI have their member order and types
// (checked below).
#include <cstddef>
#include <stdexcept>
#include <string>

#include "astraea_gb300.h"
#include "sph_gravity.cuh"

namespace astraea::cuda {
namespace {

static_assert(sizeof(ParticleBuffersDevice) == sizeof(AstraeaParticles), "particle descriptor layout");
static_assert(offsetof(ParticleBuffersDevice, posX) == offsetof(AstraeaParticles, posX), "particle descriptor layout");
static_assert(offsetof(ParticleBuffersDevice, tracerIsOcean) == offsetof(AstraeaParticles, tracerIsOcean),
              "particle descriptor layout");
static_assert(sizeof(RadixBvhDevice) == sizeof(AstraeaRadixBvh), "BVH descriptor layout");
static_assert(offsetof(RadixBvhDevice, cubTempBytes) == offsetof(AstraeaRadixBvh, cubTempBytes), "BVH descriptor layout");
static_assert(offsetof(RadixBvhDevice, nodeMaxHPacked) == offsetof(AstraeaRadixBvh, nodeMaxHPacked),
              "BVH descriptor layout");

inline AstraeaParticles* P(ParticleBuffersDevice& p) { return reinterpret_cast<AstraeaParticles*>(&p); }
inline const AstraeaParticles* P(const ParticleBuffersDevice& p) {
    return reinterpret_cast<const AstraeaParticles*>(&p);
}
inline AstraeaRadixBvh* B(RadixBvhDevice& b) { return reinterpret_cast<AstraeaRadixBvh*>(&b); }
inline const AstraeaRadixBvh* B(const RadixBvhDevice& b) { return reinterpret_cast<const AstraeaRadixBvh*>(&b); }

inline void check(AstraeaStatus s) {
    if (s != ASTRAEA_OK) throw std::runtime_error(std::string("astraea_gb300: ") + astraea_gb300_last_error());
}

}  // namespace

void RadixBvhDevice::allocate(uint32_t maxCapacity) { check(astraea_gb300_allocate_radix_bvh(B(*this), maxCapacity)); }
void RadixBvhDevice::free() { check(astraea_gb300_free_radix_bvh(B(*this))); }

void allocateRadixBvh(RadixBvhDevice& bvh, uint32_t capacity) { check(astraea_gb300_allocate_radix_bvh(B(bvh), capacity)); }
void freeRadixBvh(RadixBvhDevice& bvh) { check(astraea_gb300_free_radix_bvh(B(bvh))); }
void allocateParticleBuffers(ParticleBuffersDevice& buffers, uint32_t capacity) {
    check(astraea_gb300_allocate_particle_buffers(P(buffers), capacity));
}
void freeParticleBuffers(ParticleBuffersDevice& buffers) { check(astraea_gb300_free_particle_buffers(P(buffers))); }
void launchClearStats(ParticleBuffersDevice& p) { check(astraea_gb300_clear_stats(P(p))); }

void launchSortAndBuildBvh(ParticleBuffersDevice& p, ParticleBuffersDevice& alt, RadixBvhDevice& bvh) {
    check(astraea_gb300_sort_and_build_bvh(P(p), P(alt), B(bvh)));
}
void launchSphPass1Neighbors(ParticleBuffersDevice& p, const RadixBvhDevice& bvh) {
    check(astraea_gb300_sph_pass1_neighbors(P(p), B(bvh)));
}
void launchEvaluateEos(ParticleBuffersDevice& p) { check(astraea_gb300_evaluate_eos(P(p))); }
void launchGravityBarnesHut(ParticleBuffersDevice& p, const RadixBvhDevice& bvh, float theta) {
    check(astraea_gb300_gravity_barnes_hut(P(p), B(bvh), theta));
}
void launchSphPass2Forces(ParticleBuffersDevice& p, const RadixBvhDevice& bvh) {
    check(astraea_gb300_sph_pass2_forces(P(p), B(bvh)));
}
void launchLeapfrogKickHalf(ParticleBuffersDevice& p, float halfDtPsu, bool includeXsph, bool clampThermal) {
    check(astraea_gb300_leapfrog_kick_half(P(p), halfDtPsu, includeXsph ? 1 : 0, clampThermal ? 1 : 0));
}
void launchLeapfrogDrift(ParticleBuffersDevice& p, float dtPsu, const RadixBvhDevice& bvh) {
    check(astraea_gb300_leapfrog_drift(P(p), dtPsu, B(bvh)));
}
float launchReduceDtPsu(const ParticleBuffersDevice& p, float prevDtPsu, float maxDtPsu) {
    float dt = 0.0f;
    check(astraea_gb300_reduce_dt_psu(P(p), prevDtPsu, maxDtPsu, &dt));
    return dt;
}
void launchExtractTracers(const ParticleBuffersDevice& p, uint8_t* d_tracerRecords40B, uint32_t tracerCount,
                          uint32_t tracerGridRes, float livingComX, float livingComY, float livingComZ, float sysComX,
                          float sysComY, float sysComZ) {
    check(astraea_gb300_extract_tracers(P(p), d_tracerRecords40B, tracerCount, tracerGridRes, livingComX, livingComY,
                                        livingComZ, sysComX, sysComY, sysComZ));
}
void launchPackRenderRecords(const ParticleBuffersDevice& p, uint8_t* d_particleRecords20B, uint8_t* d_speedBytes,
                             float sysComX, float sysComY, float sysComZ) {
    check(astraea_gb300_pack_render_records(P(p), d_particleRecords20B, d_speedBytes, sysComX, sysComY, sysComZ));
}

}  // namespace astraea::cuda
