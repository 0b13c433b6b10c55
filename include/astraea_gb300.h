/*
 * astraea_gb300.h -- C-ABI of the GB300-native ASTRAEA per-step physics path.
 *
 * Every entry point here replaces one function of the ASTRAEA engine's kernel
 * interface `astraea::cuda::*` declared in engine/sph_gravity.cuh:61-92 and
 * implemented in engine/sph_gravity.cu.  The structs mirror the engine's
 * particle SoA descriptor `astraea::ParticleBuffersDevice`
 * (engine/types.hpp:114-161) and `astraea::cuda::RadixBvhDevice`
 * (engine/sph_gravity.cuh:26-59) field for field, so a caller can pass the
 * engine's own structs by pointer (the C++ shim in
 * astraea-impact-sim_gb300/csrc/shim does exactly that).
 *
 * Conventions
 *   - Every function returns an AstraeaStatus; 0 is success.  On failure
 *     astraea_gb300_last_error() returns a message (thread-local).
 *   - Work is enqueued on the stream set by astraea_gb300_set_stream
 *     (default: the legacy default stream, as the engine uses).
 *   - count == 0 is a no-op for every launch, as in the engine.
 *   - Pointers are device pointers unless a parameter says "host".
 */
#ifndef ASTRAEA_GB300_H
#define ASTRAEA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASTRAEA_GB300_ABI_VERSION 1

typedef enum AstraeaStatus {
    ASTRAEA_OK = 0,
    ASTRAEA_ERR_CUDA = 1,          /* a CUDA runtime call failed */
    ASTRAEA_ERR_CAPACITY = 2,      /* buffers smaller than the particle count */
    ASTRAEA_ERR_INVALID = 3,       /* bad argument (null pointer, bad size) */
    ASTRAEA_ERR_DEVICE_TIMEOUT = 4,/* a bounded device-side wait gave up */
    ASTRAEA_ERR_DEVICE_STATE = 5   /* device status word reported a fault */
} AstraeaStatus;

typedef struct AstraeaFloat4 { float x, y, z, w; } AstraeaFloat4;

/* Particle SoA; same member order and types as ParticleBuffersDevice
 * (engine/types.hpp:114-161): 2 x u32 then 56 device pointers. */
typedef struct AstraeaParticles {
    uint32_t capacity;
    uint32_t count;
    float* posX;      float* posY;      float* posZ;
    float* velX;      float* velY;      float* velZ;
    float* velHalfX;  float* velHalfY;  float* velHalfZ;
    float* accX;      float* accY;      float* accZ;
    float* mass;
    float* h;
    float* h0;
    float* rho;
    float* drhoDt;
    float* pressure;
    float* soundSpeed;
    float* u;
    float* duDt;
    float* tempK;
    float* radPowerW;
    float* sXX; float* sYY; float* sZZ;
    float* sXY; float* sXZ; float* sYZ;
    float* dSXX; float* dSYY; float* dSZZ;
    float* dSXY; float* dSXZ; float* dSYZ;
    float* damage;
    float* damageCbrt;
    float* dDamageCbrtDt;
    float* epsFail;
    float* divV;
    float* curlVX; float* curlVY; float* curlVZ;
    float* shepardC;
    float* surfFactor;
    float* phiGrav;
    uint8_t*  materialId;
    uint8_t*  phaseId;
    uint8_t*  bodyId;
    uint32_t* originalId;
    int32_t*  tracerIndex;
    float* tracerRestRadiusPsu;
    float* tracerRestNormalX;
    float* tracerRestNormalY;
    float* tracerRestNormalZ;
    uint8_t* tracerIsOcean;
} AstraeaParticles;

/* Linear BVH descriptor; same member order and types as RadixBvhDevice
 * (engine/sph_gravity.cuh:26-59).  Internal nodes are [0, N-2], leaves are
 * node-array entries [N-1, 2N-2]; a child value < 0 encodes leaf ~child. */
typedef struct AstraeaRadixBvh {
    uint32_t  capacity;
    uint64_t* mortonCodes;
    uint64_t* mortonCodesSorted;
    uint32_t* indicesIn;
    uint32_t* indicesSorted;
    int32_t*  leftChild;
    int32_t*  rightChild;
    int32_t*  parent;
    uint32_t* atomicVisited;
    float* aabbMinX; float* aabbMinY; float* aabbMinZ;
    float* aabbMaxX; float* aabbMaxY; float* aabbMaxZ;
    float* nodeMass;
    float* comX; float* comY; float* comZ;
    float* nodeMaxH;
    void*  cubTempStorage;   /* unused by this library; kept for layout */
    size_t cubTempBytes;     /* unused by this library; kept for layout */
    uint32_t* sceneBoundsOrdered;
    float*    sceneBoundsFloat;
    uint32_t* livingFlags;
    AstraeaFloat4* nodeComMass;     /* {comX, comY, comZ, mass}  */
    AstraeaFloat4* nodeMinExtent;   /* {minX, minY, minZ, dNode} */
    AstraeaFloat4* nodeMaxHPacked;  /* {maxX, maxY, maxZ, maxH}  */
} AstraeaRadixBvh;

/* ---- library / runtime ------------------------------------------------ */

/* Thread-local message for the last non-OK status (never NULL). */
const char* astraea_gb300_last_error(void);
/* ABI version of the loaded library (ASTRAEA_GB300_ABI_VERSION). */
int astraea_gb300_abi_version(void);
/* Stream for all subsequent launches from any thread (a cudaStream_t, or
 * NULL for the legacy default stream, which is the engine's behaviour). */
AstraeaStatus astraea_gb300_set_stream(void* stream);

/* ---- allocation (engine/sph_gravity.cu:1806-1984) ---------------------- */

/* Replaces allocateRadixBvh (engine/sph_gravity.cu:1806-1855). */
AstraeaStatus astraea_gb300_allocate_radix_bvh(AstraeaRadixBvh* bvh, uint32_t capacity);
/* Replaces freeRadixBvh (engine/sph_gravity.cu:1857-1893). */
AstraeaStatus astraea_gb300_free_radix_bvh(AstraeaRadixBvh* bvh);
/* Replaces allocateParticleBuffers (engine/sph_gravity.cu:1895-1941). */
AstraeaStatus astraea_gb300_allocate_particle_buffers(AstraeaParticles* p, uint32_t capacity);
/* Replaces freeParticleBuffers (engine/sph_gravity.cu:1943-1984). */
AstraeaStatus astraea_gb300_free_particle_buffers(AstraeaParticles* p);

/* ---- the per-step stages (engine/sph_gravity.cu:1988-2161) -------------- */

/* Replaces launchClearStats (engine/sph_gravity.cu:1988-1994). */
AstraeaStatus astraea_gb300_clear_stats(AstraeaParticles* p);
/* Replaces launchSortAndBuildBvh (engine/sph_gravity.cu:1996-2061): scene
 * AABB, 63-bit Morton codes, stable radix sort (value = original index),
 * 56-field permutation into alt, pointer swap p<->alt (both structs are
 * modified), Karras LBVH, bottom-up refit. */
AstraeaStatus astraea_gb300_sort_and_build_bvh(AstraeaParticles* p, AstraeaParticles* alt,
                                               AstraeaRadixBvh* bvh);
/* Replaces launchSphPass1Neighbors (engine/sph_gravity.cu:2063-2074). */
AstraeaStatus astraea_gb300_sph_pass1_neighbors(AstraeaParticles* p, const AstraeaRadixBvh* bvh);
/* Replaces launchEvaluateEos (engine/sph_gravity.cu:2076-2083). */
AstraeaStatus astraea_gb300_evaluate_eos(AstraeaParticles* p);
/* Replaces launchGravityBarnesHut (engine/sph_gravity.cu:2085-2097). */
AstraeaStatus astraea_gb300_gravity_barnes_hut(AstraeaParticles* p, const AstraeaRadixBvh* bvh,
                                               float theta);
/* Replaces launchSphPass2Forces (engine/sph_gravity.cu:2099-2111). */
AstraeaStatus astraea_gb300_sph_pass2_forces(AstraeaParticles* p, const AstraeaRadixBvh* bvh);
/* Replaces launchLeapfrogKickHalf (engine/sph_gravity.cu:2113-2120). */
AstraeaStatus astraea_gb300_leapfrog_kick_half(AstraeaParticles* p, float halfDtPsu,
                                               int includeXsph, int clampThermal);
/* Replaces launchLeapfrogDrift (engine/sph_gravity.cu:2122-2134).  Unlike the
 * engine kernel (which reads neighbour positions while other threads move
 * them), neighbours are read from the pre-drift positions. */
AstraeaStatus astraea_gb300_leapfrog_drift(AstraeaParticles* p, float dtPsu,
                                           const AstraeaRadixBvh* bvh);
/* Replaces launchReduceDtPsu (engine/sph_gravity.cu:2136-2161); blocks until
 * the result is on the host and writes it to *outDtPsu (host pointer).  Also
 * returns ASTRAEA_ERR_DEVICE_TIMEOUT when a bounded device wait gave up since
 * the last astraea_gb300_reset_device_status. */
AstraeaStatus astraea_gb300_reduce_dt_psu(const AstraeaParticles* p, float prevDtPsu,
                                          float maxDtPsu, float* outDtPsu);

/* Rounding of the node masses and COMs of every later tree build (stage
 * calls and the fused step).  0 (default): from exact fixed-point moment sums
 * (each node's COM is the correctly rounded quotient of its exact sums; the
 * engine's FP32 combination can place the COM of coincident particles off
 * them).  1: the engine's own FP32 bottom-up combination
 * (bottomUpBvhMomentsKernel, engine/sph_gravity.cu:531-621, with its
 * multiply-add contracted as nvcc contracts it), bit-identical to the
 * engine's node data, so the gravity walk takes exactly the engine's opening
 * decisions.  Boxes, h extremes and quadrupole moments do not depend on it.
 * Process-wide. */
AstraeaStatus astraea_gb300_set_node_rounding(int mode);

/* ---- far-field correction (no counterpart in the engine) ---------------- */

/* Far-field model of every later tree build and gravity evaluation (stage
 * calls and the fused step): 0 = monopole, the engine's
 * gravityBarnesHutKernel (engine/sph_gravity.cu:810-961), the default;
 * 1 = monopole + quadrupole: the build also refits every node's central
 * second moments and each accepted node adds its quadrupole acceleration
 * and potential, so a larger opening angle (0.7 instead of 0.5) gives the
 * same force error with about half the interactions; 2 = monopole + the
 * learned far-field correction (astraea_gb300_ff_*, below); 3 = the
 * quadrupole walk with leaf buckets and the group expansion
 * (astraea_gb300_set_far_field_expansion).  Process-wide; gravity in modes
 * 1-3 on a tree built in mode 0 returns ASTRAEA_ERR_INVALID. */
AstraeaStatus astraea_gb300_set_far_field(int mode);
/* Far-field mode 3.  The walk is mode 1's (the engine's opening test at
 * theta over groups of 32, quadrupole terms), with two changes: an opened
 * node of at most `leafBucket` particles (0..32; 0 = off) is not descended,
 * its sorted leaf range is evaluated particle-particle; an accepted node far
 * against the group (group radius about its box centre c <= gamma
 * |c - COM|) is not evaluated by every member but added to the group's
 * expansion -- its field and potential at c (monopole + quadrupole, Plummer
 * softening with the group's mean eps^2) and the monopole's first and second
 * derivatives there -- from which each member takes its second-order Taylor
 * value.  Defaults 16 and 0.3; gamma in [0, 1).  Interaction counts:
 * ASTRAEA_COUNTER_GRAVITY_GROUP_EVALS (expansion terms, not in
 * ASTRAEA_COUNTER_GRAVITY_INTERACTIONS) and ..._BUCKET_LEAVES (P-P terms from
 * buckets, included).  No engine counterpart. */
AstraeaStatus astraea_gb300_set_far_field_expansion(uint32_t leafBucket, float gamma);
/* The leaf bucket of far-field mode 3 picked by timing: the mode-3 gravity
 * of the current tree (built in mode 3) at theta with the current gamma is
 * timed (best of 3, CUDA events) for each of `count` candidate bucket sizes
 * (<= 32); the fastest becomes the mode's bucket and *outBucket, outMs
 * (host, optional) receives each candidate's time.  Buckets only add exact
 * particle-particle terms in place of node terms, so no candidate is less
 * accurate than a smaller one.  Blocks; no engine counterpart. */
AstraeaStatus astraea_gb300_autotune_expansion(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                               const uint32_t* candidates, uint32_t count, uint32_t* outBucket,
                                               float* outMs);

/* ---- render frame packing (engine/sph_gravity.cu:1554-1743, 2163-2201) -- */

/* Replaces launchPackRenderRecords (engine/sph_gravity.cu:2189-2201): one
 * 20-byte ParticleRecordPacked per particle (position in km relative to the
 * system COM, log-quantised temperature, pressure and radius, material,
 * phase|body, damage) into records20 (device, any alignment), and one
 * log-quantised speed byte per particle into speedBytes when it is not NULL.
 * count == 0 or records20 == NULL is a no-op. */
AstraeaStatus astraea_gb300_pack_render_records(const AstraeaParticles* p, uint8_t* records20, uint8_t* speedBytes,
                                                float sysComX, float sysComY, float sysComZ);
/* Replaces launchExtractTracers (engine/sph_gravity.cu:2163-2187): zeroes
 * tracerCount 40-byte CrustTracerRecordPacked records, then writes one for
 * every particle whose tracerIndex is in [0, tracerCount).  tracerGridRes is
 * unused, as in the engine.  tracerCount == 0 or records40 == NULL is a no-op. */
AstraeaStatus astraea_gb300_extract_tracers(const AstraeaParticles* p, uint8_t* records40, uint32_t tracerCount,
                                            uint32_t tracerGridRes, float livingComX, float livingComY,
                                            float livingComZ, float sysComX, float sysComY, float sysComZ);

/* Uncompressed PCLS frame (server/binary_protocol.hpp:11-59): the fields of
 * the 40-byte header that come from the telemetry snapshot, and the COMs the
 * two packing kernels take.  No engine counterpart as one call: the engine
 * packs on the device, copies three arrays to the host and assembles the
 * frame there (engine/simulation.cpp:1810-1860, binary_protocol.cpp:155-217). */
typedef struct AstraeaPclsFrameInfo {
    double   simTimeSec;
    uint64_t frameSeq;          /* low 32 bits go into the header */
    float    dtSec;
    uint32_t tracerCount;
    uint32_t tracerGridRes;
    int32_t  livingBodyPresent;
    int32_t  withSpeed;         /* append the speed-byte array */
    float    livingCom[3];
    float    sysCom[3];
} AstraeaPclsFrameInfo;
/* Bytes of the uncompressed frame: 40 + 20 N + 40 T (+ N with speed). */
AstraeaStatus astraea_gb300_pcls_frame_bytes(uint32_t particleCount, uint32_t tracerCount, int withSpeed,
                                             size_t* outBytes);
/* Writes header, particle records, tracer records and speed bytes of one
 * frame into `frame` (device, frameCapacity bytes); *outFrameBytes (host, may
 * be NULL) receives its size.  Byte-identical to buildBinaryFrame with
 * compressZlib = false on the same records; zlib stays a host step. */
AstraeaStatus astraea_gb300_pack_pcls_frame(const AstraeaParticles* p, const AstraeaPclsFrameInfo* info,
                                            uint8_t* frame, size_t frameCapacity, size_t* outFrameBytes);

/* ---- per-frame telemetry on the device (engine/simulation.cpp:567-582, 948-1285) */

/* Engine state the telemetry loops read besides the particles. */
typedef struct AstraeaTelemetryParams {
    double  targetRadiusPsu;      /* Simulation::Impl::targetRadiusPsu */
    int32_t livingBodyPresent;    /* compute the living-body spin sums */
    int32_t reserved;
} AstraeaTelemetryParams;

/* Results of the O(N) loops of computeTelemetryFromDevice and
 * sumDeviceRadPowerW, in PSU (FP64).  The engine's remaining scalar code
 * (unit conversion, energy drift, spin = spinL / spinI / T_UNIT_S, mass
 * fractions, the collision-outcome rules) runs on the host from these. */
typedef struct AstraeaTelemetry {
    double   totalMassPsu;
    double   sysComPsu[3];
    double   massBody0Psu, comBody0Psu[3], velBody0Psu[3];   /* bodyId == 0 (COM / mean velocity if mass > 0) */
    double   massOtherPsu, comOtherPsu[3], velOtherPsu[3];   /* bodyId != 0 */
    double   livingComPsu[3];                              /* body-0 COM, else the system COM */
    double   kineticPsu, potentialPsu, internalPsu;         /* sum 1/2 m v^2, 1/2 m phi, m u */
    double   momentumPsu[3], angularMomentumPsu[3];
    double   maxTempK, maxPressureGPa, maxDamage;
    double   radiatedPowerW;                                /* sum of finite positive radPowerW */
    double   spinLPsu, spinIPsu;                            /* lSpinY, I_yy of the living body */
    double   remnantPsu[3], remnantVelPsu[3], remnantMassPsu, remnantRadiusPsu;
    double   boundPlanetMassPsu, diskMassPsu, ejectaMassPsu, impactorBoundMassPsu;
    uint32_t remnantSeedIndex;                              /* particle of lowest finite phiGrav (first) */
    int32_t  remnantIterations;                             /* remnant updates made (0..5) */
} AstraeaTelemetry;

/* Replaces the host loops of computeTelemetryFromDevice and
 * sumDeviceRadPowerW: seven FP64 reduction passes on the device, one 392-byte
 * copy to *out (host).  Blocks until the result is on the host.  Allocates
 * nothing (its scratch is fixed device memory); calls must not overlap on
 * the GPU.  count == 0 zeroes *out. */
AstraeaStatus astraea_gb300_reduce_telemetry(const AstraeaParticles* p, const AstraeaTelemetryParams* params,
                                             AstraeaTelemetry* out);

/* ---- body relaxation (engine/simulation.cpp:585-781) -------------------- */

/* Replaces Simulation::Impl::relaxLoadedSingleBody: the initial forces, then
 * `steps` damped steps (dt bound 0.02 PSU, thermal clamp on) each followed by
 * COM/bulk-velocity removal, 0.85 velocity damping, u re-anchored to
 * u_cold(rho) + c_v T_anchor(originalId) and stresses/damage cleared, then 4
 * undamped diagnostic steps; *outFinalVrmsOverVesc (host) receives
 * v_rms / v_esc of the result, and u / strength are re-anchored once more.
 * anchorTempByOrigId: device array of anchorCount temperatures [K] indexed by
 * originalId (NULL: 288 K for all, the engine's fallback).  The engine copies
 * ten arrays to the host and back every iteration; here the recentring runs
 * on the device.  Blocks until done. */
AstraeaStatus astraea_gb300_relax_single_body(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh,
                                              const double* anchorTempByOrigId, uint32_t anchorCount,
                                              double nominalRadiusPsu, uint32_t steps, double* outFinalVrmsOverVesc);

/* ---- planet construction (engine/planet_builder.cpp:398-905) ------------ */

/* BodyInitSpec (engine/types.hpp:60-67). */
typedef struct AstraeaBodySpec {
    uint32_t archetype;      /* PlanetArchetype: 0 LivingTerra, 1 IronCore, 2 OceanIce,
                                3 LavaIo, 4 GasGiant, 5 ProtoTheia */
    uint32_t relaxSteps;     /* carried for the caller; the builder ignores it */
    double massKg;
    double surfaceTempK;
    double coreTempK;
    double spinOmegaRadS;
} AstraeaBodySpec;

/* RadialProfileSample (engine/planet_builder.hpp:10-17). */
typedef struct AstraeaRadialSample {
    double rM;
    double rhoKgM3;
    double pressurePa;
    double enclosedMassKg;
    double tempK;
    uint32_t material;       /* MaterialId */
    uint32_t reserved;
} AstraeaRadialSample;

/* The scalar members of BuiltPlanetHost (engine/planet_builder.hpp:19-34). */
typedef struct AstraeaPlanetInfo {
    double equatorialRadiusM;
    double actualMassKg;     /* enclosed mass of the last profile sample */
    double centralPressurePa;
    uint32_t tracerCount;
    uint32_t profileSamples;
    uint32_t shells;         /* particle shells placed */
    uint32_t reserved;
} AstraeaPlanetInfo;

/* PlanetBuilder::solveHydrostatic1D: RK4 shooting outward from the centre
 * with bisection on log P_c, on the host, no GPU work; thread-safe.  The
 * profile is bit-identical to the engine's.  *outCount receives the sample
 * count; a NULL profile or too small capacity returns ASTRAEA_ERR_CAPACITY
 * with nothing written to profile.  massKg <= 0 or archetype > 5:
 * ASTRAEA_ERR_INVALID (the engine throws std::invalid_argument). */
AstraeaStatus astraea_gb300_solve_hydrostatic(const AstraeaBodySpec* spec, AstraeaRadialSample* profile,
                                              uint32_t capacity, uint32_t* outCount, double* outRadiusM,
                                              double* outCentralPressurePa);

/* PlanetBuilder::buildPlanet followed by the engine's upload of that body
 * (engine/simulation.cpp:468-523, 852-880), as one call that writes the
 * body straight into particles [offset, offset + particleCount) of p: the
 * hydrostatic profile and shell plan on the host (bit-identical to the
 * engine's), the engine's mt19937_64 stream drawn on the host and shipped
 * in pinned chunks, particle placement and the LivingTerra surface-tracer
 * selection (tracerGridRes > 0, 6 G^2 bins) on the device.  Written: pos,
 * vel and velHalf (= vel), mass, h = h0, h0, rho, u, tempK, epsFail,
 * materialId, bodyId, originalId = offset + i, the tracer fields; zeroed:
 * stresses, damage, damageCbrt, pressure, soundSpeed, phaseId.  p->count is
 * not changed.  particleCount == 0 or massKg <= 0: ASTRAEA_ERR_INVALID (the
 * engine throws); offset + particleCount > p->capacity: ASTRAEA_ERR_CAPACITY.
 * Blocks until the body is on the device. */
AstraeaStatus astraea_gb300_build_planet(const AstraeaBodySpec* spec, uint32_t particleCount, uint32_t bodyId,
                                         uint32_t tracerGridRes, uint64_t seed, AstraeaParticles* p, uint32_t offset,
                                         AstraeaPlanetInfo* info);

/* ---- far-field mode 2: learned correction (no engine counterpart) ------- */

/* In mode 2 (astraea_gb300_set_far_field(2); trees built in that mode carry
 * second moments) the gravity walk keeps the engine's theta test and also
 * takes a node the theta test opens when every member of the group of 32
 * passes theta_far and the node is far against the group (L1 group extent
 * <= gamma r).  For each such (group, node) pair an MLP (16 -> 64 -> 64 ->
 * 12, SiLU, BF16 tensor-core arithmetic with FP32 accumulation) predicts the
 * residual between the node's exact field and its monopole at the group
 * centre c, and the residual's Jacobian; member i adds the sum over its
 * group's pairs of R + J (x_i - c).  Features: (COM - c)/r, dNode/r,
 * S/(M dNode^2) (central second moments), group extent/r.  With
 * gateTolerance > 0 every mode-2 gravity call checks the RMS relative error
 * of gateTargets sampled particles against a direct sum (gateFp64Pairs 0:
 * FP32 pair terms with FP64 sums, ~1e-6 relative of the FP64 sum, the
 * default; 1: FP64 pair terms, about twenty times the cost on this part) and,
 * above the tolerance, recomputes plain theta gravity; the decision is taken
 * on the device (the plain walk is always launched and returns at once when
 * the check passed), so the call does not block and can be graph-captured. */
typedef struct AstraeaFarFieldConfig {
    float thetaFar;          /* opening angle of the far test (default 0.8) */
    float gamma;             /* far test: L1 group extent <= gamma r (default 0.3) */
    float gateTolerance;     /* RMS relative force error at the gate; 0: no gate (default) */
    uint32_t gateTargets;    /* sampled particles of the gate (default 64, at most 1024) */
    uint32_t pairsPerGroup;  /* pair buffer per group of 32 (default 64); a full buffer opens the node */
    uint32_t gateFp64Pairs;  /* 0: FP32 pair terms, FP64 sums (default); 1: FP64 pair terms */
} AstraeaFarFieldConfig;

/* The pair records, corrections and gate state of mode 2 are kept per BVH
 * (created by its first mode-2 gravity call, which must come before any
 * stream capture), so several instances can step in mode 2 concurrently, on
 * their own streams or as branches of one graph, each gated on its own
 * spot check.  The network and the configuration are shared. */
typedef struct AstraeaFarFieldStats {
    uint64_t calls;          /* mode-2 gravity evaluations */
    uint64_t fallbacks;      /* ... that the gate sent back to the plain walk (all BVHs of the device) */
    uint32_t lastPairs;      /* (group, node) pairs corrected by the last gated call */
    uint32_t reserved;
    float lastGateRms;       /* RMS relative error of the last gate; -1 when no gate ran */
    float lastLoss;          /* loss of the last train step or gradient evaluation */
} AstraeaFarFieldStats;

AstraeaStatus astraea_gb300_ff_configure(const AstraeaFarFieldConfig* cfg);
/* Training rows from the current tree (built in mode 2): runs the mode-2
 * walk at theta (p's accelerations are overwritten with its monopole-only
 * result), with the far test on every groupStride-th group, and writes for
 * up to `capacity` recorded pairs 16 features and 16 labels (12 used: the
 * residual and Jacobian, normalised by G M / r^2 and G M / r^3, from an FP64
 * direct sum over the node's particles) to device arrays.  *outCount
 * receives the rows written. */
AstraeaStatus astraea_gb300_ff_collect(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                       uint32_t groupStride, float* features, float* labels, uint32_t capacity,
                                       uint32_t* outCount);
/* Network parameters: Xavier-uniform weights from `seed`, zero biases,
 * fresh Adam state.  6,288 FP32 parameters: W1 (16x64, in-major), b1, W2
 * (64x64), b2, W3 (64x16), b3. */
AstraeaStatus astraea_gb300_ff_init(uint64_t seed);
/* Per-output scale = RMS of the labels (device, count x 16). */
AstraeaStatus astraea_gb300_ff_fit_output_scale(const float* labels, uint32_t count);
/* Loss (mean squared error of the 12 used outputs in scaled units) and its
 * gradient over `count` rows (device arrays) by the tensor-core forward and
 * backward kernels; outGrads (host, 6,288 floats) may be NULL.  Blocks. */
AstraeaStatus astraea_gb300_ff_gradients(const float* features, const float* labels, uint32_t count,
                                         float* outGrads, float* outLoss);
/* One Adam step (beta 0.9 / 0.999) on the gradient of `count` rows;
 * *outLoss (host, may be NULL: no sync) receives the batch loss. */
AstraeaStatus astraea_gb300_ff_train_step(const float* features, const float* labels, uint32_t count,
                                          float learningRate, float* outLoss);
/* Network outputs (scaled units, count x 16, device) of `count` feature rows. */
AstraeaStatus astraea_gb300_ff_predict(const float* features, uint32_t count, float* out);
/* Host copies of the 6,288 parameters and the 16 output scales. */
AstraeaStatus astraea_gb300_ff_get_params(float* params, uint32_t capacity, float* outScale16);
AstraeaStatus astraea_gb300_ff_set_params(const float* params, uint32_t count, const float* outScale16);
/* Synchronises the device; lastPairs and lastGateRms are those of the last
 * mode-2 gravity call's BVH. */
AstraeaStatus astraea_gb300_ff_stats(AstraeaFarFieldStats* out);
/* One far-field mode-2 gravity call (current mode must be 2, tree built in
 * it) with CUDA events between its parts; outMs5 (host) receives the times of
 * the walk with its pair records, the network on the recorded pairs, the
 * per-member correction, the FP64 spot check of the gate (0 without a gate)
 * and the fallback walk (returns at once when the gate passed).  Blocks. */
AstraeaStatus astraea_gb300_ff_profile(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta, float* outMs5);

/* ---- fused step (no counterpart function in sph_gravity.cuh) ----------- */

/* One Simulation::step() kernel sequence (engine/simulation.cpp:1711-1753):
 * reduce-dt, kick(dt/2), drift, sort+build, pass 1, EOS, gravity(theta),
 * pass 2, kick(dt/2), EOS -- with dt kept on the device (no host round
 * trip) and one neighbour list per step shared by pass 1, pass 2 and the
 * next step's drift.  The previous step's dt is kept on the device between
 * calls on the same BVH; prevDtPsu is used only when no such state exists
 * (first call, or after astraea_gb300_invalidate_step_cache), exactly as the
 * engine passes Simulation::prevDtPsu to launchReduceDtPsu.  *outDtPsu (host,
 * may be NULL) receives this step's dt once the stream reaches the end of the
 * step (pinned memory: asynchronous; pageable memory: the copy blocks).
 * Needs one astraea_gb300_sort_and_build_bvh on this BVH beforehand (the
 * engine's evaluateInitialForcesOnDevice does that).  Fields the engine's
 * permutation moves but the step recomputes before reading (forces, rates,
 * EOS outputs, pass-1 outputs) are not moved, and the step's tree is kept in
 * the library's own node records: the BVH descriptor's node arrays (aabb*,
 * nodeMass, com*, nodeMaxH and the packed float4 arrays) keep the tree of the
 * last astraea_gb300_sort_and_build_bvh.  After writing fields from outside
 * the library between steps, call astraea_gb300_invalidate_step_cache: the
 * next step recomputes its dt and neighbour lists from them on the tree it
 * keeps.  That tree bounds the positions and h of its build, so positions or
 * h moved beyond them need astraea_gb300_sort_and_build_bvh first -- as in
 * the engine, whose drift also walks the tree of the last build. */
AstraeaStatus astraea_gb300_step(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh,
                                 float prevDtPsu, float maxDtPsu, float theta, float* outDtPsu);
/* Forget the neighbour lists and device-side dt kept between fused steps. */
AstraeaStatus astraea_gb300_invalidate_step_cache(const AstraeaRadixBvh* bvh);
/* Pre-allocate every library-owned scratch buffer for `capacity` particles on
 * the current device, so later calls allocate nothing (stream capture). */
AstraeaStatus astraea_gb300_reserve(const AstraeaRadixBvh* bvh, uint32_t capacity);

/* Release the library scratch kept for this BVH (its neighbour lists and
 * packed node records) without touching the BVH's own arrays; for callers
 * that allocate and free the BVH arrays themselves.  No engine counterpart
 * (the engine's fallback scratch lives until process exit). */
AstraeaStatus astraea_gb300_release_scratch(const AstraeaRadixBvh* bvh);

/* ---- autotuning (no engine counterpart) --------------------------------- */

/* Block shape of the two tree walks: warps per block (2, 4 or 8) of the
 * gravity walk and of the neighbour-list walk, and the times that chose
 * them.  The walks' results do not depend on the block shape (each group of
 * 32 particles is walked by one warp); the shape sets how many warps share
 * an SM's registers and shared memory. */
typedef struct AstraeaTuning {
    uint32_t gravityWarps;
    uint32_t neighborWarps;
    float gravityMs;         /* best time of the chosen gravity variant (0 when set by hand) */
    float neighborMs;        /* best time of the chosen neighbour-walk variant */
} AstraeaTuning;

/* Times the gravity walk and the neighbour-list walk with 2, 4 and 8 warps
 * per block on the tree of bvh as built for p (after
 * astraea_gb300_sort_and_build_bvh), best of three launches each, and keeps
 * the fastest for every later call on this device whose particle count has
 * the same floor(log2 count).  The gravity walk timed is the one the current
 * far-field mode runs at theta (mode 2: its plain fallback walk), and its
 * choice is kept for that walk only: the monopole, quadrupole (mode 1) and
 * expansion (mode 3) walks, each with and without the inside-box rule of
 * theta^2 > 1/3, are tuned separately (an untuned walk runs 4-warp blocks).
 * Overwrites p's gravity outputs and the neighbour lists (the next stage
 * calls or step recompute both).  Blocks. */
AstraeaStatus astraea_gb300_autotune(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                     AstraeaTuning* out);
/* The tuning used for `count` particles on this device ({4, 4} untuned):
 * the neighbour walk's and the monopole gravity walk's at theta^2 <= 1/3
 * (the engine's walk). */
AstraeaStatus astraea_gb300_get_tuning(uint32_t count, AstraeaTuning* out);
/* Sets it by hand (warps 2, 4 or 8), e.g. from a saved autotune result; the
 * gravity shape applies to every gravity walk. */
AstraeaStatus astraea_gb300_set_tuning(uint32_t count, const AstraeaTuning* tuning);
/* Warps per block the gravity walk of far-field mode `farFieldMode` (0-3,
 * on a tree built in that mode) at theta runs for `count` particles. */
AstraeaStatus astraea_gb300_get_gravity_warps(uint32_t count, int farFieldMode, float theta, uint32_t* outWarps);

/* ---- library primitives and diagnostics --------------------------------- */

/* Stable LSD radix sort of (u64 key, u32 value) pairs over key bits
 * [0, endBit), endBit <= 64; the call site it replaces is
 * cub::DeviceRadixSort::SortPairs in engine/sph_gravity.cu:2029-2046.
 * keysIn/valsIn are used as ping-pong buffers and are clobbered; the sorted
 * pairs land in keysOut/valsOut. */
AstraeaStatus astraea_gb300_radix_sort_pairs(uint64_t* keysIn, uint64_t* keysOut,
                                             uint32_t* valsIn, uint32_t* valsOut,
                                             uint32_t n, int endBit);
/* The same sort for callers that cannot allocate device memory (an arena or
 * pool owns all of it, or the host forbids allocation after start-up): its
 * scratch is a fixed ~2.1 MB array inside the library image, so the call
 * makes no cudaMalloc/cudaFree.  At most 1,048,576 keys (else
 * ASTRAEA_ERR_CAPACITY).  The first call on a device looks up the array's
 * address (once per device; make it before any stream capture) and keeps it
 * for the life of the process: cudaDeviceReset between calls is not
 * supported.  Calls share the array: calls whose GPU work overlaps race on it.
 * A look-back wait that gives up is reported like the allocating sort's
 * (ASTRAEA_DEVFLAG_LOOKBACK_TIMEOUT in astraea_gb300_read_device_status, and
 * ASTRAEA_ERR_DEVICE_TIMEOUT from astraea_gb300_reduce_dt_psu) until
 * astraea_gb300_reset_device_status.  No counterpart in the reference. */
AstraeaStatus astraea_gb300_radix_sort_pairs_noalloc(uint64_t* keysIn, uint64_t* keysOut,
                                                     uint32_t* valsIn, uint32_t* valsOut,
                                                     uint32_t n, int endBit);
/* Device status word (bit flags, see ASTRAEA_DEVFLAG_*) and counters
 * accumulated since the last reset; host pointers, 8 x u64 counters. */
#define ASTRAEA_DEVFLAG_LOOKBACK_TIMEOUT   0x1u
#define ASTRAEA_DEVFLAG_NEIGHBOR_OVERFLOW  0x2u
#define ASTRAEA_DEVFLAG_STACK_OVERFLOW     0x4u
#define ASTRAEA_DEVFLAG_GROUP_FALLBACK     0x8u
AstraeaStatus astraea_gb300_read_device_status(uint32_t* outFlags, uint64_t* outCounters8);
/* Every device counter accumulated since the last reset, in this order (the
 * first eight are the counters of astraea_gb300_read_device_status); up to
 * `capacity` of them, *outCount = how many were written.  Blocks.  No engine
 * counterpart. */
#define ASTRAEA_COUNTER_GRAVITY_INTERACTIONS  0u
#define ASTRAEA_COUNTER_GRAVITY_NODE_TESTS    1u
#define ASTRAEA_COUNTER_NEIGHBOR_ENTRIES      2u
#define ASTRAEA_COUNTER_GRAVITY_ROUNDS        3u
#define ASTRAEA_COUNTER_GRAVITY_STACK_PEAK    4u   /* maximum, not a sum */
#define ASTRAEA_COUNTER_FALLBACK_WALKS        5u
#define ASTRAEA_COUNTER_NEIGHBOR_CANDIDATES   6u
#define ASTRAEA_COUNTER_GRAVITY_UNDECIDED     7u
#define ASTRAEA_COUNTER_PASS1_PAIRS           8u   /* pairs with r < 2 h_i in SPH pass 1 */
#define ASTRAEA_COUNTER_PASS2_PAIRS           9u   /* pairs with r < max(2 h_i, 2 h_j) in SPH pass 2 */
#define ASTRAEA_COUNTER_DRIFT_PAIRS          10u   /* pairs inside the XSPH drift's radius */
#define ASTRAEA_COUNTER_GRAVITY_GROUP_EVALS  11u   /* far-field mode 3: far nodes taken by group expansions */
#define ASTRAEA_COUNTER_GRAVITY_BUCKET_LEAVES 12u  /* far-field mode 3: P-P terms from leaf buckets */
#define ASTRAEA_COUNTER_COUNT                13u
AstraeaStatus astraea_gb300_read_device_counters(uint64_t* outCounters, uint32_t capacity, uint32_t* outCount);
/* Stage timing of the fused step (no engine counterpart; the engine times
 * the whole step, gpuStepMs, engine/simulation.cpp:1719-1739).  While
 * enabled, astraea_gb300_step records a CUDA event on its stream where each
 * stage begins and where the step ends; astraea_gb300_read_stage_times
 * returns the stage times of the last such step on this BVH in milliseconds,
 * in the order ASTRAEA_STAGE_* (blocks until that step has finished).  The
 * refresh stage is the leaf refresh, drift neighbour lists and dt reduction
 * of a step whose cache was invalid (near 0 otherwise).  Off by default; the
 * events add a few microseconds per step.  Do not enable it while a CUDA
 * graph is being captured. */
#define ASTRAEA_STAGE_REFRESH      0
#define ASTRAEA_STAGE_KICK         1    /* opening half kick, dt resolved on the device */
#define ASTRAEA_STAGE_DRIFT        2
#define ASTRAEA_STAGE_SORT         3    /* bounds + Morton codes + radix sort */
#define ASTRAEA_STAGE_PERMUTE      4    /* permutation + Karras build */
#define ASTRAEA_STAGE_REFIT        5
#define ASTRAEA_STAGE_NEIGHBOURS   6
#define ASTRAEA_STAGE_PASS1        7
#define ASTRAEA_STAGE_EOS          8
#define ASTRAEA_STAGE_GRAVITY      9
#define ASTRAEA_STAGE_PASS2       10
#define ASTRAEA_STAGE_KICK_EOS    11    /* closing half kick + EOS + next dt candidate */
#define ASTRAEA_STAGE_COUNT       12
AstraeaStatus astraea_gb300_set_stage_timing(int enable);
AstraeaStatus astraea_gb300_read_stage_times(const AstraeaRadixBvh* bvh, float* outMs, uint32_t capacity,
                                             uint32_t* outCount);
/* Measured FP32 FMA throughput of the current device in TFLOP/s (the
 * denominator of the gravity kernel's roofline): the larger of scalar fmaf
 * chains and packed fma.rn.f32x2 chains.  Blocks; no engine counterpart. */
AstraeaStatus astraea_gb300_measure_fp32_tflops(float* outTflops);
/* The gravity stage (far-field mode 0) with each group's interaction count
 * written to groupCounts[g] (device, ceil(count / 32) words): the per-group
 * form of ASTRAEA_COUNTER_GRAVITY_INTERACTIONS, for locating a group whose
 * interaction set differs from the oracle's.  No engine counterpart. */
AstraeaStatus astraea_gb300_debug_gravity_group_counts(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                                      uint32_t* groupCounts);
/* The gravity stage (far-field mode 0) recording, for one group, every node it
 * takes as a monopole (node index >= 0) and every leaf it reaches (~particle)
 * into trace[1 ..] in walk order, trace[0] = the number recorded (device,
 * capacity + 1 words).  Diagnostic; no engine counterpart. */
AstraeaStatus astraea_gb300_debug_gravity_group_trace(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                                     uint32_t group, int32_t* trace, uint32_t capacity);
/* Both forms of that measurement (host outputs, TFLOP/s). */
AstraeaStatus astraea_gb300_measure_fp32_peaks(float* outScalarTflops, float* outPackedTflops);
AstraeaStatus astraea_gb300_reset_device_status(void);
/* FP64 direct-sum gravity at `count` listed targets (device indices; device
 * outputs: acc3[3 count] as x, y, z, and phi[count]), over all p->count
 * particles with eps_ij = (eps_i + eps_j)/2, eps = 0.8 max(h0, 1e-6): the
 * accuracy reference of the Barnes-Hut and far-field modes (the N^2 check of
 * tests/cpp/test_gravity_sph.cpp:366-378).  A target index >= count of
 * particles gives zeros.  Asynchronous; no engine counterpart. */
AstraeaStatus astraea_gb300_direct_gravity_f64(const AstraeaParticles* p, const uint32_t* targets, uint32_t count,
                                              double* acc3, double* phi);

/* Test hook: lower the onesweep look-back spin limit (0 restores default). */
AstraeaStatus astraea_gb300_set_lookback_spin_limit(uint32_t limit);
/* Failure-detection probe: runs the onesweep look-back wait on a status word
 * that nothing publishes, with the given spin limit.  The wait must give up:
 * returns ASTRAEA_ERR_DEVICE_TIMEOUT, *outResult = 2 and sets
 * ASTRAEA_DEVFLAG_LOOKBACK_TIMEOUT in the device status (no GPU fault, the
 * context stays usable).  No engine counterpart. */
AstraeaStatus astraea_gb300_debug_lookback_probe(uint32_t spinLimit, uint32_t* outResult);

#ifdef __cplusplus
}
#endif

#endif /* ASTRAEA_GB300_H */
