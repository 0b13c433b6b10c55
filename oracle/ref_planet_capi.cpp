// ref_planet_capi.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's own PlanetBuilder
// (engine/planet_builder.cpp:398-905), so the library's device planet
// builder can be checked against it and golden vectors can be generated.
// Built only by oracle/build_oracle.py from engine/planet_builder.cpp,
// engine/presets.cpp and engine/eos.cu (as host C++) where they lie in the
// reference checkout; the result goes to oracle/_ref/, never committed.
#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

#include "planet_builder.hpp"
#include "presets.hpp"

namespace {

astraea::BodyInitSpec makeSpec(int archetype, double massKg, double surfT, double coreT, double spin) {
    astraea::BodyInitSpec s{};
    s.archetype = static_cast<astraea::PlanetArchetype>(archetype);
    s.massKg = massKg;
    s.surfaceTempK = surfT;
    s.coreTempK = coreT;
    s.spinOmegaRadS = spin;
    return s;
}

}  // namespace

extern "C" {

// Profile columns: r, rho, P, M, T (double) and material (u8).  Returns the
// sample count, or -(count) when cap is too small (nothing written).
int ref_solve_hydrostatic(int archetype, double massKg, double surfT, double coreT, double spin, uint32_t cap,
                          double* r, double* rho, double* P, double* M, double* T, uint8_t* mat, double* outRadius,
                          double* outPc, double* outSeconds) {
    const auto t0 = std::chrono::steady_clock::now();
    double radius = 0.0, pc = 0.0;
    const auto prof = astraea::PlanetBuilder::solveHydrostatic1D(makeSpec(archetype, massKg, surfT, coreT, spin),
                                                                 radius, pc);
    const auto t1 = std::chrono::steady_clock::now();
    *outRadius = radius;
    *outPc = pc;
    *outSeconds = std::chrono::duration<double>(t1 - t0).count();
    if (prof.size() > cap) return -static_cast<int>(prof.size());
    for (size_t i = 0; i < prof.size(); ++i) {
        r[i] = prof[i].rM;
        rho[i] = prof[i].rhoKgM3;
        P[i] = prof[i].pressurePa;
        M[i] = prof[i].enclosedMassKg;
        T[i] = prof[i].tempK;
        mat[i] = static_cast<uint8_t>(prof[i].material);
    }
    return static_cast<int>(prof.size());
}

// f12: posX posY posZ velX velY velZ mass h0 rho u tempK epsFail;
// tr4: tracerRestRadiusPsu, tracerRestNormalX/Y/Z;
// info: equatorialRadiusM, actualMassKg, centralPressurePa, tracerCount, seconds.
int ref_build_planet(int archetype, double massKg, double surfT, double coreT, double spin, uint32_t n,
                     uint32_t bodyId, uint32_t gridRes, uint64_t seed, float* const* f12, uint8_t* mat,
                     uint8_t* body, int32_t* tracerIndex, float* const* tr4, uint8_t* isOcean, double* info) {
    const auto t0 = std::chrono::steady_clock::now();
    const astraea::BuiltPlanetHost b = astraea::PlanetBuilder::buildPlanet(
        makeSpec(archetype, massKg, surfT, coreT, spin), n, static_cast<uint8_t>(bodyId), gridRes, seed);
    const auto t1 = std::chrono::steady_clock::now();
    if (b.posX.size() != n) return -1;
    const std::vector<float>* src[12] = {&b.posX, &b.posY, &b.posZ, &b.velX, &b.velY, &b.velZ,
                                         &b.mass, &b.h0,   &b.rho,  &b.u,    &b.tempK, &b.epsFail};
    for (int k = 0; k < 12; ++k) std::memcpy(f12[k], src[k]->data(), n * sizeof(float));
    std::memcpy(mat, b.materialId.data(), n);
    std::memcpy(body, b.bodyId.data(), n);
    std::memcpy(tracerIndex, b.tracerIndex.data(), n * sizeof(int32_t));
    const std::vector<float>* tsrc[4] = {&b.tracerRestRadiusPsu, &b.tracerRestNormalX, &b.tracerRestNormalY,
                                         &b.tracerRestNormalZ};
    for (int k = 0; k < 4; ++k) std::memcpy(tr4[k], tsrc[k]->data(), n * sizeof(float));
    std::memcpy(isOcean, b.tracerIsOcean.data(), n);
    info[0] = b.equatorialRadiusM;
    info[1] = b.actualMassKg;
    info[2] = b.centralPressurePa;
    info[3] = static_cast<double>(b.tracerCount);
    info[4] = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

// Archetype defaults (engine/presets.cpp:9-88): mass, surface T, core T, spin,
// layer count, then (material, mass fraction) for three layers.
void ref_archetype(int archetype, double* out) {
    const astraea::ArchetypeComposition& c =
        astraea::getArchetypeComposition(static_cast<astraea::PlanetArchetype>(archetype));
    out[0] = c.defaultMassKg;
    out[1] = c.defaultSurfaceTempK;
    out[2] = c.defaultCoreTempK;
    out[3] = c.defaultSpinOmegaRadS;
    out[4] = c.layerCount;
    for (int i = 0; i < 3; ++i) {
        out[5 + 2 * i] = static_cast<double>(c.layers[i].material);
        out[6 + 2 * i] = c.layers[i].massFraction;
    }
}

}  // extern "C"
