// ref_eos_capi.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C entry point over the reference's own EOS, so the oracle's restatement
// can be checked against it.  Built only by oracle/build_oracle.py, together
// with engine/eos.cu compiled as host C++ straight from the reference
// checkout (its ASTRAEA_HD macro is empty without __CUDACC__,
// engine/eos.hpp:8-14).  The result goes to oracle/_ref/, which is never
// committed.
#include <cstdint>

#include "eos.hpp"

extern "C" {

void ref_eos_batch(uint32_t n, const uint8_t* mat, const float* rho, const float* u, const float* dmg,
                   float* P, float* cs, float* T, uint8_t* phase) {
    for (uint32_t i = 0; i < n; ++i) {
        const astraea::eos::EosEvalResult r =
            astraea::eos::evaluateEosPsu(static_cast<astraea::MaterialId>(mat[i]), rho[i], u[i], dmg[i]);
        P[i] = r.pressurePsu;
        cs[i] = r.soundSpeedPsu;
        T[i] = r.tempK;
        phase[i] = r.phaseId;
    }
}

double ref_cold_energy(int mat, double rhoPsu) {
    return astraea::eos::computeColdEnergyPsu(static_cast<astraea::MaterialId>(mat), rhoPsu);
}

void ref_from_rho_temp_si(int mat, double rhoKgM3, double tempK, double* outU, double* outP) {
    astraea::eos::evaluateFromRhoTempSI(static_cast<astraea::MaterialId>(mat), rhoKgM3, tempK, *outU, *outP);
}

double ref_invert_density(int mat, double targetP, double tempK, double guess) {
    return astraea::eos::invertDensityFromPressureTempSI(static_cast<astraea::MaterialId>(mat), targetP, tempK, guess);
}

}  // extern "C"
