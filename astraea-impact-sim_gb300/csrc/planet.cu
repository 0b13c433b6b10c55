// planet.cu -- planet construction straight into the device particle SoA:
// the counterpart of PlanetBuilder (engine/planet_builder.cpp:398-905) and of
// the body upload that follows it (engine/simulation.cpp:468-523, 852-880).
//
// Host part: serial, FP64, with the engine's arithmetic operation for
// operation (the file is compiled without multiply-add contraction, host and
// device), so the radial profile, the shell plan and every per-shell value
// are bit-identical to the engine's:
//   * the hydrostatic RK4 shooting and the bisection on log P_c
//     (planet_builder.cpp:55-264, 398-473) over an FP64 host restatement of
//     the Tillotson / polytrope EOS (eos.cu:126-535);
//   * the layer partition and shell plan (planet_builder.cpp:486-638);
//   * the random stream.  The engine draws from one mt19937_64, in shell
//     order, three uniforms for each shell's rotation and one per particle
//     for its Weibull fracture strain.  That stream is serial, so the host
//     draws it with the standard library's engine and distributions (as the
//     engine does) and ships the per-particle uniforms in pinned chunks.
// Device part: a kernel per chunk places the chunk's particles (golden-angle
// spiral on the rotated shell, rigid spin about +Y, Weibull strain) and
// writes every field the engine's upload writes for a body; the chunk's
// copy and kernel overlap the host drawing the next chunk.  For a
// LivingTerra body the surface tracers (planet_builder.cpp:735-902) are
// chosen on the device: candidates sorted by radius with the library's
// radix sort, the pool cut, the best candidate of every cube-sphere bin by
// one 64-bit atomicMax per candidate, the greedy fill of empty bins in one
// block, and the compaction of tracer indices.
//
// One documented difference: the engine orders tracer candidates with
// std::sort, which leaves the order of exactly equal radii unspecified; here
// equal radii keep particle order.  It can change the result only when the
// candidate pool is cut inside a run of equal radii (fewer in-shell
// candidates than three times the tracer count, yet more candidates).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "kernels.h"

namespace astraea_gb300 {
namespace planet {

namespace {

// engine/units.hpp:5-27, the same constant expressions.
constexpr double kGSi = 6.67430e-11;
constexpr double kLUnit = 1.0e6;
constexpr double kMUnit = 1.0e24;
constexpr double kTUnit = 1.0e3;
constexpr double kRhoUnit = kMUnit / (kLUnit * kLUnit * kLUnit);
constexpr double kPUnit = kMUnit / (kLUnit * kTUnit * kTUnit);
constexpr double kUUnit = (kLUnit * kLUnit) / (kTUnit * kTUnit);
constexpr double kPi = 3.14159265358979323846;

enum : int { kIron = 0, kGranite = 1, kWaterIce = 2, kHydrogenHelium = 3, kRegolith = 4 };
enum : int { kLivingTerra = 0, kGasGiant = 4 };

// FP64 EOS constants (SI) of engine/eos.cu:10-116.
struct Till {
    double rho0, a, b, APa, BPa, E0, Eiv, Ecv, alpha, beta, cv, tRef, epsFailMin, kH2, gamma;
};
constexpr Till kTill[5] = {
    {7800.0, 0.5, 1.5, 1.28e11, 1.05e11, 9.50e6, 2.40e6, 8.67e6, 5.0, 5.0, 449.0, 293.0, 1.0e-3, 0.0, 1.0},
    {2680.0, 0.5, 1.3, 1.80e10, 1.80e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 790.0, 293.0, 1.0e-4, 0.0, 1.0},
    {1000.0, 0.7, 0.15, 2.18e9, 1.325e10, 7.00e6, 4.19e5, 2.68e6, 10.0, 5.0, 4184.0, 273.15, 5.0e-4, 0.0, 1.0},
    {0.178, 0.4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 8260.0, 0.0, 1.0, 2.08e5, 1.4},
    {2000.0, 0.5, 1.3, 1.20e10, 1.20e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 800.0, 293.0, 5.0e-5, 0.0, 1.0},
};
const Till& till(int m) { return kTill[(m >= 0 && m <= 4) ? m : kGranite]; }

// Archetype layer tables of engine/presets.cpp:9-88.
struct Composition {
    int layers;
    int mat[3];
    double frac[3];
};
constexpr Composition kComp[6] = {
    {3, {kIron, kGranite, kWaterIce}, {0.320, 0.675, 0.005}},
    {2, {kIron, kGranite, kGranite}, {0.680, 0.320, 0.0}},
    {3, {kIron, kGranite, kWaterIce}, {0.150, 0.450, 0.400}},
    {2, {kIron, kGranite, kGranite}, {0.250, 0.750, 0.0}},
    {3, {kIron, kGranite, kHydrogenHelium}, {0.050, 0.100, 0.850}},
    {3, {kIron, kGranite, kRegolith}, {0.220, 0.580, 0.200}},
};

// The engine's helpers (eos.cu:128-134, std::max / std::clamp semantics).
inline double maxD(double a, double b) { return a > b ? a : b; }
inline double clampD(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline double stdMax(double a, double b) { return (a < b) ? b : a; }
inline double stdMin(double a, double b) { return (b < a) ? b : a; }
inline double stdClamp(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

// ------------------------------------------------------------ host EOS ---
double coldEnergyPsu(int m, double rhoPsu) {                        // eos.cu:283-318
    const Till& t = till(m);
    const double rho = maxD(rhoPsu, 0.0);
    if (m == kHydrogenHelium) return t.kH2 * rho;
    const double rho0 = t.rho0 / kRhoUnit;
    const double eta = rho / rho0;
    if (eta <= 1.0) return 0.0;
    const double mu = eta - 1.0;
    const double A = t.APa / kPUnit;
    const double B = t.BPa / kPUnit;
    double ta, tb;
    if (mu < 1.0e-5) {
        const double mu2 = mu * mu;
        const double mu3 = mu2 * mu;
        const double mu4 = mu3 * mu;
        const double mu5 = mu4 * mu;
        ta = 0.5 * mu2 - (2.0 / 3.0) * mu3 + 0.75 * mu4 - 0.8 * mu5;
        tb = (1.0 / 3.0) * mu3 - 0.5 * mu4 + 0.6 * mu5;
    } else {
        const double le = std::log1p(mu);
        ta = le - (mu / eta);
        tb = (mu * (2.0 + mu)) / eta - 2.0 * le;
    }
    return (A * ta + B * tb) / rho0;
}

// Pressure branches without damage (eos.cu:136-174, 176-227); only P is used.
double tillCompressed(const Till& t, double rho, double eta, double mu, double uE) {
    const double A = t.APa / kPUnit;
    const double B = t.BPa / kPUnit;
    const double E0 = t.E0 / kUUnit;
    const double bEff = (mu >= 0.0) ? B : 0.0;
    const double den = E0 * eta * eta;
    const double ratio = (den > 1.0e-30) ? (uE / den) : 1.0e30;
    const double invW = 1.0 / (ratio + 1.0);
    return (t.a + t.b * invW) * rho * uE + A * mu + bEff * mu * mu;
}

double tillExpanded(const Till& t, double rho, double eta, double mu, double uE) {
    const double A = t.APa / kPUnit;
    const double E0 = t.E0 / kUUnit;
    const double x = 1.0 / eta - 1.0;
    const double ax2 = t.alpha * x * x;
    const double bx = t.beta * x;
    const double eA = (ax2 < 700.0) ? std::exp(-ax2) : 0.0;
    if (eA == 0.0) return t.a * rho * uE;
    const double eB = (bx < 700.0) ? std::exp(-bx) : 0.0;
    const double den = E0 * eta * eta;
    const double ratio = (den > 1.0e-30) ? (uE / den) : 1.0e30;
    const double invW = 1.0 / (ratio + 1.0);
    const double ideal = t.a * rho * uE;
    const double inner = (t.b * rho * uE * invW) + A * mu * eB;
    return ideal + inner * eA;
}

// evaluateFromRhoTempSI (eos.cu:390-442): specific energy and pressure, SI.
void stateFromRhoTemp(int m, double rhoKg, double tempK, double& uSi, double& pSi) {
    const Till& t = till(m);
    const double rho = maxD(rhoKg, 1.0e-12);
    const double T = maxD(tempK, 0.0);
    if (m == kHydrogenHelium) {
        const double uTh = t.cv * T;
        uSi = t.kH2 * rho + uTh;
        pSi = t.kH2 * rho * rho + (t.gamma - 1.0) * rho * uTh;
        return;
    }
    const double rhoPsu = rho / kRhoUnit;
    const double uColdPsu = coldEnergyPsu(m, rhoPsu);
    const double uColdSi = uColdPsu * kUUnit;
    uSi = uColdSi + t.cv * T;
    const double excess = maxD(0.0, uSi - uColdSi - t.cv * t.tRef);
    const double uE = uColdPsu + excess / kUUnit;
    const double rho0 = t.rho0 / kRhoUnit;
    const double eta = rhoPsu / rho0;
    const double mu = eta - 1.0;
    const double Eiv = t.Eiv / kUUnit;
    const double Ecv = t.Ecv / kUUnit;
    double P;
    if (eta >= 1.0 || uE < Eiv) {
        P = tillCompressed(t, rhoPsu, eta, mu, uE);
    } else if (uE >= Ecv) {
        P = tillExpanded(t, rhoPsu, eta, mu, uE);
    } else {
        const double pc = tillCompressed(t, rhoPsu, eta, mu, uE);
        const double pe = tillExpanded(t, rhoPsu, eta, mu, uE);
        const double f = clampD((uE - Eiv) / maxD(1.0e-30, Ecv - Eiv), 0.0, 1.0);
        P = (1.0 - f) * pc + f * pe;
    }
    pSi = P * kPUnit;
}

// invertDensityFromPressureTempSI (eos.cu:444-535): bracket, then
// secant-in-bracket iterations.
double densityFromPressureTemp(int m, double targetP, double tempK, double guess) {
    const Till& t = till(m);
    if (m == kHydrogenHelium) {
        if (targetP <= 0.0) return 1.0e-6;
        const double bLin = (t.gamma - 1.0) * t.cv * maxD(tempK, 0.0);
        const double disc = std::sqrt(bLin * bLin + 4.0 * t.kH2 * targetP);
        return (2.0 * targetP) / maxD(1.0e-30, bLin + disc);
    }
    auto pressureAt = [&](double rho) {
        double u = 0.0, p = 0.0;
        stateFromRhoTemp(m, rho, tempK, u, p);
        return p;
    };
    double start = (guess > 0.0) ? guess : t.rho0;
    start = clampD(start, 0.05 * t.rho0, 50.0 * t.rho0);
    double lo = start, hi = start;
    const double pStart = pressureAt(start);
    if (pStart > targetP) {
        for (int i = 0; i < 64; ++i) {
            lo *= (i < 12) ? 0.85 : 0.5;
            if (lo < 1.0e-6) lo = 1.0e-6;
            if (pressureAt(lo) <= targetP || lo <= 1.0e-6) break;
        }
    } else if (pStart < targetP) {
        for (int i = 0; i < 64; ++i) {
            hi *= (i < 12) ? 1.25 : 2.0;
            if (pressureAt(hi) >= targetP || hi > 1.0e8) break;
        }
    } else {
        return start;
    }
    double fLo = pressureAt(lo) - targetP;
    double fHi = pressureAt(hi) - targetP;
    if (fLo >= 0.0) return lo;
    if (fHi <= 0.0) return hi;
    double rho = 0.5 * (lo + hi);
    for (int it = 0; it < 64; ++it) {
        const double f = pressureAt(rho) - targetP;
        if (std::abs(f) <= 1.0e-9 * maxD(1.0, std::abs(targetP))) return rho;
        if (f < 0.0) {
            lo = rho;
            fLo = f;
        } else {
            hi = rho;
            fHi = f;
        }
        if (hi - lo <= 1.0e-12 * maxD(1.0, rho)) return 0.5 * (lo + hi);
        double next = 0.5 * (lo + hi);
        const double den = fHi - fLo;
        if (std::abs(den) > 1.0e-30) {
            const double sec = lo - fLo * (hi - lo) / den;
            if (sec > lo && sec < hi) next = sec;
        }
        rho = next;
    }
    return 0.5 * (lo + hi);
}

// --------------------------------------------------- hydrostatic shooting
struct Shot {
    double radius = 0.0;
    double mass = 0.0;
    bool capped = false;
};

// One outward integration from the centre at central pressure pc
// (planet_builder.cpp:55-264).  The state is (r, P, M) with the density of
// the current layer re-solved from (P, T(P)) at every evaluation.
class Shooter {
public:
    Shooter(const BodySpec& spec, double pc, double pSurf, double dr)
        : spec_(spec), comp_(kComp[spec.archetype]), pc_(pc), pSurf_(pSurf), dr_(dr) {}

    Shot run(std::vector<Sample>* rec) {
        Shot out;
        const double target = spec_.massKg;
        const double bail = 20.0 * target;
        double layerEnd[3] = {0.0, 0.0, 0.0};
        double cum = 0.0;
        for (int i = 0; i < comp_.layers; ++i) {
            cum += comp_.frac[i];
            layerEnd[i] = (i + 1 == comp_.layers) ? std::numeric_limits<double>::infinity() : (cum * target);
        }
        int layer = 0;
        double r = 0.0, P = pc_, M = 0.0;
        double T = spec_.coreTempK;
        double guess = till(comp_.mat[0]).rho0;
        double rho = density(comp_.mat[0], P, guess, &T);
        guess = rho;
        record(rec, 0.0, rho, P, 0.0, T, comp_.mat[0]);

        for (int step = 0; step < 12000; ++step) {
            const int mat = comp_.mat[layer];
            const bool finer = spec_.archetype == kGasGiant && layer + 1 < comp_.layers;
            const double h = finer ? (0.25 * dr_) : dr_;
            double nP = P, nM = M;
            if (r == 0.0) {
                nP = P - (2.0 / 3.0) * kPi * kGSi * rho * rho * h * h;
                nM = (4.0 / 3.0) * kPi * rho * h * h * h;
            } else {
                rk4(mat, r, P, M, h, guess, &nP, &nM);
            }
            const bool surface = nP <= pSurf_;
            const bool boundary = (layer + 1 < comp_.layers) && (nM >= layerEnd[layer]);
            const double fracP =
                surface ? ((P - nP > 1.0e-30) ? stdClamp((P - pSurf_) / (P - nP), 0.0, 1.0) : 1.0) : 2.0;
            const double fracM =
                boundary ? ((nM - M > 1.0e-30) ? stdClamp((layerEnd[layer] - M) / (nM - M), 0.0, 1.0) : 1.0) : 2.0;

            if (surface && (!boundary || fracP <= fracM)) {
                double rS = r + fracP * h;
                double mS = M;
                if (r == 0.0) {
                    const double dp = stdMax(0.0, P - pSurf_);
                    const double rA = std::sqrt(dp / ((2.0 / 3.0) * kPi * kGSi * rho * rho));
                    rS = stdMin(h, rA);
                    mS = (4.0 / 3.0) * kPi * rho * rS * rS * rS;
                } else {
                    double unused = 0.0;
                    rk4(mat, r, P, M, fracP * h, guess, &unused, &mS);
                }
                recordSurface(rec, rS, mS, mat, guess);
                out.radius = rS;
                out.mass = mS;
                return out;
            }

            if (boundary) {
                const double mB = layerEnd[layer];
                double sub = 0.0;
                if (r == 0.0) {
                    sub = std::cbrt((3.0 * mB) / (4.0 * kPi * rho));
                    sub = stdClamp(sub, 0.0, h);
                    nP = P - (2.0 / 3.0) * kPi * kGSi * rho * rho * sub * sub;
                    nM = mB;
                } else {
                    // bisection on the sub-step towards the layer's end mass
                    double lo = 0.0, hi = h;
                    sub = fracM * h;
                    for (int it = 0; it < 4; ++it) {
                        rk4(mat, r, P, M, sub, guess, &nP, &nM);
                        if (std::abs(nM - mB) <= 1.0e-10 * target) break;
                        if (nM < mB) {
                            lo = sub;
                        } else {
                            hi = sub;
                        }
                        sub = 0.5 * (lo + hi);
                    }
                    rk4(mat, r, P, M, sub, guess, &nP, &nM);
                }
                if (nP <= pSurf_) {
                    const double den = P - nP;
                    const double f = (den > 1.0e-30) ? stdClamp((P - pSurf_) / den, 0.0, 1.0) : 1.0;
                    const double rS = r + f * sub;
                    double unused = 0.0, mS = M;
                    rk4(mat, r, P, M, f * sub, guess, &unused, &mS);
                    recordSurface(rec, rS, mS, mat, guess);
                    out.radius = rS;
                    out.mass = mS;
                    return out;
                }
                r += sub;
                P = nP;
                M = mB;
                if (rec) {
                    double tE = 0.0;
                    const double rhoE = density(mat, P, guess, &tE);
                    record(rec, r, rhoE, P, M, tE, mat);
                }
                ++layer;
                const int next = comp_.mat[layer];
                double tN = 0.0;
                guess = till(next).rho0;
                rho = density(next, P, guess, &tN);
                guess = rho;
                record(rec, r, rho, P, M, tN, next);
                continue;
            }

            r += h;
            P = nP;
            M = nM;
            double tC = spec_.coreTempK;
            rho = density(mat, P, guess, &tC);
            guess = rho;
            record(rec, r, rho, P, M, tC, mat);
            if (M > bail) {
                out.radius = r;
                out.mass = M;
                out.capped = true;
                return out;
            }
        }
        out.radius = r;
        out.mass = M;
        return out;
    }

private:
    // planet_builder.cpp:21-46: linear geotherm in pressure, then the EOS
    // inverted for density (floored at 1e-3 kg/m^3 for hydrogen-helium).
    double density(int mat, double P, double guess, double* T) const {
        const double den = stdMax(pc_ - pSurf_, 1.0);
        const double frac = stdClamp((P - pSurf_) / den, 0.0, 1.0);
        *T = spec_.surfaceTempK + (spec_.coreTempK - spec_.surfaceTempK) * frac;
        double rho = densityFromPressureTemp(mat, stdMax(P, 0.0), *T, guess);
        if (mat == kHydrogenHelium) rho = stdMax(rho, 1.0e-3);
        return rho;
    }

    double derivs(int mat, double r, double P, double M, double guess, double* dP, double* dM) const {
        double T = 0.0;
        const double rho = density(mat, P, guess, &T);
        *dM = 4.0 * kPi * r * r * rho;
        if (r <= 1.0e-9) {
            *dP = -(4.0 / 3.0) * kPi * kGSi * rho * rho * r;
        } else {
            *dP = -kGSi * M * rho / (r * r);
        }
        return rho;
    }

    void rk4(int mat, double r0, double p0, double m0, double h, double guess, double* pOut, double* mOut) const {
        double k1P, k1M, k2P, k2M, k3P, k3M, k4P, k4M;
        const double rho1 = derivs(mat, r0, p0, m0, guess, &k1P, &k1M);
        const double rho2 = derivs(mat, r0 + 0.5 * h, stdMax(pSurf_, p0 + 0.5 * h * k1P), m0 + 0.5 * h * k1M, rho1,
                                   &k2P, &k2M);
        const double rho3 = derivs(mat, r0 + 0.5 * h, stdMax(pSurf_, p0 + 0.5 * h * k2P), m0 + 0.5 * h * k2M, rho2,
                                   &k3P, &k3M);
        derivs(mat, r0 + h, stdMax(pSurf_, p0 + h * k3P), m0 + h * k3M, rho3, &k4P, &k4M);
        *pOut = p0 + (h / 6.0) * (k1P + 2.0 * k2P + 2.0 * k3P + k4P);
        *mOut = m0 + (h / 6.0) * (k1M + 2.0 * k2M + 2.0 * k3M + k4M);
    }

    static void record(std::vector<Sample>* rec, double r, double rho, double P, double M, double T, int mat) {
        if (rec) rec->push_back(Sample{r, rho, P, M, T, mat});
    }

    void recordSurface(std::vector<Sample>* rec, double rS, double mS, int mat, double guess) const {
        if (!rec) return;
        double tS = spec_.surfaceTempK;
        const double rhoS = density(mat, pSurf_, guess, &tS);
        record(rec, rS, rhoS, pSurf_, mS, tS, mat);
    }

    const BodySpec& spec_;
    const Composition& comp_;
    double pc_, pSurf_, dr_;
};

// interpolateProfileAtMass (planet_builder.cpp:267-300).
Sample sampleAtMass(const std::vector<Sample>& prof, double m) {
    if (prof.empty()) return Sample{0.0, 0.0, 0.0, 0.0, 0.0, kGranite};
    if (m <= prof.front().M) return prof.front();
    if (m >= prof.back().M) return prof.back();
    const auto it = std::lower_bound(prof.begin(), prof.end(), m, [](const Sample& s, double v) { return s.M < v; });
    if (it == prof.begin()) return *it;
    const Sample& hi = *it;
    const Sample& lo = *(it - 1);
    const double dm = hi.M - lo.M;
    const double t = (dm > 1.0e-30) ? stdClamp((m - lo.M) / dm, 0.0, 1.0) : 0.0;
    Sample s;
    s.r = lo.r + t * (hi.r - lo.r);
    s.rho = lo.rho + t * (hi.rho - lo.rho);
    s.P = lo.P + t * (hi.P - lo.P);
    s.M = m;
    s.T = lo.T + t * (hi.T - lo.T);
    s.mat = (t < 0.5) ? lo.mat : hi.mat;
    return s;
}

// One shell of the plan: particles [first, first + count) of the body.
struct ShellDev {
    double rPsu;
    double rot[9];
    double epsMin;
    float mass, h0, rho, u, tempK;
    uint32_t first, count;
    uint32_t mat;
};

// Shoemake's uniform random rotation from three uniforms (the engine's
// randomRotationMatrix, planet_builder.cpp:303-326).
template <class Rng>
void randomRotation(Rng& rng, double* m) {
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    const double u1 = u01(rng);
    const double u2 = 2.0 * kPi * u01(rng);
    const double u3 = 2.0 * kPi * u01(rng);
    const double s1 = std::sqrt(stdMax(0.0, 1.0 - u1));
    const double s2 = std::sqrt(stdMax(0.0, u1));
    const double qx = s1 * std::sin(u2), qy = s1 * std::cos(u2);
    const double qz = s2 * std::sin(u3), qw = s2 * std::cos(u3);
    const double xx = qx * qx, yy = qy * qy, zz = qz * qz;
    const double xy = qx * qy, xz = qx * qz, yz = qy * qz;
    const double wx = qw * qx, wy = qw * qy, wz = qw * qz;
    m[0] = 1.0 - 2.0 * (yy + zz);
    m[1] = 2.0 * (xy - wz);
    m[2] = 2.0 * (xz + wy);
    m[3] = 2.0 * (xy + wz);
    m[4] = 1.0 - 2.0 * (xx + zz);
    m[5] = 2.0 * (yz - wx);
    m[6] = 2.0 * (xz - wy);
    m[7] = 2.0 * (yz + wx);
    m[8] = 1.0 - 2.0 * (xx + yy);
}

// ---------------------------------------------------------------- device
__device__ __forceinline__ void writeBody(const AstraeaParticles& p, uint32_t o, float px, float py, float pz,
                                          float vx, float vz, const ShellDev& s, float eps, uint8_t body) {
    p.posX[o] = px; p.posY[o] = py; p.posZ[o] = pz;
    p.velX[o] = vx; p.velY[o] = 0.0f; p.velZ[o] = vz;
    p.velHalfX[o] = vx; p.velHalfY[o] = 0.0f; p.velHalfZ[o] = vz;
    p.mass[o] = s.mass;
    p.h[o] = s.h0;
    p.h0[o] = s.h0;
    p.rho[o] = s.rho;
    p.u[o] = s.u;
    p.tempK[o] = s.tempK;
    p.epsFail[o] = eps;
    p.sXX[o] = 0.0f; p.sYY[o] = 0.0f; p.sZZ[o] = 0.0f;
    p.sXY[o] = 0.0f; p.sXZ[o] = 0.0f; p.sYZ[o] = 0.0f;
    p.damage[o] = 0.0f;
    p.damageCbrt[o] = 0.0f;
    p.pressure[o] = 0.0f;
    p.soundSpeed[o] = 0.0f;
    p.phaseId[o] = 0u;
    p.materialId[o] = static_cast<uint8_t>(s.mat);
    p.bodyId[o] = body;
    p.originalId[o] = o;
    p.tracerIndex[o] = -1;
    p.tracerRestRadiusPsu[o] = 0.0f;
    p.tracerRestNormalX[o] = 0.0f;
    p.tracerRestNormalY[o] = 0.0f;
    p.tracerRestNormalZ[o] = 0.0f;
    p.tracerIsOcean[o] = 0u;
}

// Particles [g0, g1) of the body (planet_builder.cpp:675-729); draws[g - g0]
// is the particle's uniform in (1e-6, 1 - 1e-6).
__global__ void placeKernel(AstraeaParticles p, uint32_t offset, uint8_t body, const ShellDev* __restrict__ shells,
                            uint32_t shellCount, const double* __restrict__ draws, uint32_t g0, uint32_t g1,
                            double golden, double spinT) {
    const uint32_t g = g0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= g1) return;
    uint32_t lo = 0, hi = shellCount - 1;          // last shell with first <= g
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (shells[mid].first <= g) lo = mid; else hi = mid - 1u;
    }
    const ShellDev& s = shells[lo];
    const uint32_t k = g - s.first;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (s.rPsu > 0.0) {
        const double zl = (s.count == 1u) ? 1.0
                                          : (1.0 - 2.0 * (static_cast<double>(k) + 0.5) / static_cast<double>(s.count));
        const double q = 1.0 - zl * zl;
        const double rxy = sqrt((0.0 < q) ? q : 0.0);
        const double th = golden * static_cast<double>(k);
        const double ux = rxy * cos(th);
        const double uy = rxy * sin(th);
        px = s.rPsu * (s.rot[0] * ux + s.rot[1] * uy + s.rot[2] * zl);
        py = s.rPsu * (s.rot[3] * ux + s.rot[4] * uy + s.rot[5] * zl);
        pz = s.rPsu * (s.rot[6] * ux + s.rot[7] * uy + s.rot[8] * zl);
    }
    const double w = -log(draws[g - g0]);
    double scale = pow((w < 1.0e-6) ? 1.0e-6 : w, 1.0 / 9.0);
    scale = (scale < 1.0) ? 1.0 : ((3.0 < scale) ? 3.0 : scale);
    writeBody(p, offset + g, static_cast<float>(px), static_cast<float>(py), static_cast<float>(pz),
              static_cast<float>(spinT * pz), static_cast<float>(-spinT * px), s,
              static_cast<float>(s.epsMin * scale), body);
}

// ------------------------------------------------------- tracer selection
// cubeFaceUvToUnitNormal / unitNormalToCubeFaceUv (planet_builder.cpp:329-396).
__device__ __forceinline__ float3 cubeFaceNormal(uint32_t face, float u, float v) {
    const float sx = 2.0f * u - 1.0f;
    const float sy = 2.0f * v - 1.0f;
    float x = 0.0f, y = 0.0f, z = 0.0f;
    switch (face % 6u) {
        case 0: x = 1.0f; y = sy; z = -sx; break;
        case 1: x = -1.0f; y = sy; z = sx; break;
        case 2: x = sx; y = 1.0f; z = -sy; break;
        case 3: x = sx; y = -1.0f; z = sy; break;
        case 4: x = sx; y = sy; z = 1.0f; break;
        default: x = -sx; y = sy; z = -1.0f; break;
    }
    const float inv = 1.0f / sqrtf(x * x + y * y + z * z);
    return make_float3(x * inv, y * inv, z * inv);
}

__device__ __forceinline__ uint32_t cubeBin(float3 n, uint32_t G) {
    const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
    float sx, sy;
    uint32_t face;
    if (ax >= ay && ax >= az) {
        const float d = (ax < 1.0e-12f) ? 1.0e-12f : ax;
        if (n.x >= 0.0f) { face = 0; sx = -n.z / d; sy = n.y / d; }
        else { face = 1; sx = n.z / d; sy = n.y / d; }
    } else if (ay >= ax && ay >= az) {
        const float d = (ay < 1.0e-12f) ? 1.0e-12f : ay;
        if (n.y >= 0.0f) { face = 2; sx = n.x / d; sy = -n.z / d; }
        else { face = 3; sx = n.x / d; sy = n.z / d; }
    } else {
        const float d = (az < 1.0e-12f) ? 1.0e-12f : az;
        if (n.z >= 0.0f) { face = 4; sx = n.x / d; sy = n.y / d; }
        else { face = 5; sx = -n.x / d; sy = n.y / d; }
    }
    float u = 0.5f * (sx + 1.0f), v = 0.5f * (sy + 1.0f);
    u = (u < 0.0f) ? 0.0f : ((1.0f < u) ? 1.0f : u);
    v = (v < 0.0f) ? 0.0f : ((1.0f < v) ? 1.0f : v);
    const float fg = static_cast<float>(G);
    const uint32_t gx = min(G - 1u, static_cast<uint32_t>(u * fg));
    const uint32_t gy = min(G - 1u, static_cast<uint32_t>(v * fg));
    return face * (G * G) + gy * G + gx;
}

__device__ __forceinline__ float3 binTarget(uint32_t bin, uint32_t G) {
    const uint32_t face = bin / (G * G);
    const uint32_t rem = bin - face * G * G;
    const uint32_t gy = rem / G, gx = rem - gy * G;
    const float fg = static_cast<float>(G);
    return cubeFaceNormal(face, (static_cast<float>(gx) + 0.5f) / fg, (static_cast<float>(gy) + 0.5f) / fg);
}

// 64-bit preference key: larger dot first, then earlier candidate position.
__device__ __forceinline__ unsigned long long prefKey(float dot, uint32_t c) {
    if (dot == 0.0f) dot = 0.0f;                   // -0 and +0 compare equal
    const uint32_t b = __float_as_uint(dot);
    const uint32_t ord = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return (static_cast<unsigned long long>(ord) << 32) | (0xFFFFFFFFu - c);
}

__device__ __forceinline__ float radiusOf(const AstraeaParticles& p, uint32_t o) {
    const float x = p.posX[o], y = p.posY[o], z = p.posZ[o];
    return sqrtf(x * x + y * y + z * z);
}

// Sort keys: candidates (r > 1e-6) by descending radius, then the rest
// after them; equal keys keep particle order (stable sort).
__global__ void tracerKeysKernel(AstraeaParticles p, uint32_t offset, uint32_t n, uint64_t* keys, uint32_t* vals,
                                 float* radii, uint32_t* candCount) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float r = radiusOf(p, offset + i);
    radii[i] = r;
    const bool cand = r > 1.0e-6f;
    keys[i] = cand ? static_cast<uint64_t>(~__float_as_uint(r)) : (1ull << 32);
    vals[i] = i;
    if (cand) atomicAdd(candCount, 1u);
}

// First position q in [minPool, L) whose candidate is outside the surface
// shell (planet_builder.cpp:776-786).
__global__ void poolCutKernel(AstraeaParticles p, uint32_t offset, const uint32_t* list, const float* radii,
                              uint32_t minPool, uint32_t L, uint32_t* cut) {
    const uint32_t q = minPool + blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= L) return;
    const uint32_t first = list[0];
    const float rMax = radii[first];
    const float dr = p.h0[offset + first];
    const uint32_t pid = list[q];
    const bool inShell = (radii[pid] >= rMax - 1.8f * dr) || (p.materialId[offset + pid] == kWaterIce);
    if (!inShell) atomicMin(cut, q);
}

__device__ __forceinline__ float3 candNormal(const AstraeaParticles& p, uint32_t o, float r) {
    if (r > 1.0e-6f) {
        const float inv = 1.0f / r;
        return make_float3(p.posX[o] * inv, p.posY[o] * inv, p.posZ[o] * inv);
    }
    return make_float3(0.0f, 0.0f, 1.0f);
}

// Pass A (planet_builder.cpp:832-858): every pool candidate offers itself to
// its own bin; the bin keeps the best dot with its centre direction.
__global__ void binOfferKernel(AstraeaParticles p, uint32_t offset, const uint32_t* list, const float* radii,
                               uint32_t P, uint32_t G, float3* candN, unsigned long long* best) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P) return;
    const uint32_t pid = list[c];
    const float3 nrm = candNormal(p, offset + pid, radii[pid]);
    candN[c] = nrm;
    const uint32_t bin = cubeBin(nrm, G);
    const float3 t = binTarget(bin, G);
    const float dot = nrm.x * t.x + nrm.y * t.y + nrm.z * t.z;
    atomicMax(&best[bin], prefKey(dot, c));
}

__device__ __forceinline__ void assignTracer(const AstraeaParticles& p, uint32_t offset, uint32_t pid, uint32_t bin,
                                             float r, float3 nrm) {
    const uint32_t o = offset + pid;
    p.tracerIndex[o] = static_cast<int32_t>(bin);
    p.tracerRestRadiusPsu[o] = r;
    p.tracerRestNormalX[o] = nrm.x;
    p.tracerRestNormalY[o] = nrm.y;
    p.tracerRestNormalZ[o] = nrm.z;
    p.tracerIsOcean[o] = (p.materialId[o] == kWaterIce) ? 1u : 0u;
}

__global__ void binAssignKernel(AstraeaParticles p, uint32_t offset, const uint32_t* list, const float* radii,
                                const float3* candN, const unsigned long long* best, uint32_t T, uint8_t* used,
                                uint8_t* filled, uint32_t* assigned) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= T) return;
    const unsigned long long k = best[b];
    if (k == 0ull) {
        filled[b] = 0u;
        return;
    }
    const uint32_t c = 0xFFFFFFFFu - static_cast<uint32_t>(k & 0xFFFFFFFFull);
    used[c] = 1u;
    filled[b] = 1u;
    const uint32_t pid = list[c];
    assignTracer(p, offset, pid, b, radii[pid], candN[c]);
    atomicAdd(assigned, 1u);
}

// Pass B (planet_builder.cpp:860-881): bins left empty, in bin order, take
// the best unused pool candidate.  One block; the bins are sequential.
constexpr int kFillThreads = 1024;
__global__ void __launch_bounds__(kFillThreads) binFillKernel(AstraeaParticles p, uint32_t offset,
                                                              const uint32_t* list, const float* radii,
                                                              const float3* candN, uint32_t P, uint32_t G, uint32_t T,
                                                              uint8_t* used, uint8_t* filled, uint32_t* assigned) {
    __shared__ unsigned long long warpBest[kFillThreads / 32];
    for (uint32_t b = 0; b < T; ++b) {
        if (filled[b]) continue;                   // uniform across the block
        const float3 t = binTarget(b, G);
        unsigned long long mine = 0ull;
        for (uint32_t c = threadIdx.x; c < P; c += kFillThreads) {
            if (used[c]) continue;
            const float3 n = candN[c];
            const unsigned long long k = prefKey(n.x * t.x + n.y * t.y + n.z * t.z, c);
            mine = (k > mine) ? k : mine;
        }
        for (int s = 16; s > 0; s >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xFFFFFFFFu, mine, s);
            mine = (o > mine) ? o : mine;
        }
        if ((threadIdx.x & 31) == 0) warpBest[threadIdx.x >> 5] = mine;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long top = 0ull;
            for (int w = 0; w < kFillThreads / 32; ++w) top = (warpBest[w] > top) ? warpBest[w] : top;
            if (top != 0ull) {
                const uint32_t c = 0xFFFFFFFFu - static_cast<uint32_t>(top & 0xFFFFFFFFull);
                used[c] = 1u;
                filled[b] = 1u;
                const uint32_t pid = list[c];
                assignTracer(p, offset, pid, b, radii[pid], candN[c]);
                *assigned += 1u;
            }
        }
        __syncthreads();
    }
}

// Compaction (planet_builder.cpp:884-892): tracer ids renumbered 0.. in
// particle order when fewer bins than 6 G^2 were filled.
__global__ void tracerPidKernel(const AstraeaParticles p, uint32_t offset, uint32_t n, uint64_t* keys,
                                uint32_t* vals, uint32_t* count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (p.tracerIndex[offset + i] < 0) return;
    const uint32_t slot = atomicAdd(count, 1u);
    keys[slot] = i;
    vals[slot] = i;
}

__global__ void tracerRenumberKernel(AstraeaParticles p, uint32_t offset, const uint32_t* sortedPid, uint32_t m) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) p.tracerIndex[offset + sortedPid[k]] = static_cast<int32_t>(k);
}

// ------------------------------------------------------------ host glue
template <class T>
struct DevBuf {
    T* ptr = nullptr;
    ~DevBuf() {
        if (ptr) cudaFree(ptr);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&ptr, (n ? n : 1) * sizeof(T)); }
};

struct PinnedBuf {
    double* ptr = nullptr;
    ~PinnedBuf() {
        if (ptr) cudaFreeHost(ptr);
    }
};

#define PB_CHECK(expr)                         \
    do {                                       \
        const cudaError_t pbErr = (expr);      \
        if (pbErr != cudaSuccess) return pbErr; \
    } while (0)

inline unsigned blocksFor(size_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

bool validSpec(const BodySpec& spec, std::string* err) {
    if (spec.archetype < 0 || spec.archetype > 5) {
        *err = "archetype must be 0..5";
        return false;
    }
    if (!(spec.massKg > 0.0)) {                    // planet_builder.cpp:402-404
        *err = "massKg must be positive";
        return false;
    }
    return true;
}

// PlanetBuilder::solveHydrostatic1D (planet_builder.cpp:398-473).
bool solveHydrostatic(const BodySpec& spec, std::vector<Sample>& profile, double& radiusM, double& pcPa,
                      std::string* err) {
    if (!validSpec(spec, err)) return false;
    const Composition& comp = kComp[spec.archetype];
    const double pSurf = (spec.archetype == kGasGiant) ? 1.0e5 : 0.0;
    double invRho = 0.0;
    for (int i = 0; i < comp.layers; ++i) {
        double rho0 = till(comp.mat[i]).rho0;
        if (comp.mat[i] == kHydrogenHelium) rho0 = 600.0;
        invRho += comp.frac[i] / stdMax(rho0, 1.0);
    }
    const double rhoEst = 1.0 / stdMax(invRho, 1.0e-6);
    double rEst = std::cbrt((3.0 * spec.massKg) / (4.0 * kPi * rhoEst));
    if (spec.archetype == kGasGiant) rEst = stdMax(rEst, 6.5e7);
    const double dr = stdMax(rEst / 800.0, 1.0e2);
    const double pEst = (3.0 * kGSi * spec.massKg * spec.massKg) / (8.0 * kPi * rEst * rEst * rEst * rEst);
    auto shoot = [&](double pc, std::vector<Sample>* rec) { return Shooter(spec, pc, pSurf, dr).run(rec); };

    double logLo = std::log(stdMax(pSurf + 1.0e4, 1.0e-3 * pEst));
    double logHi = std::log(stdMax(pSurf + 1.0e6, 1.0e3 * pEst));
    for (int i = 0; i < 20; ++i) {
        const Shot s = shoot(std::exp(logLo), nullptr);
        if (!s.capped && s.mass <= spec.massKg) break;
        logLo -= 2.0;
    }
    for (int i = 0; i < 20; ++i) {
        const Shot s = shoot(std::exp(logHi), nullptr);
        if (s.capped || s.mass >= spec.massKg) break;
        logHi += 2.0;
    }
    double logMid = 0.5 * (logLo + logHi);
    for (int it = 0; it < 60; ++it) {
        logMid = 0.5 * (logLo + logHi);
        const Shot s = shoot(std::exp(logMid), nullptr);
        const double rel = (s.mass - spec.massKg) / spec.massKg;
        if (!s.capped && std::abs(rel) <= 1.0e-6) break;
        if (s.capped || s.mass > spec.massKg) {
            logHi = logMid;
        } else {
            logLo = logMid;
        }
        if (logHi - logLo < 1.0e-12) break;
    }
    pcPa = std::exp(logMid);
    profile.clear();
    profile.reserve(1500);
    radiusM = shoot(pcPa, &profile).radius;
    if (profile.empty()) {
        *err = "hydrostatic solver returned an empty profile";
        return false;
    }
    return true;
}

// Shell plan of one body (planet_builder.cpp:486-638) plus the per-shell
// constants of :656-673.  Shells with no particles are dropped (the engine
// skips them before drawing).
static void planShells(const BodySpec& spec, uint32_t n, const std::vector<Sample>& prof, double actualMass,
                       std::vector<ShellDev>& shells) {
    const Composition& comp = kComp[spec.archetype];
    const int L = comp.layers;
    uint32_t parts[3] = {0, 0, 0};
    double cumEnd[3] = {0.0, 0.0, 0.0};
    double cum = 0.0;
    uint32_t assigned = 0;
    for (int k = 0; k < L; ++k) {
        cum += comp.frac[k];
        cumEnd[k] = (k + 1 == L) ? actualMass : (cum * actualMass);
        if (k + 1 == L) {
            parts[k] = n - assigned;
        } else {
            uint32_t c = static_cast<uint32_t>(std::llround(comp.frac[k] * n));
            if (n >= static_cast<uint32_t>(L) && c == 0) c = 1;
            const uint32_t avail = n - assigned - ((n >= static_cast<uint32_t>(L)) ? static_cast<uint32_t>(L - 1 - k) : 0u);
            c = std::min(c, avail);
            parts[k] = c;
            assigned += c;
        }
    }
    const double nominalMass = actualMass / static_cast<double>(n);
    uint32_t first = 0;
    double mStart = 0.0;
    for (int k = 0; k < L; ++k) {
        const uint32_t nk = parts[k];
        const double mEnd = cumEnd[k];
        if (nk == 0) {
            mStart = mEnd;
            continue;
        }
        const double layerMass = stdMax(mEnd - mStart, 0.0);
        const double pMassKg = layerMass / static_cast<double>(nk);
        const double pMassPsu = pMassKg / kMUnit;
        const int mat = comp.mat[k];
        const Sample sIn = sampleAtMass(prof, mStart);
        const Sample sOut = sampleAtMass(prof, mEnd);

        // shell boundaries in enclosed mass, radial step ~ (m/rho)^(1/3)
        std::vector<double> bounds{mStart};
        double curM = mStart, curR = sIn.r;
        if (k == 0 && nk >= 2 && sOut.r > 0.0) {
            const double cM = stdMin(mStart + pMassKg, mEnd);
            const double cR = std::cbrt((3.0 * cM) / (4.0 * kPi * stdMax(sIn.rho, 1.0e-3)));
            if (cM < mEnd && cR < sOut.r) {
                bounds.push_back(cM);
                curM = cM;
                curR = cR;
            }
        }
        auto massAt = [&](double rT) {
            const auto it = std::lower_bound(prof.begin(), prof.end(), rT,
                                             [](const Sample& s, double v) { return s.r < v; });
            double m = mEnd;
            if (it != prof.end() && it != prof.begin()) {
                const Sample& hi = *it;
                const Sample& lo = *(it - 1);
                const double d = hi.r - lo.r;
                const double t = (d > 1.0e-30) ? stdClamp((rT - lo.r) / d, 0.0, 1.0) : 0.0;
                m = lo.M + t * (hi.M - lo.M);
            }
            return stdClamp(m, curM + 1.0e-9 * layerMass, mEnd);
        };
        while (curM < mEnd) {
            const Sample sC = sampleAtMass(prof, curM);
            const double spacing = std::cbrt(nominalMass / stdMax(sC.rho, 1.0e-3));
            const double stepR = (k == 0 && nk >= 64 && curR < 3.5 * spacing) ? (0.62 * spacing) : spacing;
            const double nextR = curR + stepR;
            if (nextR >= sOut.r - 0.35 * stepR) {
                bounds.push_back(mEnd);
                break;
            }
            const double nextM = massAt(nextR);
            bounds.push_back(nextM);
            if (nextM >= mEnd) break;
            curM = nextM;
            curR = nextR;
        }
        if (bounds.size() < 2) bounds.push_back(mEnd);
        if (bounds.size() == 2 && nk >= 128 && sOut.r > sIn.r) {
            // a thick single-shell crust is split into three radial sub-shells
            const double avgRho = stdMax(0.5 * (sIn.rho + sOut.rho), 1.0e-3);
            const double layerSpacing = std::cbrt(nominalMass / avgRho);
            if ((sOut.r - sIn.r) > 0.25 * layerSpacing) {
                bounds.assign(1, mStart);
                curM = mStart;
                for (int sub = 1; sub < 3; ++sub) {
                    const double fr = static_cast<double>(sub) / 3.0;
                    const double nextM = massAt(sIn.r + fr * (sOut.r - sIn.r));
                    if (nextM > curM && nextM < mEnd) {
                        bounds.push_back(nextM);
                        curM = nextM;
                    }
                }
                bounds.push_back(mEnd);
            }
        }

        // particle counts per shell: floor of the mass share, then largest
        // remainders (the engine's std::sort order, the same call here)
        const size_t S = bounds.size() - 1;
        std::vector<uint32_t> counts(S, 0);
        std::vector<double> rem(S, 0.0);
        uint32_t sum = 0;
        for (size_t s = 0; s < S; ++s) {
            const double dm = bounds[s + 1] - bounds[s];
            const double exact = (layerMass > 0.0) ? (static_cast<double>(nk) * (dm / layerMass)) : 0.0;
            const uint32_t fl = static_cast<uint32_t>(std::floor(exact));
            counts[s] = fl;
            rem[s] = exact - static_cast<double>(fl);
            sum += fl;
        }
        if (sum < nk) {
            std::vector<size_t> idx(S);
            std::iota(idx.begin(), idx.end(), 0);
            std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return rem[a] > rem[b]; });
            for (uint32_t r = 0; r < nk - sum; ++r) counts[idx[r % S]] += 1;
        }

        const Till& t = till(mat);
        for (size_t s = 0; s < S; ++s) {
            const uint32_t ns = counts[s];
            if (ns == 0) continue;
            const double mMid = 0.5 * (bounds[s] + bounds[s + 1]);
            const Sample smp = sampleAtMass(prof, mMid);
            const double rShell = (s == 0 && k == 0 && ns == 1) ? 0.0 : smp.r;
            const double rho = stdMax(smp.rho, 1.0e-3);
            double uSi = 0.0, pSi = 0.0;
            stateFromRhoTemp(mat, rho, smp.T, uSi, pSi);
            const double rhoPsu = rho / kRhoUnit;
            ShellDev sh{};
            sh.rPsu = rShell / kLUnit;
            sh.epsMin = t.epsFailMin;
            sh.mass = static_cast<float>(pMassPsu);
            sh.h0 = static_cast<float>(1.2 * std::cbrt(pMassPsu / rhoPsu));
            sh.rho = static_cast<float>(rhoPsu);
            sh.u = static_cast<float>(uSi / kUUnit);
            sh.tempK = static_cast<float>(smp.T);
            sh.first = first;
            sh.count = ns;
            sh.mat = static_cast<uint32_t>(mat);
            shells.push_back(sh);
            first += ns;
        }
        mStart = mEnd;
    }
}

cudaError_t buildOnDevice(const BodySpec& spec, uint32_t n, uint8_t bodyId, uint32_t gridRes, uint64_t seed,
                          const AstraeaParticles& p, uint32_t offset, DevStatus* status, uint32_t spinLimit,
                          cudaStream_t st, BuildResult* out, std::string* err) {
    std::vector<Sample> prof;
    double radius = 0.0, pc = 0.0;
    if (!solveHydrostatic(spec, prof, radius, pc, err)) return cudaErrorInvalidValue;
    const double actualMass = prof.back().M;
    std::vector<ShellDev> shells;
    planShells(spec, n, prof, actualMass, shells);
    if (shells.empty() || shells.back().first + shells.back().count != n) {
        *err = "shell plan does not cover the particle count";
        return cudaErrorInvalidValue;
    }

    // The engine's stream (planet_builder.cpp:516-517, 671, 711): per shell,
    // three rotation uniforms, then one uniform per particle.  The host
    // draws it into pinned chunks; each full chunk is copied and placed on
    // the stream while the host draws the next.  A shell's row (with its
    // rotation) goes to the device with the first chunk that reaches it.
    std::mt19937_64 rng(seed ^ (static_cast<uint64_t>(bodyId) * 0x9e3779b97f4a7c15ULL));
    std::uniform_real_distribution<double> u01(1.0e-6, 1.0 - 1.0e-6);
    const uint32_t chunk = std::min(1u << 20, n);
    const uint32_t S = static_cast<uint32_t>(shells.size());
    PinnedBuf stage[2];
    ShellDev* table = nullptr;
    DevBuf<double> dDraws[2];
    DevBuf<ShellDev> dShells;
    cudaEvent_t done[2] = {nullptr, nullptr};
    struct Cleanup {                               // runs before the buffers are freed
        cudaStream_t st;
        cudaEvent_t* ev;
        ShellDev** table;
        ~Cleanup() {
            cudaStreamSynchronize(st);
            for (int i = 0; i < 2; ++i)
                if (ev[i]) cudaEventDestroy(ev[i]);
            if (*table) cudaFreeHost(*table);
        }
    } cleanup{st, done, &table};
    for (int b = 0; b < 2; ++b) {
        PB_CHECK(cudaMallocHost(&stage[b].ptr, chunk * sizeof(double)));
        PB_CHECK(dDraws[b].alloc(chunk));
        PB_CHECK(cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
    }
    PB_CHECK(cudaMallocHost(&table, S * sizeof(ShellDev)));
    std::copy(shells.begin(), shells.end(), table);
    PB_CHECK(dShells.alloc(S));
    const double golden = kPi * (3.0 - std::sqrt(5.0));
    const double spinT = spec.spinOmegaRadS * kTUnit;

    uint32_t rowsUp = 0, chunkStart = 0, fill = 0, chunkIdx = 0;
    auto flush = [&](uint32_t rowsReady) -> cudaError_t {
        const int b = chunkIdx & 1;
        if (rowsReady > rowsUp) {
            PB_CHECK(cudaMemcpyAsync(dShells.ptr + rowsUp, table + rowsUp, (rowsReady - rowsUp) * sizeof(ShellDev),
                                     cudaMemcpyHostToDevice, st));
            rowsUp = rowsReady;
        }
        PB_CHECK(cudaMemcpyAsync(dDraws[b].ptr, stage[b].ptr, fill * sizeof(double), cudaMemcpyHostToDevice, st));
        placeKernel<<<blocksFor(fill, 256), 256, 0, st>>>(p, offset, bodyId, dShells.ptr, rowsUp, dDraws[b].ptr,
                                                          chunkStart, chunkStart + fill, golden, spinT);
        PB_CHECK(cudaGetLastError());
        PB_CHECK(cudaEventRecord(done[b], st));
        chunkStart += fill;
        fill = 0;
        ++chunkIdx;
        if (chunkIdx >= 2) PB_CHECK(cudaEventSynchronize(done[chunkIdx & 1]));   // that stage is free again
        return cudaSuccess;
    };
    for (uint32_t s = 0; s < S; ++s) {
        randomRotation(rng, table[s].rot);
        for (uint32_t k = 0; k < table[s].count; ++k) {
            stage[chunkIdx & 1].ptr[fill++] = u01(rng);
            if (fill == chunk) PB_CHECK(flush(s + 1));
        }
    }
    if (fill > 0) PB_CHECK(flush(S));

    uint32_t tracers = 0;
    const uint32_t T = (spec.archetype == kLivingTerra && gridRes > 0) ? 6u * gridRes * gridRes : 0u;
    if (T > 0 && n >= T) {
        DevBuf<uint64_t> keysA, keysB;
        DevBuf<uint32_t> valsA, valsB, words;
        DevBuf<float> radii;
        PB_CHECK(keysA.alloc(n));
        PB_CHECK(keysB.alloc(n));
        PB_CHECK(valsA.alloc(n));
        PB_CHECK(valsB.alloc(n));
        PB_CHECK(radii.alloc(n));
        PB_CHECK(words.alloc(4));
        PB_CHECK(cudaMemsetAsync(words.ptr, 0, 4 * sizeof(uint32_t), st));
        tracerKeysKernel<<<blocksFor(n, 256), 256, 0, st>>>(p, offset, n, keysA.ptr, valsA.ptr, radii.ptr, words.ptr);
        PB_CHECK(cudaGetLastError());
        uint32_t maxTiles = 0;
        const size_t sw = sortScratchWords(n, &maxTiles);
        DevBuf<uint32_t> sortScratch;
        PB_CHECK(sortScratch.alloc(sw));
        bool inA = true;
        PB_CHECK(radixSortPairs(keysA.ptr, valsA.ptr, keysB.ptr, valsB.ptr, n, 33, sortScratch.ptr, sw, maxTiles,
                                status, spinLimit, KeySource::Array, nullptr, &inA, st));
        const uint32_t* list = inA ? valsA.ptr : valsB.ptr;
        uint32_t nCand = 0;
        PB_CHECK(cudaMemcpyAsync(&nCand, words.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PB_CHECK(cudaStreamSynchronize(st));
        const uint32_t L = std::max(nCand, T);     // fallback fills the list up to T in particle order
        const uint32_t minPool = std::min(L, 3u * T);
        uint32_t cut = L;
        PB_CHECK(cudaMemcpyAsync(words.ptr + 1, &cut, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        if (L > minPool) {
            poolCutKernel<<<blocksFor(L - minPool, 256), 256, 0, st>>>(p, offset, list, radii.ptr, minPool, L,
                                                                       words.ptr + 1);
            PB_CHECK(cudaGetLastError());
        }
        PB_CHECK(cudaMemcpyAsync(&cut, words.ptr + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PB_CHECK(cudaStreamSynchronize(st));
        const uint32_t P = std::max(cut, T);
        DevBuf<float3> candN;
        DevBuf<unsigned long long> best;
        DevBuf<uint8_t> used, filled;
        PB_CHECK(candN.alloc(P));
        PB_CHECK(best.alloc(T));
        PB_CHECK(used.alloc(P));
        PB_CHECK(filled.alloc(T));
        PB_CHECK(cudaMemsetAsync(best.ptr, 0, T * sizeof(unsigned long long), st));
        PB_CHECK(cudaMemsetAsync(used.ptr, 0, P, st));
        PB_CHECK(cudaMemsetAsync(words.ptr + 2, 0, 2 * sizeof(uint32_t), st));
        binOfferKernel<<<blocksFor(P, 256), 256, 0, st>>>(p, offset, list, radii.ptr, P, gridRes, candN.ptr, best.ptr);
        PB_CHECK(cudaGetLastError());
        binAssignKernel<<<blocksFor(T, 256), 256, 0, st>>>(p, offset, list, radii.ptr, candN.ptr, best.ptr, T,
                                                           used.ptr, filled.ptr, words.ptr + 2);
        PB_CHECK(cudaGetLastError());
        binFillKernel<<<1, kFillThreads, 0, st>>>(p, offset, list, radii.ptr, candN.ptr, P, gridRes, T, used.ptr,
                                                  filled.ptr, words.ptr + 2);
        PB_CHECK(cudaGetLastError());
        PB_CHECK(cudaMemcpyAsync(&tracers, words.ptr + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PB_CHECK(cudaStreamSynchronize(st));
        if (tracers < T) {
            // renumber in particle order: gather the tracer particles, sort
            tracerPidKernel<<<blocksFor(n, 256), 256, 0, st>>>(p, offset, n, keysA.ptr, valsA.ptr, words.ptr + 3);
            PB_CHECK(cudaGetLastError());
            bool inA2 = true;
            PB_CHECK(radixSortPairs(keysA.ptr, valsA.ptr, keysB.ptr, valsB.ptr, tracers, 32, sortScratch.ptr, sw,
                                    maxTiles, status, spinLimit, KeySource::Array, nullptr, &inA2, st));
            tracerRenumberKernel<<<blocksFor(tracers, 256), 256, 0, st>>>(p, offset, inA2 ? valsA.ptr : valsB.ptr,
                                                                          tracers);
            PB_CHECK(cudaGetLastError());
            PB_CHECK(cudaStreamSynchronize(st));
        }
    }
    out->radiusM = radius;
    out->massKg = actualMass;
    out->pcPa = pc;
    out->tracerCount = tracers;
    out->profileCount = static_cast<uint32_t>(prof.size());
    out->shellCount = static_cast<uint32_t>(shells.size());
    return cudaSuccess;
}

}  // namespace planet
}  // namespace astraea_gb300
