// oracle.cpp -- CPU restatement of the ASTRAEA per-step physics path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GB300 kernels
// and the CPU baseline timed by bench.py; nothing in the product library links
// or calls it.  It restates engine/sph_gravity.cu (the reference kernels) and
// engine/eos.cu (the reference EOS) of Ananasjik/astraea-impact-sim function by
// function, keeping the reference's floating-point expression order, its
// warp-wide traversal semantics (groups of 32 consecutive sorted particles,
// a node is opened for the whole group if any member needs it), and its
// per-lane summation order (depth-first, left child first).  Compile with
// -ffp-contract=off so no multiply-add is fused.
//
// Extra "truth" entry points evaluate the same physics in FP64: a direct-sum
// gravity (the N^2 check of tests/cpp/test_gravity_sph.cpp:366-378) and the
// SPH passes instantiated with double arithmetic.
//
// The particle and BVH descriptors are the C-ABI structs of
// include/astraea_gb300.h, here holding HOST pointers.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <random>
#include <vector>

#include "astraea_gb300.h"

namespace {

constexpr int kGroup = 32;            // warp width of the reference traversal
constexpr int kStackSize = 192;       // engine/sph_gravity.cu:22
constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;
constexpr float kGPsuF = 66.7430f;    // engine/units.hpp:27 (float of G_PSU)
constexpr double kGPsuD = 6.67430e-11 * 1.0e24 * 1.0e3 * 1.0e3 / (1.0e6 * 1.0e6 * 1.0e6);
constexpr double kSigmaSB = 5.670374419e-8;   // engine/units.hpp:6

// ---------------------------------------------------------------- EOS ----
// Restates engine/eos.cu.  Table values are the published constants in
// engine/eos.cu:10-116 (Tillotson 1962 / Melosh 1989, Benz & Asphaug 1999,
// Allen 1967, polytrope n=1, Jutzi 2008).
struct MatParams {
    double rho0, a, b, A, B, E0, Eiv, Ecv, alpha, beta, cv, tMelt, tRef, mu, Y0, epsFailMin, kH2, gamma;
};
const MatParams kMat[5] = {
    {7800.0, 0.5, 1.5, 1.28e11, 1.05e11, 9.50e6, 2.40e6, 8.67e6, 5.0, 5.0, 449.0, 1811.0, 293.0, 7.70e10, 6.80e8, 1.0e-3, 0.0, 1.0},
    {2680.0, 0.5, 1.3, 1.80e10, 1.80e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 790.0, 1600.0, 293.0, 2.20e10, 3.50e9, 1.0e-4, 0.0, 1.0},
    {1000.0, 0.7, 0.15, 2.18e9, 1.325e10, 7.00e6, 4.19e5, 2.68e6, 10.0, 5.0, 4184.0, 273.15, 273.15, 3.50e9, 1.00e7, 5.0e-4, 0.0, 1.0},
    {0.178, 0.4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 8260.0, 0.0, 0.0, 0.0, 0.0, 1.0, 2.08e5, 1.4},
    {2000.0, 0.5, 1.3, 1.20e10, 1.20e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 800.0, 1500.0, 293.0, 8.00e9, 5.00e7, 5.0e-5, 0.0, 1.0},
};
constexpr int kHH = 3;

inline int matIndex(int m) { return (m < 0 || m > 4) ? 1 : m; }   // eos.cu:271-275

// engine/eos.cu:283-318
double coldEnergy(int mat, double rho) {
    const MatParams& p = kMat[matIndex(mat)];
    rho = rho > 0.0 ? rho : 0.0;
    if (matIndex(mat) == kHH) return p.kH2 * rho;
    const double rho0 = p.rho0 / 1.0e6;
    const double eta = rho / rho0;
    if (eta <= 1.0) return 0.0;
    const double mu = eta - 1.0;
    const double A = p.A / 1.0e12, B = p.B / 1.0e12;
    double ta, tb;
    if (mu < 1.0e-5) {
        const double m2 = mu * mu, m3 = m2 * mu, m4 = m3 * mu, m5 = m4 * mu;
        ta = 0.5 * m2 - (2.0 / 3.0) * m3 + 0.75 * m4 - 0.8 * m5;
        tb = (1.0 / 3.0) * m3 - 0.5 * m4 + 0.6 * m5;
    } else {
        const double le = std::log1p(mu);
        ta = le - (mu / eta);
        tb = (mu * (2.0 + mu)) / eta - 2.0 * le;
    }
    return (A * ta + B * tb) / rho0;
}

struct PDeriv { double p, dpdrho, dpdu; bool damagedTension; };

// engine/eos.cu:136-176 (compressed / cold branch)
PDeriv tillotsonCompressed(const MatParams& p, double rho, double rho0, double eta, double mu, double uE, double dmg) {
    const double A = p.A / 1.0e12, B = p.B / 1.0e12, E0 = p.E0 / 1.0e6;
    const double bEff = (mu >= 0.0) ? B : 0.0;
    const double den = E0 * eta * eta;
    const double ratio = (den > 1.0e-30) ? (uE / den) : 1.0e30;
    const double w = ratio + 1.0;
    const double iw = 1.0 / w;
    const double wm1w2 = (ratio > 1.0e15) ? 0.0 : (ratio * iw * iw);
    PDeriv r;
    r.p = (p.a + p.b * iw) * rho * uE + A * mu + bEff * mu * mu;
    r.dpdrho = (p.a + p.b * iw) * uE + 2.0 * p.b * uE * wm1w2 + (A + 2.0 * bEff * mu) / rho0;
    r.dpdu = (p.a + p.b * iw * iw) * rho;
    r.damagedTension = false;
    if (r.p < 0.0 && dmg > 0.0) {
        const double keep = 1.0 - dmg;
        r.p *= keep; r.dpdrho *= keep; r.dpdu *= keep;
        r.damagedTension = true;
    }
    return r;
}

// engine/eos.cu:178-227 (expanded / hot branch)
PDeriv tillotsonExpanded(const MatParams& p, double rho, double rho0, double eta, double mu, double uE) {
    const double A = p.A / 1.0e12, E0 = p.E0 / 1.0e6;
    const double x = 1.0 / eta - 1.0;
    const double ax2 = p.alpha * x * x;
    const double bx = p.beta * x;
    const double eA = (ax2 < 700.0) ? std::exp(-ax2) : 0.0;
    PDeriv r;
    r.damagedTension = false;
    if (eA == 0.0) {
        r.p = p.a * rho * uE; r.dpdrho = p.a * uE; r.dpdu = p.a * rho;
        return r;
    }
    const double eB = (bx < 700.0) ? std::exp(-bx) : 0.0;
    const double den = E0 * eta * eta;
    const double ratio = (den > 1.0e-30) ? (uE / den) : 1.0e30;
    const double w = ratio + 1.0;
    const double iw = 1.0 / w;
    const double wm1w2 = (ratio > 1.0e15) ? 0.0 : (ratio * iw * iw);
    const double ideal = p.a * rho * uE;
    const double inner = (p.b * rho * uE * iw) + A * mu * eB;
    const double pe = ideal + inner * eA;
    const double r0r2 = rho0 / (rho * rho);
    const double expDrho = (eB > 0.0) ? ((A / rho0 + A * mu * p.beta * r0r2) * eB) : 0.0;
    r.p = pe;
    r.dpdrho = p.a * uE + eA * (p.b * uE * iw + 2.0 * p.b * uE * wm1w2 + expDrho) + 2.0 * p.alpha * x * r0r2 * (pe - ideal);
    r.dpdu = (p.a + p.b * eA * iw * iw) * rho;
    return r;
}

// engine/eos.cu:229-267
uint8_t phaseOf(int mat, const MatParams& p, double rho, double u, double T) {
    mat = matIndex(mat);
    if (mat == kHH) return (T > 10000.0) ? 3 : 5;
    const double rhoKg = rho * 1.0e6;
    const double ecv = p.Ecv / 1.0e6;
    if (mat == 2) {
        if (T > 15000.0) return 3;
        if (u >= ecv || (T > 647.0 && rhoKg < 322.0)) return 2;
        if (T >= 273.15) return 4;
        return 0;
    }
    if (T > 12000.0) return 3;
    if (u >= ecv && rhoKg < 0.8 * p.rho0) return 2;
    if (T >= p.tMelt) return 1;
    return 0;
}

struct EosOut { float p, cs, T; uint8_t phase; };

// engine/eos.cu:320-388
EosOut evaluateEos(int mat, float rhoIn, float uIn, float dIn) {
    const int mi = matIndex(mat);
    const MatParams& p = kMat[mi];
    const double rho = std::max(static_cast<double>(rhoIn), 1.0e-12);
    const double u = static_cast<double>(uIn);
    double dmg = static_cast<double>(dIn);
    dmg = dmg < 0.0 ? 0.0 : (dmg > 1.0 ? 1.0 : dmg);
    const double cv = p.cv / 1.0e6;
    const double uCold = coldEnergy(mi, rho);
    if (mi == kHH) {
        const double uTh = std::max(0.0, u - uCold);
        const double T = std::max(3.0, uTh / cv);
        const double P = p.kH2 * rho * rho + (p.gamma - 1.0) * rho * uTh;
        const double cs2 = 2.0 * p.kH2 * rho + p.gamma * (p.gamma - 1.0) * uTh;
        const double cs = std::max(0.05, std::sqrt(std::max(0.0, cs2)));
        return {static_cast<float>(P), static_cast<float>(cs), static_cast<float>(T), phaseOf(mi, p, rho, u, T)};
    }
    const double rho0 = p.rho0 / 1.0e6;
    const double eta = rho / rho0;
    const double mu = eta - 1.0;
    const double T = std::max(3.0, (u - uCold) / cv);
    const double uE = uCold + std::max(0.0, u - uCold - cv * p.tRef);
    const double Eiv = p.Eiv / 1.0e6, Ecv = p.Ecv / 1.0e6, A = p.A / 1.0e12;
    PDeriv r;
    if (eta >= 1.0 || uE < Eiv) {
        r = tillotsonCompressed(p, rho, rho0, eta, mu, uE, dmg);
    } else if (uE >= Ecv) {
        r = tillotsonExpanded(p, rho, rho0, eta, mu, uE);
    } else {
        const PDeriv c = tillotsonCompressed(p, rho, rho0, eta, mu, uE, dmg);
        const PDeriv e = tillotsonExpanded(p, rho, rho0, eta, mu, uE);
        const double den = std::max(1.0e-30, Ecv - Eiv);
        double f = (uE - Eiv) / den;
        f = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
        r.p = (1.0 - f) * c.p + f * e.p;
        r.dpdrho = (1.0 - f) * c.dpdrho + f * e.dpdrho;
        r.dpdu = (1.0 - f) * c.dpdu + f * e.dpdu + (e.p - c.p) / den;
        r.damagedTension = c.damagedTension;
    }
    const double cs2 = r.dpdrho + (r.p / (rho * rho)) * r.dpdu;
    const bool condensed = (eta >= 1.0) || (uE < Eiv && rho >= 0.9 * rho0 && !r.damagedTension);
    const double cMin = condensed ? std::max(0.05, std::sqrt(A / rho0)) : 0.05;
    const double cs = std::max(cMin, std::sqrt(std::max(0.0, cs2)));
    return {static_cast<float>(r.p), static_cast<float>(cs), static_cast<float>(T), phaseOf(mi, p, rho, u, T)};
}

// --------------------------------------------------- kernel constants ----
// engine/sph_gravity.cu:27-73: u_ref = cv * 300 K, and the strength table.
inline float u0RefPsu(int m) { return static_cast<float>((kMat[matIndex(m)].cv * 300.0) / 1.0e6); }
struct Strength { float mu, tMelt, K, Y0; };
inline Strength strengthOf(int m) {
    switch (matIndex(m)) {
        case 0: return {static_cast<float>(7.70e10 / 1e12), 1811.0f, static_cast<float>(1.28e11 / 1e12), static_cast<float>(6.80e8 / 1e12)};
        case 1: return {static_cast<float>(2.20e10 / 1e12), 1600.0f, static_cast<float>(1.80e10 / 1e12), static_cast<float>(3.50e9 / 1e12)};
        case 2: return {static_cast<float>(3.50e9 / 1e12), 273.15f, static_cast<float>(2.18e9 / 1e12), static_cast<float>(1.00e7 / 1e12)};
        case 3: return {0.0f, 0.0f, 0.0f, 0.0f};
        default: return {static_cast<float>(8.00e9 / 1e12), 1500.0f, static_cast<float>(1.20e10 / 1e12), static_cast<float>(5.00e7 / 1e12)};
    }
}

// ------------------------------------------------------ small helpers ----
inline uint32_t toOrdered(float f) {
    uint32_t u; std::memcpy(&u, &f, 4);
    const uint32_t mask = static_cast<uint32_t>(-static_cast<int32_t>(u >> 31)) | 0x80000000u;
    return u ^ mask;
}
inline float fromOrdered(uint32_t u) {
    const uint32_t mask = ((u >> 31) - 1u) | 0x80000000u;
    u ^= mask; float f; std::memcpy(&f, &u, 4); return f;
}
inline uint64_t spread21(uint64_t v) {   // bit interleave, engine/sph_gravity.cu:151-159
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x001f00000000ffffULL;
    v = (v | (v << 16)) & 0x001f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}
inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

template <typename R> inline R wendland(R r, R H) {      // sph_gravity.cu:199-208
    if (r >= H || H <= R(0)) return R(0);
    const R q = r / H, omq = R(1) - q, omq2 = omq * omq;
    const R norm = R(21) / (R(2) * R(kPiD) * H * H * H);
    return norm * omq2 * omq2 * (R(1) + R(4) * q);
}
template <> inline float wendland<float>(float r, float H) {
    if (r >= H || H <= 0.0f) return 0.0f;
    const float q = r / H, omq = 1.0f - q, omq2 = omq * omq;
    const float norm = 21.0f / (2.0f * kPiF * H * H * H);
    return norm * omq2 * omq2 * (1.0f + 4.0f * q);
}
template <typename R> inline R wendlandGrad(R r, R H) {  // sph_gravity.cu:211-220
    if (r >= H || H <= R(0)) return R(0);
    const R q = r / H, omq = R(1) - q, H2 = H * H, H5 = H2 * H2 * H;
    return -(R(210) / (R(kPiD) * H5)) * omq * omq * omq;
}
template <> inline float wendlandGrad<float>(float r, float H) {
    if (r >= H || H <= 0.0f) return 0.0f;
    const float q = r / H, omq = 1.0f - q, H2 = H * H, H5 = H2 * H2 * H;
    return -(210.0f / (kPiF * H5)) * omq * omq * omq;
}
template <typename R> inline R balsara(R div, R cx, R cy, R cz, R cs, R h) {  // :222-228
    const R ad = std::fabs(div);
    const R ac = std::sqrt(cx * cx + cy * cy + cz * cz);
    const R den = ad + ac + R(1.0e-4f) * std::max(cs, R(0.05f)) / std::max(h, R(1.0e-6f));
    return ad / std::max(den, R(1.0e-30f));
}
inline float maxPrincipal(float P, float xx, float yy, float zz, float xy, float xz, float yz) {  // :230-254
    const float p2 = xx * xx + yy * yy + zz * zz + 2.0f * (xy * xy + xz * xz + yz * yz);
    if (p2 <= 1.0e-24f) return -P;
    const float q = std::sqrt(p2 * (1.0f / 6.0f));
    const float iq = 1.0f / q;
    const float bxx = xx * iq, byy = yy * iq, bzz = zz * iq, bxy = xy * iq, bxz = xz * iq, byz = yz * iq;
    const float det = bxx * (byy * bzz - byz * byz) - bxy * (bxy * bzz - byz * bxz) + bxz * (bxy * byz - byy * bxz);
    const float r = std::min(1.0f, std::max(-1.0f, 0.5f * det));
    const float phi = std::acos(r) * (1.0f / 3.0f);
    return -P + 2.0f * q * std::cos(phi);
}
inline float pointBoxDist2(float px, float py, float pz, float mnx, float mny, float mnz, float mxx, float mxy, float mxz) {
    const float dx = std::max(0.0f, std::max(mnx - px, px - mxx));
    const float dy = std::max(0.0f, std::max(mny - py, py - mxy));
    const float dz = std::max(0.0f, std::max(mnz - pz, pz - mxz));
    return dx * dx + dy * dy + dz * dz;
}
inline float effPressure(float P, uint8_t phase) { return phase != 0 ? std::max(P, 0.0f) : P; }

struct NodeBox { float mnx, mny, mnz, mxx, mxy, mxz, maxH, dNode, cx, cy, cz, m; };
inline NodeBox nodeBox(const AstraeaRadixBvh& b, int c) {
    NodeBox o;
    o.mnx = b.aabbMinX[c]; o.mny = b.aabbMinY[c]; o.mnz = b.aabbMinZ[c];
    o.mxx = b.aabbMaxX[c]; o.mxy = b.aabbMaxY[c]; o.mxz = b.aabbMaxZ[c];
    o.maxH = b.nodeMaxH[c];
    o.dNode = std::max(o.mxx - o.mnx, std::max(o.mxy - o.mny, o.mxz - o.mnz));
    o.cx = b.comX[c]; o.cy = b.comY[c]; o.cz = b.comZ[c]; o.m = b.nodeMass[c];
    return o;
}

int numGroups(uint32_t n) { return static_cast<int>((n + kGroup - 1) / kGroup); }

// Timing sample for the CPU baseline: tree-walking stages visit only groups
// g with g % g_groupStride == 0 (1 = all groups, the normal checker mode).
int g_groupStride = 1;

// |d|^2 at the engine's decision points (the gravity member test, the SPH
// range tests, the dt candidate), rounded as the engine's compiled kernels
// round dx*dx + dy*dy + dz*dz: nvcc contracts it into fma(dz, dz, fma(dx, dx,
// dy*dy)) (form 1, the default).  Forms 0 (the unfused sequence (dx^2 + dy^2)
// + dz^2) and 2 (fma(dz, dz, fma(dy, dy, dx^2))) are kept so a test can show
// which form the reference kernels' results follow: on the 1M impact they
// take exactly form 1's gravity opening decisions.
int g_r2Form = 1;
inline float engineLen2(float dx, float dy, float dz) {
    if (g_r2Form == 1) return std::fma(dz, dz, std::fma(dx, dx, dy * dy));
    if (g_r2Form == 2) return std::fma(dz, dz, std::fma(dy, dy, dx * dx));
    return dx * dx + dy * dy + dz * dz;
}
// a*b + c as the engine's compiled kernel rounds it (one fma, form 1 and 2)
inline float engineMulAdd(float a, float b, float c) { return g_r2Form == 0 ? a * b + c : std::fma(a, b, c); }
inline bool skipGroup(int g) { return g_groupStride > 1 && (g % g_groupStride) != 0; }

// Depth-first walk shared by the SPH-style traversals: `open(c)` decides
// whether the group descends into internal node c; `leaf(j)` visits particle
// j.  The stack discipline (pop, left child then right child, push opened
// internal children, drop pushes past kStackSize) is that of the reference
// warp loops, e.g. engine/sph_gravity.cu:687-766.
template <class Open, class Leaf>
void walkGroup(const AstraeaRadixBvh& b, Open open, Leaf leaf) {
    int stack[kStackSize];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int ch[2] = {b.leftChild[node], b.rightChild[node]};
        for (int k = 0; k < 2; ++k) {
            const int c = ch[k];
            if (c < 0) {
                leaf(static_cast<uint32_t>(~c));
            } else if (open(c) && sp < kStackSize) {
                stack[sp++] = c;
            }
        }
    }
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- EOS API
void oracle_eos_batch(uint32_t n, const uint8_t* mat, const float* rho, const float* u, const float* dmg,
                      float* P, float* cs, float* T, uint8_t* phase) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
        const EosOut r = evaluateEos(mat[i], rho[i], u[i], dmg[i]);
        P[i] = r.p; cs[i] = r.cs; T[i] = r.T; phase[i] = r.phase;
    }
}
double oracle_cold_energy(int mat, double rho) { return coldEnergy(mat, rho); }

// --------------------------------------------------------- clear stats ----
// engine/sph_gravity.cu:624-641
void oracle_clear_stats(AstraeaParticles* p) {
    for (uint32_t i = 0; i < p->count; ++i) {
        p->accX[i] = p->accY[i] = p->accZ[i] = 0.0f;
        p->drhoDt[i] = 0.0f; p->duDt[i] = 0.0f; p->radPowerW[i] = 0.0f;
        p->dSXX[i] = p->dSYY[i] = p->dSZZ[i] = p->dSXY[i] = p->dSXZ[i] = p->dSYZ[i] = 0.0f;
        p->dDamageCbrtDt[i] = 0.0f; p->divV[i] = 0.0f;
        p->curlVX[i] = p->curlVY[i] = p->curlVZ[i] = 0.0f;
        p->shepardC[i] = 1.0f; p->surfFactor[i] = 0.0f; p->phiGrav[i] = 0.0f;
    }
}

// ------------------------------------------------------ bounds + Morton ----
// engine/sph_gravity.cu:258-361 (min/max are order independent, so a serial
// scan gives the same bounds as the block reduction + ordered-uint atomics).
void oracle_scene_bounds(uint32_t n, const float* x, const float* y, const float* z, float* out6) {
    uint32_t o[6] = {toOrdered(1.0e30f), toOrdered(1.0e30f), toOrdered(1.0e30f),
                     toOrdered(-1.0e30f), toOrdered(-1.0e30f), toOrdered(-1.0e30f)};
    float mn[3] = {1.0e30f, 1.0e30f, 1.0e30f}, mx[3] = {-1.0e30f, -1.0e30f, -1.0e30f};
    for (uint32_t i = 0; i < n; ++i) {
        mn[0] = std::fmin(mn[0], x[i]); mx[0] = std::fmax(mx[0], x[i]);
        mn[1] = std::fmin(mn[1], y[i]); mx[1] = std::fmax(mx[1], y[i]);
        mn[2] = std::fmin(mn[2], z[i]); mx[2] = std::fmax(mx[2], z[i]);
    }
    for (int k = 0; k < 3; ++k) {
        o[k] = std::min(o[k], toOrdered(mn[k]));
        o[3 + k] = std::max(o[3 + k], toOrdered(mx[k]));
    }
    for (int k = 0; k < 6; ++k) out6[k] = fromOrdered(o[k]);
}

void oracle_morton(uint32_t n, const float* x, const float* y, const float* z, const float* b6, uint64_t* codes) {
    const float minX = b6[0], minY = b6[1], minZ = b6[2];
    const float sx = b6[3] - minX, sy = b6[4] - minY, sz = b6[5] - minZ;
    const float ix = (sx > 1.0e-6f) ? (2097151.0f / sx) : 0.0f;
    const float iy = (sy > 1.0e-6f) ? (2097151.0f / sy) : 0.0f;
    const float iz = (sz > 1.0e-6f) ? (2097151.0f / sz) : 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const float fx = std::fmin(std::fmax((x[i] - minX) * ix, 0.0f), 2097151.0f);
        const float fy = std::fmin(std::fmax((y[i] - minY) * iy, 0.0f), 2097151.0f);
        const float fz = std::fmin(std::fmax((z[i] - minZ) * iz, 0.0f), 2097151.0f);
        const uint64_t qx = static_cast<uint32_t>(fx), qy = static_cast<uint32_t>(fy), qz = static_cast<uint32_t>(fz);
        codes[i] = (spread21(qx) << 2) | (spread21(qy) << 1) | spread21(qz);
    }
}

// Stable sort by key (ties keep ascending input index), the semantics of
// cub::DeviceRadixSort::SortPairs over bits [0, 63) used at
// engine/sph_gravity.cu:2042-2046 (all Morton codes are < 2^63).
void oracle_sort_pairs(uint32_t n, const uint64_t* keys, uint64_t* keysSorted, uint32_t* perm) {
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    for (uint32_t i = 0; i < n; ++i) { perm[i] = idx[i]; keysSorted[i] = keys[idx[i]]; }
}

// Karras 2012 binary radix tree, engine/sph_gravity.cu:173-187 + 477-528.
static inline int deltaK(const uint64_t* c, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (c[i] != c[j]) return clz64(c[i] ^ c[j]);
    return 64 + clz32(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
}
void oracle_karras(uint32_t nU, const uint64_t* codes, int32_t* left, int32_t* right, int32_t* parent) {
    const int n = static_cast<int>(nU);
    if (n == 1) { parent[0] = -1; return; }
    for (int i = 0; i + 1 < n; ++i) {
        const int d = (deltaK(codes, n, i, i + 1) - deltaK(codes, n, i, i - 1) >= 0) ? 1 : -1;
        const int dMin = deltaK(codes, n, i, i - d);
        int lmax = 2;
        while (deltaK(codes, n, i, i + lmax * d) > dMin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (deltaK(codes, n, i, i + (l + t) * d) > dMin) l += t;
        const int j = i + l * d;
        const int dNode = deltaK(codes, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (deltaK(codes, n, i, i + (s + t) * d) > dNode) s += t;
        } while (t > 1);
        const int g = i + s * d + ((d < 0) ? d : 0);
        const int first = std::min(i, j), last = std::max(i, j);
        left[i] = (first == g) ? ~g : g;
        right[i] = (last == g + 1) ? ~(g + 1) : (g + 1);
        parent[(first == g) ? (n - 1 + g) : g] = i;
        parent[(last == g + 1) ? (n - 1 + g + 1) : (g + 1)] = i;
    }
    parent[0] = -1;
}

// engine/sph_gravity.cu:363-430 (gather) + 1745-1784 (pointer swap).
#define ORACLE_FIELDS_F32(X) X(posX) X(posY) X(posZ) X(velX) X(velY) X(velZ) X(velHalfX) X(velHalfY) X(velHalfZ) \
    X(accX) X(accY) X(accZ) X(mass) X(h) X(h0) X(rho) X(drhoDt) X(pressure) X(soundSpeed) X(u) X(duDt) X(tempK)     \
    X(radPowerW) X(sXX) X(sYY) X(sZZ) X(sXY) X(sXZ) X(sYZ) X(dSXX) X(dSYY) X(dSZZ) X(dSXY) X(dSXZ) X(dSYZ)          \
    X(damage) X(damageCbrt) X(dDamageCbrtDt) X(epsFail) X(divV) X(curlVX) X(curlVY) X(curlVZ) X(shepardC)          \
    X(surfFactor) X(phiGrav) X(tracerRestRadiusPsu) X(tracerRestNormalX) X(tracerRestNormalY) X(tracerRestNormalZ)
#define ORACLE_FIELDS_OTHER(X) X(materialId) X(phaseId) X(bodyId) X(originalId) X(tracerIndex) X(tracerIsOcean)

void oracle_permute_swap(AstraeaParticles* p, AstraeaParticles* alt, const uint32_t* perm) {
    const uint32_t n = p->count;
#define GATHER(f) for (uint32_t i = 0; i < n; ++i) alt->f[i] = p->f[perm[i]];
    ORACLE_FIELDS_F32(GATHER) ORACLE_FIELDS_OTHER(GATHER)
#undef GATHER
#define SWAP(f) std::swap(p->f, alt->f);
    ORACLE_FIELDS_F32(SWAP) ORACLE_FIELDS_OTHER(SWAP)
#undef SWAP
    alt->count = p->count;
}

// Leaf init + bottom-up refit in FP32, engine/sph_gravity.cu:440-475, 531-620.
// A serial post-order pass computes exactly what the atomic second-arrival
// scheme computes (each node combines its two finished children once).
void oracle_refit(const AstraeaParticles* p, AstraeaRadixBvh* b, uint32_t* livingFlags) {
    const uint32_t n = p->count;
    livingFlags[0] = livingFlags[1] = 0u;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t L = n - 1 + i;
        const float x = p->posX[i], y = p->posY[i], z = p->posZ[i], m = p->mass[i], H = 2.0f * p->h[i];
        b->aabbMinX[L] = b->aabbMaxX[L] = x; b->aabbMinY[L] = b->aabbMaxY[L] = y; b->aabbMinZ[L] = b->aabbMaxZ[L] = z;
        b->nodeMass[L] = m; b->comX[L] = x; b->comY[L] = y; b->comZ[L] = z; b->nodeMaxH[L] = H;
        if (p->tracerIndex[i] >= 0) {
            livingFlags[0] = 1u;
            if (p->damage[i] < 0.8f) livingFlags[1] = 1u;
        }
    }
    if (n < 2) return;
    // iterative post-order over internal nodes
    std::vector<int> order;
    order.reserve(n);
    std::vector<int> st;
    st.push_back(0);
    while (!st.empty()) {
        const int v = st.back(); st.pop_back();
        order.push_back(v);
        if (b->leftChild[v] >= 0) st.push_back(b->leftChild[v]);
        if (b->rightChild[v] >= 0) st.push_back(b->rightChild[v]);
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const int v = *it;
        const int lc = b->leftChild[v], rc = b->rightChild[v];
        const int l = lc < 0 ? static_cast<int>(n - 1) + ~lc : lc;
        const int r = rc < 0 ? static_cast<int>(n - 1) + ~rc : rc;
        const float mnx = std::fmin(b->aabbMinX[l], b->aabbMinX[r]);
        const float mny = std::fmin(b->aabbMinY[l], b->aabbMinY[r]);
        const float mnz = std::fmin(b->aabbMinZ[l], b->aabbMinZ[r]);
        const float mxx = std::fmax(b->aabbMaxX[l], b->aabbMaxX[r]);
        const float mxy = std::fmax(b->aabbMaxY[l], b->aabbMaxY[r]);
        const float mxz = std::fmax(b->aabbMaxZ[l], b->aabbMaxZ[r]);
        const float mh = std::fmax(b->nodeMaxH[l], b->nodeMaxH[r]);
        const float ml = b->nodeMass[l], mr = b->nodeMass[r], ms = ml + mr;
        float cx, cy, cz;
        if (ms > 0.0f) {
            // (ml cl + mr cr) / m as the engine's compiled kernel rounds it:
            // the sum contracted into fma(ml, cl, mr cr) (engineMulAdd)
            const float im = 1.0f / ms;
            cx = engineMulAdd(ml, b->comX[l], mr * b->comX[r]) * im;
            cy = engineMulAdd(ml, b->comY[l], mr * b->comY[r]) * im;
            cz = engineMulAdd(ml, b->comZ[l], mr * b->comZ[r]) * im;
        } else {
            cx = 0.5f * (b->comX[l] + b->comX[r]);
            cy = 0.5f * (b->comY[l] + b->comY[r]);
            cz = 0.5f * (b->comZ[l] + b->comZ[r]);
        }
        b->aabbMinX[v] = mnx; b->aabbMinY[v] = mny; b->aabbMinZ[v] = mnz;
        b->aabbMaxX[v] = mxx; b->aabbMaxY[v] = mxy; b->aabbMaxZ[v] = mxz;
        b->nodeMaxH[v] = mh; b->nodeMass[v] = ms; b->comX[v] = cx; b->comY[v] = cy; b->comZ[v] = cz;
    }
}

// Whole launchSortAndBuildBvh (engine/sph_gravity.cu:1996-2061) on host
// arrays; bvh must hold host arrays of the reference sizes.
void oracle_sort_and_build(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* b, float* bounds6Out) {
    const uint32_t n = p->count;
    if (n == 0) return;
    float b6[6];
    oracle_scene_bounds(n, p->posX, p->posY, p->posZ, b6);
    if (bounds6Out) std::memcpy(bounds6Out, b6, sizeof(b6));
    oracle_morton(n, p->posX, p->posY, p->posZ, b6, b->mortonCodes);
    for (uint32_t i = 0; i < n; ++i) b->indicesIn[i] = i;
    oracle_sort_pairs(n, b->mortonCodes, b->mortonCodesSorted, b->indicesSorted);
    oracle_permute_swap(p, alt, b->indicesSorted);
    oracle_karras(n, b->mortonCodesSorted, b->leftChild, b->rightChild, b->parent);
    uint32_t lf[2];
    oracle_refit(p, b, lf);
    if (b->livingFlags) { b->livingFlags[0] = lf[0]; b->livingFlags[1] = lf[1]; }
}

// ------------------------------------------------------------ SPH pass 1 ----
// engine/sph_gravity.cu:645-788, instantiated in float (reference) or double.
}  // extern "C"
template <typename R>
static void pass1Impl(AstraeaParticles* p, const AstraeaRadixBvh* b) {
    const uint32_t n = p->count;
    const int G = numGroups(n);
    std::vector<float> hNew(p->h, p->h + n);   // groups skipped by a timing sample keep h
#pragma omp parallel for schedule(dynamic, 4)
    for (int g = 0; g < G; ++g) {
        if (skipGroup(g)) continue;
        const uint32_t i0 = static_cast<uint32_t>(g) * kGroup;
        const int act = static_cast<int>(std::min<uint32_t>(kGroup, n - i0));
        R xi[kGroup], yi[kGroup], zi[kGroup], vx[kGroup], vy[kGroup], vz[kGroup], hi[kGroup], h0i[kGroup], Hi[kGroup], Hi2[kGroup];
        R shep[kGroup], nsX[kGroup] = {}, nsY[kGroup] = {}, nsZ[kGroup] = {};
        R gg[kGroup][9] = {};
        int cnt[kGroup];
        float Hi2f[kGroup], xf[kGroup], yf[kGroup], zf[kGroup];
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            xi[l] = p->posX[i]; yi[l] = p->posY[i]; zi[l] = p->posZ[i];
            xf[l] = p->posX[i]; yf[l] = p->posY[i]; zf[l] = p->posZ[i];
            vx[l] = p->velX[i]; vy[l] = p->velY[i]; vz[l] = p->velZ[i];
            const float hf = std::fmax(p->h[i], 1.0e-6f);
            const float Hf = 2.0f * hf;
            hi[l] = hf; h0i[l] = std::fmax(p->h0[i], 1.0e-6f);
            Hi[l] = Hf; Hi2f[l] = Hf * Hf; Hi2[l] = R(Hi2f[l]);
            const R mi = p->mass[i], rhoI = std::fmax(p->rho[i], 1.0e-9f);
            const R w0 = R(21) / (R(2) * R(kPiD) * Hi[l] * Hi[l] * Hi[l]);
            shep[l] = (sizeof(R) == 4) ? R((static_cast<float>(mi) / static_cast<float>(rhoI)) * (21.0f / (2.0f * kPiF * Hf * Hf * Hf)))
                                       : (mi / rhoI) * w0;
            cnt[l] = 1;
        }
        if (n >= 2) {
            walkGroup(*b,
                [&](int c) {
                    for (int l = 0; l < act; ++l)
                        if (pointBoxDist2(xf[l], yf[l], zf[l], b->aabbMinX[c], b->aabbMinY[c], b->aabbMinZ[c],
                                          b->aabbMaxX[c], b->aabbMaxY[c], b->aabbMaxZ[c]) <= Hi2f[l])
                            return true;
                    return false;
                },
                [&](uint32_t j) {
                    const float pxj = p->posX[j], pyj = p->posY[j], pzj = p->posZ[j];
                    for (int l = 0; l < act; ++l) {
                        const uint32_t i = i0 + l;
                        const float dxf = xf[l] - pxj, dyf = yf[l] - pyj, dzf = zf[l] - pzj;
                        const float r2f = engineLen2(dxf, dyf, dzf);
                        if (j == i || !(r2f < Hi2f[l])) continue;
                        ++cnt[l];
                        const R dx = xi[l] - R(pxj), dy = yi[l] - R(pyj), dz = zi[l] - R(pzj);
                        const R r2 = (sizeof(R) == 4) ? R(r2f) : dx * dx + dy * dy + dz * dz;
                        const R r = std::sqrt(r2);
                        const R vol = R(p->mass[j]) / R(std::fmax(p->rho[j], 1.0e-9f));
                        const R w = wendland<R>(r, Hi[l]);
                        shep[l] += vol * w;
                        nsX[l] -= vol * dx * w; nsY[l] -= vol * dy * w; nsZ[l] -= vol * dz * w;
                        const R gc = wendlandGrad<R>(r, Hi[l]);
                        const R gx = gc * dx, gy = gc * dy, gz = gc * dz;
                        const R dvx = R(p->velX[j]) - vx[l], dvy = R(p->velY[j]) - vy[l], dvz = R(p->velZ[j]) - vz[l];
                        R* G9 = gg[l];
                        G9[0] += vol * dvx * gx; G9[1] += vol * dvx * gy; G9[2] += vol * dvx * gz;
                        G9[3] += vol * dvy * gx; G9[4] += vol * dvy * gy; G9[5] += vol * dvy * gz;
                        G9[6] += vol * dvz * gx; G9[7] += vol * dvz * gy; G9[8] += vol * dvz * gz;
                    }
                });
        }
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            p->shepardC[i] = static_cast<float>(shep[l]);
            const R nn = std::sqrt(nsX[l] * nsX[l] + nsY[l] * nsY[l] + nsZ[l] * nsZ[l]);
            R fs = std::min(R(1), std::max(R(0), R(1.6f) * std::max(R(1) - shep[l], nn / hi[l]) - R(0.15f)));
            if (cnt[l] <= 2) fs = R(1);
            p->surfFactor[i] = static_cast<float>(fs);
            const R* G9 = gg[l];
            p->divV[i] = static_cast<float>(G9[0] + G9[4] + G9[8]);
            p->curlVX[i] = static_cast<float>(G9[7] - G9[5]);
            p->curlVY[i] = static_cast<float>(G9[2] - G9[6]);
            p->curlVZ[i] = static_cast<float>(G9[3] - G9[1]);
            const float ratio = 56.0f / static_cast<float>(cnt[l]);
            const float fac = std::fmin(1.08f, std::fmax(0.92f, std::cbrt(ratio)));
            hNew[i] = std::fmin(6.0f * static_cast<float>(h0i[l]), std::fmax(0.35f * static_cast<float>(h0i[l]), static_cast<float>(hi[l]) * fac));
        }
    }
    for (uint32_t i = 0; i < n; ++i) p->h[i] = hNew[i];
}
extern "C" {
void oracle_sph_pass1(AstraeaParticles* p, const AstraeaRadixBvh* b) { if (p->count) pass1Impl<float>(p, b); }
void oracle_sph_pass1_f64(AstraeaParticles* p, const AstraeaRadixBvh* b) { if (p->count) pass1Impl<double>(p, b); }

void oracle_evaluate_eos(AstraeaParticles* p) {
    oracle_eos_batch(p->count, p->materialId, p->rho, p->u, p->damage, p->pressure, p->soundSpeed, p->tempK, p->phaseId);
}

// --------------------------------------------------------- Barnes-Hut ----
// engine/sph_gravity.cu:810-961 (float), per group of 32.
// S6 == nullptr: the reference kernel.  Otherwise (the library's far-field
// mode 1) each accepted node also adds its quadrupole field, with S6 the
// node's central second moments {xx, yy, zz, xy, xz, yz} from
// oracle_node_moments: Q = 3 S - tr(S) I, r = x_i - COM, the softened 1/r of
// the monopole, a += G [Q r / r^5 - 5/2 (r.Q.r) r / r^7], phi -= G (r.Q.r) / (2 r^5).
}  // extern "C"

// R = float: the reference kernel's arithmetic.  R = double: the FP64 host
// path -- the same tree, the same float acceptance tests (so the same
// interaction set), each pair term and the sums in double.
template <typename R>
static void gravityImpl(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, const float* S6,
                        uint64_t* interactionsOut, uint32_t* groupCounts = nullptr) {
    const uint32_t n = p->count;
    if (n == 0) return;
    if (n == 1) { p->accX[0] = p->accY[0] = p->accZ[0] = p->phiGrav[0] = 0.0f; return; }
    const float th = std::fmax(0.0f, theta);
    const float theta2 = th * th;
    const bool checkInside = theta2 > 0.333333f;
    const int G = numGroups(n);
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
    for (int g = 0; g < G; ++g) {
        if (skipGroup(g)) continue;
        const uint32_t i0 = static_cast<uint32_t>(g) * kGroup;
        const int act = static_cast<int>(std::min<uint32_t>(kGroup, n - i0));
        const uint64_t totalBefore = total;
        float xi[kGroup], yi[kGroup], zi[kGroup], eI[kGroup], eI2[kGroup];
        R ax[kGroup] = {}, ay[kGroup] = {}, az[kGroup] = {}, ph[kGroup] = {};
        const R G = static_cast<R>(sizeof(R) == 4 ? static_cast<double>(kGPsuF) : kGPsuD);
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            xi[l] = p->posX[i]; yi[l] = p->posY[i]; zi[l] = p->posZ[i];
            eI[l] = 0.8f * std::fmax(p->h0[i], 1.0e-6f); eI2[l] = eI[l] * eI[l];
        }
        int stack[kStackSize];
        int sp = 0;
        stack[sp++] = 0;
        float dxs[kGroup], dys[kGroup], dzs[kGroup], r2s[kGroup];
        while (sp > 0) {
            const int node = stack[--sp];
            const int ch[2] = {b->leftChild[node], b->rightChild[node]};
            for (int k = 0; k < 2; ++k) {
                const int c = ch[k];
                if (c < 0) {
                    const uint32_t j = static_cast<uint32_t>(~c);
                    const float pxj = p->posX[j], pyj = p->posY[j], pzj = p->posZ[j], mj = p->mass[j];
                    const float eJ = 0.8f * std::fmax(p->h0[j], 1.0e-6f);
                    for (int l = 0; l < act; ++l) {
                        if (i0 + l == j) continue;
                        const R dx = R(xi[l]) - R(pxj), dy = R(yi[l]) - R(pyj), dz = R(zi[l]) - R(pzj);
                        const R r2 = dx * dx + dy * dy + dz * dz;
                        const R eij = R(0.5f) * (R(eI[l]) + R(eJ));
                        const R den = r2 + eij * eij + R(1.0e-20f);
                        const R iR = R(1) / std::sqrt(den);
                        const R iR3 = iR * iR * iR;
                        const R f = -G * R(mj) * iR3;
                        ax[l] += f * dx; ay[l] += f * dy; az[l] += f * dz;
                        ph[l] -= G * R(mj) * iR;
                        ++total;
                    }
                } else {
                    const NodeBox nb = nodeBox(*b, c);
                    bool anyOpen = false;
                    for (int l = 0; l < act; ++l) {
                        const float dx = xi[l] - nb.cx, dy = yi[l] - nb.cy, dz = zi[l] - nb.cz;
                        const float r2 = engineLen2(dx, dy, dz);
                        dxs[l] = dx; dys[l] = dy; dzs[l] = dz; r2s[l] = r2;
                        bool acc = (nb.dNode * nb.dNode < theta2 * r2) && (r2 > 1.0e-20f);
                        if (acc && checkInside && xi[l] >= nb.mnx && xi[l] <= nb.mxx && yi[l] >= nb.mny &&
                            yi[l] <= nb.mxy && zi[l] >= nb.mnz && zi[l] <= nb.mxz)
                            acc = false;
                        if (!acc) anyOpen = true;
                    }
                    if (!anyOpen || sp >= kStackSize) {
                        for (int l = 0; l < act; ++l) {
                            const R dx = R(xi[l]) - R(nb.cx), dy = R(yi[l]) - R(nb.cy), dz = R(zi[l]) - R(nb.cz);
                            const R r2 = (sizeof(R) == 4) ? R(r2s[l]) : dx * dx + dy * dy + dz * dz;
                            const R den = r2 + R(eI2[l]) + R(1.0e-20f);
                            const R iR = R(1) / std::sqrt(den);
                            const R iR3 = iR * iR * iR;
                            const R f = -G * R(nb.m) * iR3;
                            ax[l] += f * dx; ay[l] += f * dy; az[l] += f * dz;
                            ph[l] -= G * R(nb.m) * iR;
                            if (S6 != nullptr) {
                                const float iRf = static_cast<float>(iR);
                                const float* sc = S6 + 6 * static_cast<size_t>(c);
                                const float tr = sc[0] + sc[1] + sc[2];
                                const float qxx = kGPsuF * (3.0f * sc[0] - tr), qyy = kGPsuF * (3.0f * sc[1] - tr);
                                const float qzz = kGPsuF * (3.0f * sc[2] - tr), qxy = kGPsuF * 3.0f * sc[3];
                                const float qxz = kGPsuF * 3.0f * sc[4], qyz = kGPsuF * 3.0f * sc[5];
                                const float dx = dxs[l], dy = dys[l], dz = dzs[l];
                                const float qr0 = qxx * dx + qxy * dy + qxz * dz;
                                const float qr1 = qxy * dx + qyy * dy + qyz * dz;
                                const float qr2 = qxz * dx + qyz * dy + qzz * dz;
                                const float rqr = dx * qr0 + dy * qr1 + dz * qr2;
                                const float i2 = iRf * iRf, i5 = iRf * i2 * i2, i7 = i5 * i2;
                                const float t = -2.5f * rqr * i7;
                                ax[l] += qr0 * i5 + t * dx;
                                ay[l] += qr1 * i5 + t * dy;
                                az[l] += qr2 * i5 + t * dz;
                                ph[l] += -0.5f * rqr * i5;
                            }
                            ++total;
                        }
                    } else {
                        stack[sp++] = c;
                    }
                }
            }
        }
        if (groupCounts != nullptr) groupCounts[g] = static_cast<uint32_t>(total - totalBefore);
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            p->accX[i] = static_cast<float>(ax[l]); p->accY[i] = static_cast<float>(ay[l]);
            p->accZ[i] = static_cast<float>(az[l]); p->phiGrav[i] = static_cast<float>(ph[l]);
        }
    }
    if (interactionsOut) *interactionsOut = total;
}

extern "C" {
void oracle_gravity_ff(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, const float* S6,
                       uint64_t* interactionsOut) {
    gravityImpl<float>(p, b, theta, S6, interactionsOut);
}

void oracle_gravity(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, uint64_t* interactionsOut) {
    gravityImpl<float>(p, b, theta, nullptr, interactionsOut);
}

void oracle_gravity_f64(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, uint64_t* interactionsOut) {
    gravityImpl<double>(p, b, theta, nullptr, interactionsOut);
}

// The reference kernel with each group's interaction count in groupCounts[g].
void oracle_gravity_group_counts(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, uint32_t* groupCounts) {
    gravityImpl<float>(p, b, theta, nullptr, nullptr, groupCounts);
}

// Far-field mode 3 of the library (astraea_gb300_set_far_field_expansion):
// the quadrupole walk of oracle_gravity_ff at theta with (1) leaf buckets:
// an opened node of at most leafBucket particles is not descended, its sorted
// leaf range is evaluated particle-particle; (2) the group expansion: an
// accepted node with group radius^2 <= gamma^2 |c - COM|^2 (c the group's
// box centre, IEEE single-precision operations as the library's) adds, about
// c, its monopole + quadrupole field and potential with Plummer softening
// eps_g^2 (the members' mean eps^2) and the monopole's first and second
// derivatives; each member takes a + J d + 1/2 H:dd and
// phi - a.d - 1/2 d.J.d, d = x - c.  counts[0]: member-evaluated terms
// (as oracle_gravity), [1]: expansion terms, [2]: P-P terms from buckets.
void oracle_gravity_expand(AstraeaParticles* p, const AstraeaRadixBvh* b, float theta, const float* S6,
                           uint32_t leafBucket, float gamma, uint64_t* counts) {
    const uint32_t n = p->count;
    if (n == 0) return;
    if (n == 1) { p->accX[0] = p->accY[0] = p->accZ[0] = p->phiGrav[0] = 0.0f; return; }
    // sorted leaf range of every internal node
    std::vector<uint32_t> first(n - 1), last(n - 1);
    {
        std::vector<int> order;
        order.reserve(n - 1);
        std::vector<int> st{0};
        while (!st.empty()) {
            const int v = st.back(); st.pop_back();
            order.push_back(v);
            if (b->leftChild[v] >= 0) st.push_back(b->leftChild[v]);
            if (b->rightChild[v] >= 0) st.push_back(b->rightChild[v]);
        }
        for (size_t k = order.size(); k-- > 0;) {
            const int v = order[k], l = b->leftChild[v], r = b->rightChild[v];
            first[v] = l < 0 ? static_cast<uint32_t>(~l) : first[l];
            last[v] = r < 0 ? static_cast<uint32_t>(~r) : last[r];
        }
    }
    const float th = std::fmax(0.0f, theta);
    const float theta2 = th * th, gamma2 = gamma * gamma;
    const bool checkInside = theta2 > 0.333333f;
    const int G = numGroups(n);
    uint64_t total = 0, groupEvals = 0, bucketLeaves = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total, groupEvals, bucketLeaves)
    for (int g = 0; g < G; ++g) {
        const uint32_t i0 = static_cast<uint32_t>(g) * kGroup;
        const int act = static_cast<int>(std::min<uint32_t>(kGroup, n - i0));
        float xi[kGroup], yi[kGroup], zi[kGroup], eI[kGroup], eI2[kGroup];
        float ax[kGroup] = {}, ay[kGroup] = {}, az[kGroup] = {}, ph[kGroup] = {};
        float gmin[3] = {3.0e38f, 3.0e38f, 3.0e38f}, gmax[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        float e2sum = 0.0f;
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            xi[l] = p->posX[i]; yi[l] = p->posY[i]; zi[l] = p->posZ[i];
            eI[l] = 0.8f * std::fmax(p->h0[i], 1.0e-6f); eI2[l] = eI[l] * eI[l];
            gmin[0] = std::fmin(gmin[0], xi[l]); gmax[0] = std::fmax(gmax[0], xi[l]);
            gmin[1] = std::fmin(gmin[1], yi[l]); gmax[1] = std::fmax(gmax[1], yi[l]);
            gmin[2] = std::fmin(gmin[2], zi[l]); gmax[2] = std::fmax(gmax[2], zi[l]);
            e2sum += eI2[l];
        }
        const float cgx = 0.5f * (gmin[0] + gmax[0]), cgy = 0.5f * (gmin[1] + gmax[1]), cgz = 0.5f * (gmin[2] + gmax[2]);
        float rg2 = 0.0f;
        for (int l = 0; l < act; ++l) {
            const float dx = xi[l] - cgx, dy = yi[l] - cgy, dz = zi[l] - cgz;
            rg2 = std::fmax(rg2, (dx * dx + dy * dy) + dz * dz);
        }
        const float epsG2 = e2sum / static_cast<float>(act);
        double T[20] = {};
        auto pp = [&](uint32_t j) {
            const float pxj = p->posX[j], pyj = p->posY[j], pzj = p->posZ[j], mj = p->mass[j];
            const float eJ = 0.8f * std::fmax(p->h0[j], 1.0e-6f);
            for (int l = 0; l < act; ++l) {
                if (i0 + l == j) continue;
                const float dx = xi[l] - pxj, dy = yi[l] - pyj, dz = zi[l] - pzj;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float eij = 0.5f * (eI[l] + eJ);
                const float iR = 1.0f / std::sqrt(r2 + eij * eij + 1.0e-20f);
                const float f = -kGPsuF * mj * iR * iR * iR;
                ax[l] += f * dx; ay[l] += f * dy; az[l] += f * dz;
                ph[l] -= kGPsuF * mj * iR;
                ++total;
            }
        };
        int stack[kStackSize];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int node = stack[--sp];
            const int ch[2] = {b->leftChild[node], b->rightChild[node]};
            for (int k = 0; k < 2; ++k) {
                const int c = ch[k];
                if (c < 0) { pp(static_cast<uint32_t>(~c)); continue; }
                const NodeBox nb = nodeBox(*b, c);
                bool anyOpen = false;
                for (int l = 0; l < act && !anyOpen; ++l) {
                    const float dx = xi[l] - nb.cx, dy = yi[l] - nb.cy, dz = zi[l] - nb.cz;
                    const float r2 = engineLen2(dx, dy, dz);
                    bool acc = (nb.dNode * nb.dNode < theta2 * r2) && (r2 > 1.0e-20f);
                    if (acc && checkInside && xi[l] >= nb.mnx && xi[l] <= nb.mxx && yi[l] >= nb.mny &&
                        yi[l] <= nb.mxy && zi[l] >= nb.mnz && zi[l] <= nb.mxz)
                        acc = false;
                    if (!acc) anyOpen = true;
                }
                if (anyOpen && sp < kStackSize) {
                    if (leafBucket > 0 && last[c] - first[c] < leafBucket) {
                        for (uint32_t j = first[c]; j <= last[c]; ++j) {
                            pp(j);
                            bucketLeaves += static_cast<uint64_t>(act) - ((j >= i0 && j < i0 + act) ? 1u : 0u);
                        }
                    } else {
                        stack[sp++] = c;
                    }
                    continue;
                }
                const float* sc = S6 + 6 * static_cast<size_t>(c);
                const float tr = sc[0] + sc[1] + sc[2];
                const float qxx = kGPsuF * (3.0f * sc[0] - tr), qyy = kGPsuF * (3.0f * sc[1] - tr);
                const float qzz = kGPsuF * (3.0f * sc[2] - tr), qxy = kGPsuF * 3.0f * sc[3];
                const float qxz = kGPsuF * 3.0f * sc[4], qyz = kGPsuF * 3.0f * sc[5];
                const float ux = cgx - nb.cx, uy = cgy - nb.cy, uz = cgz - nb.cz;
                const float R2 = (ux * ux + uy * uy) + uz * uz;
                if (rg2 <= gamma2 * R2) {             // the group's expansion (FP64 sums of FP64 terms)
                    const double rx = ux, ry = uy, rz = uz, gm = static_cast<double>(kGPsuF) * nb.m;
                    const double s2 = rx * rx + ry * ry + rz * rz + epsG2;
                    const double is = 1.0 / std::sqrt(s2), is2 = is * is, is3 = is * is2, is5 = is3 * is2, is7 = is5 * is2;
                    const double q0 = qxx * rx + qxy * ry + qxz * rz, q1 = qxy * rx + qyy * ry + qyz * rz;
                    const double q2 = qxz * rx + qyz * ry + qzz * rz, rqr = rx * q0 + ry * q1 + rz * q2;
                    const double tq = -2.5 * rqr * is7;
                    T[0] += -gm * is - 0.5 * rqr * is5;
                    T[1] += -gm * is3 * rx + q0 * is5 + tq * rx;
                    T[2] += -gm * is3 * ry + q1 * is5 + tq * ry;
                    T[3] += -gm * is3 * rz + q2 * is5 + tq * rz;
                    const double a3 = -gm * is3, b5 = 3.0 * gm * is5;
                    T[4] += a3 + b5 * rx * rx; T[5] += a3 + b5 * ry * ry; T[6] += a3 + b5 * rz * rz;
                    T[7] += b5 * rx * ry; T[8] += b5 * rx * rz; T[9] += b5 * ry * rz;
                    const double c5 = 3.0 * gm * is5, c7 = -15.0 * gm * is7;
                    T[10] += 3.0 * c5 * rx + c7 * rx * rx * rx; T[11] += 3.0 * c5 * ry + c7 * ry * ry * ry;
                    T[12] += 3.0 * c5 * rz + c7 * rz * rz * rz; T[13] += c5 * ry + c7 * rx * rx * ry;
                    T[14] += c5 * rz + c7 * rx * rx * rz; T[15] += c5 * rx + c7 * rx * ry * ry;
                    T[16] += c5 * rz + c7 * ry * ry * rz; T[17] += c5 * rx + c7 * rx * rz * rz;
                    T[18] += c5 * ry + c7 * ry * rz * rz; T[19] += c7 * rx * ry * rz;
                    ++groupEvals;
                    continue;
                }
                for (int l = 0; l < act; ++l) {          // monopole + quadrupole at the member
                    const float dx = xi[l] - nb.cx, dy = yi[l] - nb.cy, dz = zi[l] - nb.cz;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    const float iR = 1.0f / std::sqrt(r2 + eI2[l] + 1.0e-20f);
                    const float iR3 = iR * iR * iR;
                    const float f = -kGPsuF * nb.m * iR3;
                    ax[l] += f * dx; ay[l] += f * dy; az[l] += f * dz;
                    ph[l] -= kGPsuF * nb.m * iR;
                    const float qr0 = qxx * dx + qxy * dy + qxz * dz, qr1 = qxy * dx + qyy * dy + qyz * dz;
                    const float qr2 = qxz * dx + qyz * dy + qzz * dz, rqr = dx * qr0 + dy * qr1 + dz * qr2;
                    const float i2 = iR * iR, i5 = iR * i2 * i2, i7 = i5 * i2, t = -2.5f * rqr * i7;
                    ax[l] += qr0 * i5 + t * dx; ay[l] += qr1 * i5 + t * dy; az[l] += qr2 * i5 + t * dz;
                    ph[l] += -0.5f * rqr * i5;
                    ++total;
                }
            }
        }
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            const double dx = static_cast<double>(xi[l] - cgx), dy = static_cast<double>(yi[l] - cgy),
                         dz = static_cast<double>(zi[l] - cgz);
            const double jx = T[4] * dx + T[7] * dy + T[8] * dz, jy = T[7] * dx + T[5] * dy + T[9] * dz;
            const double jz = T[8] * dx + T[9] * dy + T[6] * dz;
            const double xx = dx * dx, yy = dy * dy, zz = dz * dz, xy = dx * dy, xz = dx * dz, yz = dy * dz;
            const double hx = T[10] * xx + T[15] * yy + T[17] * zz + 2.0 * (T[13] * xy + T[14] * xz + T[19] * yz);
            const double hy = T[13] * xx + T[11] * yy + T[18] * zz + 2.0 * (T[15] * xy + T[19] * xz + T[16] * yz);
            const double hz = T[14] * xx + T[16] * yy + T[12] * zz + 2.0 * (T[19] * xy + T[17] * xz + T[18] * yz);
            p->accX[i] = static_cast<float>(ax[l] + T[1] + jx + 0.5 * hx);
            p->accY[i] = static_cast<float>(ay[l] + T[2] + jy + 0.5 * hy);
            p->accZ[i] = static_cast<float>(az[l] + T[3] + jz + 0.5 * hz);
            p->phiGrav[i] = static_cast<float>(ph[l] + T[0] - (T[1] * dx + T[2] * dy + T[3] * dz) -
                                               0.5 * (jx * dx + jy * dy + jz * dz));
        }
    }
    if (counts) { counts[0] = total; counts[1] = groupEvals; counts[2] = bucketLeaves; }
}

// Central second moments of every internal node, S = sum m (x - c)(x - c)^T,
// combined bottom-up with the parallel-axis rule in FP32 exactly as the
// library's moments refit does (children first, then
// S = S_L + S_R + m_L d_L d_L^T + m_R d_R d_R^T with d = c_child - c and the
// node COMs of b).  Leaves have S = 0.
void oracle_node_moments(const AstraeaParticles* p, const AstraeaRadixBvh* b, float* S6) {
    const uint32_t n = p->count;
    if (n < 2) return;
    std::vector<int> order;
    order.reserve(n - 1);
    std::vector<int> stack{0};
    while (!stack.empty()) {
        const int c = stack.back();
        stack.pop_back();
        order.push_back(c);
        for (int ch : {b->leftChild[c], b->rightChild[c]})
            if (ch >= 0) stack.push_back(ch);
    }
    auto child = [&](int ch, float& m, float& cx, float& cy, float& cz, const float*& s) {
        static const float zero[6] = {0, 0, 0, 0, 0, 0};
        if (ch < 0) {
            const int j = ~ch;
            m = p->mass[j]; cx = p->posX[j]; cy = p->posY[j]; cz = p->posZ[j]; s = zero;
        } else {
            m = b->nodeMass[ch]; cx = b->comX[ch]; cy = b->comY[ch]; cz = b->comZ[ch]; s = S6 + 6 * static_cast<size_t>(ch);
        }
    };
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const int c = *it;
        float mL, lx, ly, lz, mR, rx, ry, rz;
        const float *sL, *sR;
        child(b->leftChild[c], mL, lx, ly, lz, sL);
        child(b->rightChild[c], mR, rx, ry, rz, sR);
        lx -= b->comX[c]; ly -= b->comY[c]; lz -= b->comZ[c];
        rx -= b->comX[c]; ry -= b->comY[c]; rz -= b->comZ[c];
        float* o = S6 + 6 * static_cast<size_t>(c);
        o[0] = sL[0] + sR[0] + mL * lx * lx + mR * rx * rx;
        o[1] = sL[1] + sR[1] + mL * ly * ly + mR * ry * ry;
        o[2] = sL[2] + sR[2] + mL * lz * lz + mR * rz * rz;
        o[3] = sL[3] + sR[3] + mL * lx * ly + mR * rx * ry;
        o[4] = sL[4] + sR[4] + mL * lx * lz + mR * rx * rz;
        o[5] = sL[5] + sR[5] + mL * ly * lz + mR * ry * rz;
    }
}

// FP64 direct sum with eps_ij = (eps_i + eps_j)/2, eps = 0.8 h0, for the
// listed targets (tests/cpp/test_gravity_sph.cpp:359-379 criterion).
void oracle_direct_gravity_f64(uint32_t n, const float* x, const float* y, const float* z, const float* m,
                               const float* h0, uint32_t nt, const uint32_t* targets, double* acc3, double* phi) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < static_cast<int64_t>(nt); ++t) {
        const uint32_t i = targets[t];
        const double xi = x[i], yi = y[i], zi = z[i], ei = 0.8 * static_cast<double>(h0[i]);
        double ax = 0, ay = 0, az = 0, ph = 0;
        for (uint32_t j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
            const double e = 0.5 * (ei + 0.8 * static_cast<double>(h0[j]));
            const double d2 = dx * dx + dy * dy + dz * dz + e * e;
            const double inv = 1.0 / std::sqrt(d2);
            const double f = -kGPsuD * m[j] * inv * inv * inv;
            ax += f * dx; ay += f * dy; az += f * dz; ph -= kGPsuD * m[j] * inv;
        }
        acc3[3 * t] = ax; acc3[3 * t + 1] = ay; acc3[3 * t + 2] = az;
        if (phi) phi[t] = ph;
    }
}

// ------------------------------------------------------------ SPH pass 2 ----
// engine/sph_gravity.cu:965-1287.
}  // extern "C"
template <typename R>
static void pass2Impl(AstraeaParticles* p, const AstraeaRadixBvh* b) {
    const uint32_t n = p->count;
    const int G = numGroups(n);
    const bool livingIntact = b->livingFlags ? (b->livingFlags[1] != 0u) : false;
#pragma omp parallel for schedule(dynamic, 4)
    for (int g = 0; g < G; ++g) {
        if (skipGroup(g)) continue;
        const uint32_t i0 = static_cast<uint32_t>(g) * kGroup;
        const int act = static_cast<int>(std::min<uint32_t>(kGroup, n - i0));
        struct Lane {
            float xf, yf, zf, Hf, hf;
            R x, y, z, vx, vy, vz, m, h, H, rho, iRho2, P, cs, T, dmg, fs, fBal, Ri, pOr2;
            R s[6];
            uint8_t mat;
            R ax, ay, az, drC, drD, duP, duAv, duT, duS, g[9];
        } L[kGroup];
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            Lane& q = L[l];
            std::memset(&q, 0, sizeof(Lane));
            q.xf = p->posX[i]; q.yf = p->posY[i]; q.zf = p->posZ[i];
            q.x = q.xf; q.y = q.yf; q.z = q.zf;
            q.vx = p->velX[i]; q.vy = p->velY[i]; q.vz = p->velZ[i];
            q.m = p->mass[i];
            q.hf = std::fmax(p->h[i], 1.0e-6f); q.Hf = 2.0f * q.hf;
            q.h = q.hf; q.H = q.Hf;
            const float rhof = std::fmax(p->rho[i], 1.0e-9f);
            q.rho = rhof;
            q.iRho2 = R(1) / (q.rho * q.rho);
            q.P = effPressure(p->pressure[i], p->phaseId[i]);
            q.cs = std::fmax(p->soundSpeed[i], 0.05f);
            q.T = p->tempK[i]; q.dmg = p->damage[i]; q.fs = p->surfFactor[i]; q.mat = p->materialId[i];
            q.s[0] = p->sXX[i]; q.s[1] = p->sYY[i]; q.s[2] = p->sZZ[i]; q.s[3] = p->sXY[i]; q.s[4] = p->sXZ[i]; q.s[5] = p->sYZ[i];
            q.fBal = balsara<R>(p->divV[i], p->curlVX[i], p->curlVY[i], p->curlVZ[i], q.cs, q.h);
            q.Ri = (q.P < R(0)) ? (R(0.3f) * (-q.P) * q.iRho2) : R(0);
            q.pOr2 = q.P * q.iRho2;
        }
        if (n >= 2) {
            walkGroup(*b,
                [&](int c) {
                    for (int l = 0; l < act; ++l) {
                        const float rad = std::fmax(L[l].Hf, 1.09f * b->nodeMaxH[c]);
                        if (pointBoxDist2(L[l].xf, L[l].yf, L[l].zf, b->aabbMinX[c], b->aabbMinY[c], b->aabbMinZ[c],
                                          b->aabbMaxX[c], b->aabbMaxY[c], b->aabbMaxZ[c]) <= rad * rad)
                            return true;
                    }
                    return false;
                },
                [&](uint32_t j) {
                    const float pxj = p->posX[j], pyj = p->posY[j], pzj = p->posZ[j];
                    const float hjf = std::fmax(p->h[j], 1.0e-6f), Hjf = 2.0f * hjf;
                    bool bal = false;
                    R fBalJ = 0;
                    for (int l = 0; l < act; ++l) {
                        const uint32_t i = i0 + l;
                        Lane& q = L[l];
                        const float dxf = q.xf - pxj, dyf = q.yf - pyj, dzf = q.zf - pzj;
                        const float r2f = engineLen2(dxf, dyf, dzf);
                        const float Hmf = std::fmax(q.Hf, Hjf);
                        if (j == i || !(r2f < Hmf * Hmf)) continue;
                        const R dx = q.x - R(pxj), dy = q.y - R(pyj), dz = q.z - R(pzj);
                        const R r2 = (sizeof(R) == 4) ? R(r2f) : dx * dx + dy * dy + dz * dz;
                        const R hj = hjf, Hj = Hjf, mj = p->mass[j];
                        const R rhoJ = std::fmax(p->rho[j], 1.0e-9f);
                        const R pJ = effPressure(p->pressure[j], p->phaseId[j]);
                        const R csJ = std::fmax(p->soundSpeed[j], 0.05f);
                        const R dvx = q.vx - R(p->velX[j]), dvy = q.vy - R(p->velY[j]), dvz = q.vz - R(p->velZ[j]);
                        const R vDotR = dvx * dx + dvy * dy + dvz * dz;
                        if (vDotR < R(0) && !bal) {
                            fBalJ = balsara<R>(p->divV[j], p->curlVX[j], p->curlVY[j], p->curlVZ[j], csJ, hj);
                            bal = true;
                        }
                        const R r = std::sqrt(r2);
                        const R gI = wendlandGrad<R>(r, q.H), gJ = wendlandGrad<R>(r, Hj);
                        const R gb = R(0.5f) * (gI + gJ);
                        const R gx = gb * dx, gy = gb * dy, gz = gb * dz;
                        const R iRhoJ2 = R(1) / (rhoJ * rhoJ);
                        const R vDotG = dvx * gx + dvy * gy + dvz * gz;
                        q.drC += (mj / rhoJ) * vDotG;
                        if (p->materialId[j] == q.mat) {
                            const R rDotG = -(dx * gx + dy * gy + dz * gz);
                            const R dd = r2 + R(0.01f) * q.H * q.H;
                            q.drD += (mj / rhoJ) * (R(2) * (rhoJ - q.rho) / dd) * rDotG;
                        }
                        R pi = 0;
                        if (vDotR < R(0)) {
                            const R hB = R(0.5f) * (q.h + hj), cB = R(0.5f) * (q.cs + csJ), rB = R(0.5f) * (q.rho + rhoJ);
                            const R muIJ = (hB * vDotR) / (r2 + R(0.01f) * hB * hB);
                            pi = ((R(-1) * cB * muIJ + R(2) * muIJ * muIJ) / rB) * (R(0.5f) * (q.fBal + fBalJ));
                        }
                        R tens = 0;
                        const R Rj = (pJ < R(0)) ? (R(0.3f) * (-pJ) * iRhoJ2) : R(0);
                        if (q.Ri + Rj > R(0)) {
                            const R Hb = R(0.5f) * (q.H + Hj);
                            if (r < Hb) {
                                const R qb = r / Hb, om = R(1) - qb, om2 = om * om;
                                const R fr = (om2 * om2 * (R(1) + R(4) * qb)) * (R(1) / R(0.6328125f));
                                const R fr2 = fr * fr;
                                tens = (q.Ri + Rj) * (fr2 * fr2);
                            }
                        }
                        const R pT = q.pOr2 + pJ * iRhoJ2;
                        const R iso = -mj * (pT + pi + tens);
                        q.ax += iso * gx; q.ay += iso * gy; q.az += iso * gz;
                        q.duP += mj * vDotG;
                        q.duAv += R(0.5f) * mj * pi * vDotG;
                        q.duT += R(0.5f) * mj * tens * vDotG;
                        const R sj[6] = {R(p->sXX[j]), R(p->sYY[j]), R(p->sZZ[j]), R(p->sXY[j]), R(p->sXZ[j]), R(p->sYZ[j])};
                        const R tXX = q.s[0] * q.iRho2 + sj[0] * iRhoJ2, tYY = q.s[1] * q.iRho2 + sj[1] * iRhoJ2;
                        const R tZZ = q.s[2] * q.iRho2 + sj[2] * iRhoJ2, tXY = q.s[3] * q.iRho2 + sj[3] * iRhoJ2;
                        const R tXZ = q.s[4] * q.iRho2 + sj[4] * iRhoJ2, tYZ = q.s[5] * q.iRho2 + sj[5] * iRhoJ2;
                        q.ax += mj * (tXX * gx + tXY * gy + tXZ * gz);
                        q.ay += mj * (tXY * gx + tYY * gy + tYZ * gz);
                        q.az += mj * (tXZ * gx + tYZ * gy + tZZ * gz);
                        const R wx = -dvx, wy = -dvy, wz = -dvz;
                        q.duS += mj * ((q.s[0] * wx + q.s[3] * wy + q.s[4] * wz) * gx +
                                       (q.s[3] * wx + q.s[1] * wy + q.s[5] * wz) * gy +
                                       (q.s[4] * wx + q.s[5] * wy + q.s[2] * wz) * gz);
                        const R vol = mj / rhoJ;
                        const R gxi = gI * dx, gyi = gI * dy, gzi = gI * dz;
                        q.g[0] += vol * wx * gxi; q.g[1] += vol * wx * gyi; q.g[2] += vol * wx * gzi;
                        q.g[3] += vol * wy * gxi; q.g[4] += vol * wy * gyi; q.g[5] += vol * wy * gzi;
                        q.g[6] += vol * wz * gxi; q.g[7] += vol * wz * gyi; q.g[8] += vol * wz * gzi;
                    }
                });
        }
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            Lane& q = L[l];
            p->accX[i] += static_cast<float>(q.ax);
            p->accY[i] += static_cast<float>(q.ay);
            p->accZ[i] += static_cast<float>(q.az);
            const R mask = (p->shepardC[i] > 0.85f) ? (R(1) - q.fs) : R(0);
            p->drhoDt[i] = static_cast<float>(q.rho * q.drC + R(0.05f) * q.H * q.cs * mask * q.drD);
            const R duStress = q.iRho2 * q.duS;
            // FP64 radiative cooling epilogue, engine/sph_gravity.cu:1222-1235
            const double tAmb = (livingIntact && p->bodyId[i] == 0u && p->damage[i] < 0.8f) ? 255.0 : 3.0;
            const double mSi = std::fmax(static_cast<double>(p->mass[i]) * 1.0e24, 1.0);
            const double rhoSi = std::fmax(static_cast<double>(static_cast<float>(q.rho)) * 1.0e6, 1.0e-3);
            const double rP = std::cbrt((3.0 * mSi) / (4.0 * kPiD * rhoSi));
            const double area = kPiD * rP * rP;
            const double T = static_cast<double>(p->tempK[i]);
            const double T4 = T * T * T * T, Ta4 = tAmb * tAmb * tAmb * tAmb;
            const double dT4 = std::fmax(0.0, T4 - Ta4);
            const double pRad = static_cast<double>(p->surfFactor[i]) * 0.9 * kSigmaSB * area * dT4;
            p->radPowerW[i] = static_cast<float>(pRad);
            const float duRad = static_cast<float>(-pRad / (std::fmax(static_cast<double>(p->mass[i]), 1.0e-30) * 1.0e27));
            p->duDt[i] = static_cast<float>(q.pOr2 * q.duP + q.duAv + q.duT + duStress + R(duRad));
            const Strength st = strengthOf(q.mat);
            if (st.mu <= 0.0f || st.tMelt <= 0.0f) {
                p->dSXX[i] = p->dSYY[i] = p->dSZZ[i] = p->dSXY[i] = p->dSXZ[i] = p->dSYZ[i] = 0.0f;
                p->dDamageCbrtDt[i] = 0.0f;
                continue;
            }
            const R tN = q.T / R(st.tMelt);
            const R soft = std::max(R(0), R(1) - tN * tN);
            const R muE = (R(1) - q.dmg) * R(st.mu) * soft;
            const R* g = q.g;
            const R tr3 = (g[0] + g[4] + g[8]) * (R(1) / R(3));
            const R eXX = g[0] - tr3, eYY = g[4] - tr3, eZZ = g[8] - tr3;
            const R eXY = R(0.5f) * (g[1] + g[3]), eXZ = R(0.5f) * (g[2] + g[6]), eYZ = R(0.5f) * (g[5] + g[7]);
            const R rXY = R(0.5f) * (g[1] - g[3]), rXZ = R(0.5f) * (g[2] - g[6]), rYZ = R(0.5f) * (g[5] - g[7]);
            const R rYX = -rXY, rZX = -rXZ, rZY = -rYZ;
            const R* s = q.s;  // xx yy zz xy xz yz
            p->dSXX[i] = static_cast<float>(R(2) * muE * eXX + R(2) * (s[3] * rXY + s[4] * rXZ));
            p->dSYY[i] = static_cast<float>(R(2) * muE * eYY + R(2) * (s[3] * rYX + s[5] * rYZ));
            p->dSZZ[i] = static_cast<float>(R(2) * muE * eZZ + R(2) * (s[4] * rZX + s[5] * rZY));
            p->dSXY[i] = static_cast<float>(R(2) * muE * eXY + s[0] * rYX + s[4] * rYZ + s[1] * rXY + s[5] * rXZ);
            p->dSXZ[i] = static_cast<float>(R(2) * muE * eXZ + s[0] * rZX + s[3] * rZY + s[2] * rXZ + s[5] * rXY);
            p->dSYZ[i] = static_cast<float>(R(2) * muE * eYZ + s[3] * rZX + s[1] * rZY + s[4] * rYX + s[2] * rYZ);
            const float Tf = p->tempK[i], Df = p->damage[i];
            if (Tf < st.tMelt && Df < 1.0f) {
                const float Pf = static_cast<float>(q.P);
                const float sig = maxPrincipal(Pf, p->sXX[i], p->sYY[i], p->sZZ[i], p->sXY[i], p->sXZ[i], p->sYZ[i]);
                const float stiff = std::fmax(st.K + (4.0f / 3.0f) * st.mu, 1.0e-12f);
                const float eT = std::fmax(0.0f, sig) / stiff;
                const float eF = std::fmax(p->epsFail[i], 1.0e-8f);
                const float rhof = std::fmax(p->rho[i], 1.0e-9f);
                const float cC = std::fmax(std::fmax(p->soundSpeed[i], 0.05f), std::sqrt((st.K + (4.0f / 3.0f) * st.mu) / rhof));
                p->dDamageCbrtDt[i] = (eT > eF) ? (0.4f * cC / q.hf) : 0.0f;
            } else {
                p->dDamageCbrtDt[i] = 0.0f;
            }
        }
    }
}
extern "C" {
void oracle_sph_pass2(AstraeaParticles* p, const AstraeaRadixBvh* b) { if (p->count) pass2Impl<float>(p, b); }
void oracle_sph_pass2_f64(AstraeaParticles* p, const AstraeaRadixBvh* b) { if (p->count) pass2Impl<double>(p, b); }

// ------------------------------------------------------------ KDK kick ----
// engine/sph_gravity.cu:1291-1374.
void oracle_kick_half(AstraeaParticles* p, float hdt, int clampThermal) {
    const uint32_t n = p->count;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < static_cast<int64_t>(n); ++ii) {
        const uint32_t i = static_cast<uint32_t>(ii);
        const float vx = p->velX[i] + hdt * p->accX[i];
        const float vy = p->velY[i] + hdt * p->accY[i];
        const float vz = p->velZ[i] + hdt * p->accZ[i];
        p->velX[i] = vx; p->velY[i] = vy; p->velZ[i] = vz;
        p->velHalfX[i] = vx; p->velHalfY[i] = vy; p->velHalfZ[i] = vz;
        const float rhoN = std::fmax(p->rho[i] + hdt * p->drhoDt[i], 1.0e-9f);
        p->rho[i] = rhoN;
        const int m = matIndex(p->materialId[i]);
        const Strength st = strengthOf(m);
        float uN = p->u[i] + hdt * p->duDt[i];
        if (clampThermal) {
            const double uMin = coldEnergy(m, static_cast<double>(rhoN)) + 3.0 * (kMat[m].cv / 1.0e6);
            uN = std::fmax(uN, static_cast<float>(uMin));
        } else {
            uN = std::fmax(uN, 0.0f);
        }
        p->u[i] = uN;
        float dc = p->damageCbrt[i] + hdt * p->dDamageCbrtDt[i];
        dc = std::fmin(1.0f, std::fmax(p->damageCbrt[i], dc));
        const float D = dc * dc * dc;
        p->damageCbrt[i] = dc; p->damage[i] = D;
        if (clampThermal) {
            const EosOut e = evaluateEos(m, rhoN, uN, D);
            p->pressure[i] = e.p; p->soundSpeed[i] = e.cs; p->tempK[i] = e.T; p->phaseId[i] = e.phase;
        }
        if (st.mu <= 0.0f || st.tMelt <= 0.0f || p->tempK[i] >= st.tMelt) {
            p->sXX[i] = p->sYY[i] = p->sZZ[i] = p->sXY[i] = p->sXZ[i] = p->sYZ[i] = 0.0f;
            continue;
        }
        float sxx = p->sXX[i] + hdt * p->dSXX[i], syy = p->sYY[i] + hdt * p->dSYY[i], szz = p->sZZ[i] + hdt * p->dSZZ[i];
        const float sxy = p->sXY[i] + hdt * p->dSXY[i], sxz = p->sXZ[i] + hdt * p->dSXZ[i], syz = p->sYZ[i] + hdt * p->dSYZ[i];
        const float tr3 = (sxx + syy + szz) * (1.0f / 3.0f);
        sxx -= tr3; syy -= tr3; szz -= tr3;
        const float tR = p->tempK[i] / st.tMelt;
        const float yI = (1.0f - D) * st.Y0 * std::fmax(0.0f, 1.0f - tR);
        const float yF = D * std::fmin(st.Y0, 0.6f * std::fmax(0.0f, p->pressure[i]));
        const float Y = std::fmax(yI, yF);
        const float j2 = 0.5f * (sxx * sxx + syy * syy + szz * szz + 2.0f * (sxy * sxy + sxz * sxz + syz * syz));
        const float eq = std::sqrt(3.0f * j2 + 1.0e-30f);
        const float sc = (Y <= 0.0f) ? 0.0f : std::fmin(1.0f, Y / eq);
        p->sXX[i] = sxx * sc; p->sYY[i] = syy * sc; p->sZZ[i] = szz * sc;
        p->sXY[i] = sxy * sc; p->sXZ[i] = sxz * sc; p->sYZ[i] = syz * sc;
    }
}

}  // extern "C"

// ------------------------------------------------------------ XSPH drift ----
// engine/sph_gravity.cu:1376-1489, with neighbours read from the pre-drift
// positions (the reference kernel reads them while other threads write).
// R = float: the reference kernel's arithmetic; R = double: the FP64 host
// path (the same neighbour sets, sums and the position update in double).
template <typename R>
static void driftImpl(AstraeaParticles* p, float dt, const AstraeaRadixBvh* b, int useBvh) {
    const uint32_t n = p->count;
    std::vector<float> nx(p->posX, p->posX + n), ny(p->posY, p->posY + n), nz(p->posZ, p->posZ + n);
    const int G = numGroups(n);
#pragma omp parallel for schedule(dynamic, 4)
    for (int g = 0; g < G; ++g) {
        if (skipGroup(g)) continue;
        const uint32_t i0 = static_cast<uint32_t>(g) * kGroup;
        const int act = static_cast<int>(std::min<uint32_t>(kGroup, n - i0));
        float xi[kGroup], yi[kGroup], zi[kGroup], vxi[kGroup], vyi[kGroup], vzi[kGroup], Hi[kGroup], rhoI[kGroup];
        R sx[kGroup] = {}, sy[kGroup] = {}, sz[kGroup] = {};
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            xi[l] = p->posX[i]; yi[l] = p->posY[i]; zi[l] = p->posZ[i];
            vxi[l] = p->velX[i]; vyi[l] = p->velY[i]; vzi[l] = p->velZ[i];
            Hi[l] = 2.0f * std::fmax(p->h[i], 1.0e-6f); rhoI[l] = std::fmax(p->rho[i], 1.0e-9f);
        }
        if (useBvh && n >= 2) {
            walkGroup(*b,
                [&](int c) {
                    for (int l = 0; l < act; ++l) {
                        const float rad = std::fmax(Hi[l], 1.09f * b->nodeMaxH[c]);
                        if (pointBoxDist2(xi[l], yi[l], zi[l], b->aabbMinX[c], b->aabbMinY[c], b->aabbMinZ[c],
                                          b->aabbMaxX[c], b->aabbMaxY[c], b->aabbMaxZ[c]) <= rad * rad)
                            return true;
                    }
                    return false;
                },
                [&](uint32_t j) {
                    const float pxj = p->posX[j], pyj = p->posY[j], pzj = p->posZ[j];
                    const float Hj = 2.0f * std::fmax(p->h[j], 1.0e-6f);
                    for (int l = 0; l < act; ++l) {
                        if (i0 + l == j) continue;
                        const float dx = xi[l] - pxj, dy = yi[l] - pyj, dz = zi[l] - pzj;
                        const float r2 = engineLen2(dx, dy, dz);
                        const float Hm = std::fmax(Hi[l], Hj);
                        if (!(r2 < Hm * Hm)) continue;
                        const R r = (sizeof(R) == 4) ? R(std::sqrt(r2))
                                                     : std::sqrt(R(dx) * R(dx) + R(dy) * R(dy) + R(dz) * R(dz));
                        const R wb = R(0.5f) * (wendland<R>(r, R(Hi[l])) + wendland<R>(r, R(Hj)));
                        const R rb = R(0.5f) * (R(rhoI[l]) + R(std::fmax(p->rho[j], 1.0e-9f)));
                        const R co = (R(p->mass[j]) / rb) * wb;
                        sx[l] += co * (R(p->velX[j]) - R(vxi[l]));
                        sy[l] += co * (R(p->velY[j]) - R(vyi[l]));
                        sz[l] += co * (R(p->velZ[j]) - R(vzi[l]));
                    }
                });
        }
        for (int l = 0; l < act; ++l) {
            const uint32_t i = i0 + l;
            nx[i] = static_cast<float>(R(xi[l]) + R(dt) * (R(vxi[l]) + R(0.25f) * sx[l]));
            ny[i] = static_cast<float>(R(yi[l]) + R(dt) * (R(vyi[l]) + R(0.25f) * sy[l]));
            nz[i] = static_cast<float>(R(zi[l]) + R(dt) * (R(vzi[l]) + R(0.25f) * sz[l]));
        }
    }
    std::memcpy(p->posX, nx.data(), n * 4); std::memcpy(p->posY, ny.data(), n * 4); std::memcpy(p->posZ, nz.data(), n * 4);
}

extern "C" {
void oracle_drift(AstraeaParticles* p, float dt, const AstraeaRadixBvh* b, int useBvh) {
    driftImpl<float>(p, dt, b, useBvh);
}
void oracle_drift_f64(AstraeaParticles* p, float dt, const AstraeaRadixBvh* b, int useBvh) {
    driftImpl<double>(p, dt, b, useBvh);
}

// --------------------------------------------------------------- dt ----
// engine/sph_gravity.cu:1493-1550 + host clamp 2136-2161.
float oracle_reduce_dt(const AstraeaParticles* p, float prevDt, float maxDt, float* rawMinOut) {
    const float floorDt = std::fmin(1.0e-5f, maxDt);
    const float upper = (prevDt > 0.0f) ? std::fmin(prevDt * 1.15f, maxDt) : maxDt;
    const uint32_t n = p->count;
    if (n == 0) return upper;
    float mn = 1.0e30f;
    for (uint32_t i = 0; i < n; ++i) {
        const float hi = std::fmax(p->h[i], 1.0e-6f), cs = std::fmax(p->soundSpeed[i], 0.05f);
        // the engine's kernel contracts |v|^2, 2.2 cs + |v| and u + 0.01 u_s
        // into fmas (engineLen2 / engineMulAdd)
        const float v = std::sqrt(engineLen2(p->velX[i], p->velY[i], p->velZ[i]));
        const float dtC = 0.25f * hi / (engineMulAdd(2.2f, cs, v) + 1.0e-6f);
        const float a = std::sqrt(engineLen2(p->accX[i], p->accY[i], p->accZ[i]));
        const float dtA = 0.25f * std::sqrt(hi / (a + 1.0e-8f));
        const int m = matIndex(p->materialId[i]);
        const float uI = std::fmax(p->u[i], 0.0f);
        const float uS = std::fmax(uI, u0RefPsu(m));
        const float dtT = 0.20f * engineMulAdd(0.01f, uS, uI) / (std::fabs(p->duDt[i]) + 1.0e-8f);
        const float d = std::fmin(dtC, std::fmin(dtA, dtT));
        if (std::isfinite(d) && d > 0.0f) mn = std::fmin(mn, d);
    }
    if (rawMinOut) *rawMinOut = mn;
    float raw = mn;
    if (!(std::isfinite(raw) && raw > 0.0f) || raw >= 1.0e30f) raw = upper;
    return std::fmin(upper, std::fmax(floorDt, raw));
}

// ------------------------------------------------------------ full step ----
// engine/simulation.cpp:1711-1753 kernel sequence.
float oracle_step(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* b, float prevDt, float maxDt,
                  float theta) {
    const float dt = oracle_reduce_dt(p, prevDt, maxDt, nullptr);
    oracle_kick_half(p, 0.5f * dt, 0);
    const int useBvh = (b->capacity >= p->count && b->leftChild != nullptr && p->count >= 2u) ? 1 : 0;
    oracle_drift(p, dt, b, useBvh);
    oracle_sort_and_build(p, alt, b, nullptr);
    oracle_sph_pass1(p, b);
    oracle_evaluate_eos(p);
    oracle_gravity(p, b, theta, nullptr);
    oracle_sph_pass2(p, b);
    oracle_kick_half(p, 0.5f * dt, 0);
    oracle_evaluate_eos(p);
    return dt;
}

// The FP64 host path of the same step (the CPU baseline): the stages that
// walk the tree (drift, pass 1, gravity, pass 2) in double over the same
// neighbour and interaction sets; sort, tree and refit as above; the EOS is
// the reference's FP64 EOS in both paths.
float oracle_step_f64(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* b, float prevDt, float maxDt,
                      float theta) {
    const float dt = oracle_reduce_dt(p, prevDt, maxDt, nullptr);
    oracle_kick_half(p, 0.5f * dt, 0);
    const int useBvh = (b->capacity >= p->count && b->leftChild != nullptr && p->count >= 2u) ? 1 : 0;
    oracle_drift_f64(p, dt, b, useBvh);
    oracle_sort_and_build(p, alt, b, nullptr);
    oracle_sph_pass1_f64(p, b);
    oracle_evaluate_eos(p);
    oracle_gravity_f64(p, b, theta, nullptr);
    oracle_sph_pass2_f64(p, b);
    oracle_kick_half(p, 0.5f * dt, 0);
    oracle_evaluate_eos(p);
    return dt;
}

// ---------------------------------------------------------- render ----
// engine/sph_gravity.cu:1583-1585
static inline float finite0(float v) { return std::isfinite(v) ? v : 0.0f; }
static inline void putU32(uint8_t* d, uint32_t v) { for (int k = 0; k < 4; ++k) d[k] = static_cast<uint8_t>(v >> (8 * k)); }
static inline void putF32(uint8_t* d, float f) { uint32_t v; std::memcpy(&v, &f, 4); putU32(d, v); }
static inline void putU16(uint8_t* d, uint16_t v) { d[0] = static_cast<uint8_t>(v); d[1] = static_cast<uint8_t>(v >> 8); }

// packRenderRecordsKernel, engine/sph_gravity.cu:1670-1743 (20-byte records,
// little-endian, layout of ParticleRecordPacked :1570-1581).
void oracle_pack_render_records(const AstraeaParticles* p, uint8_t* rec20, uint8_t* speed, float sx, float sy,
                                float sz) {
    const float kInvLog20000 = 1.0f / 9.9034875525361280f;
    const float kInvLog1e7 = 1.0f / 16.118095650958320f;
    const float kInvLog2000 = 1.0f / 7.6009024595420823f;
    for (uint32_t i = 0; i < p->count; ++i) {
        uint8_t* d = rec20 + 20u * static_cast<size_t>(i);
        putF32(d + 0, finite0((p->posX[i] - sx) * 1000.0f));
        putF32(d + 4, finite0((p->posY[i] - sy) * 1000.0f));
        putF32(d + 8, finite0((p->posZ[i] - sz) * 1000.0f));
        const float T = std::fmax(10.0f, finite0(p->tempK[i]));
        const float tNorm = std::fmin(1.0f, std::fmax(0.0f, std::log(T * 0.1f) * kInvLog20000));
        putU16(d + 12, static_cast<uint16_t>(std::lrint(65535.0f * tNorm)));
        const float pGPa = finite0(p->pressure[i]) * 1000.0f;
        uint16_t pu = 0;
        if (pGPa > 1.0e-3f) {
            const float pNorm = std::fmin(1.0f, std::fmax(0.0f, std::log(pGPa * 1000.0f) * kInvLog1e7));
            pu = static_cast<uint16_t>(std::lrint(1.0f + 65534.0f * pNorm));
        }
        putU16(d + 14, pu);
        d[16] = p->materialId[i];
        d[17] = static_cast<uint8_t>(((p->bodyId[i] & 0x0Fu) << 4) | (p->phaseId[i] & 0x0Fu));
        const float dam = std::fmin(1.0f, std::fmax(0.0f, finite0(p->damage[i])));
        d[18] = static_cast<uint8_t>(std::lrint(dam * 255.0f));
        const float vol = std::fmax(p->mass[i], 0.0f) / std::fmax(p->rho[i], 1.0e-9f);
        const float rKm = std::cbrt((3.0f * vol) / (4.0f * kPiF)) * 1000.0f;
        const float rNorm = std::fmin(1.0f, std::fmax(0.0f, std::log(std::fmax(rKm, 1.0f)) * kInvLog2000));
        d[19] = static_cast<uint8_t>(std::lrint(255.0f * rNorm));
        if (speed != nullptr) {
            const float vx = p->velX[i], vy = p->velY[i], vz = p->velZ[i];
            const float sp = finite0(std::sqrt(vx * vx + vy * vy + vz * vz));
            const float vNorm = std::fmin(1.0f, std::fmax(0.0f, std::log(std::fmax(sp, 0.05f) * 20.0f) * kInvLog2000));
            speed[i] = static_cast<uint8_t>(std::lrint(255.0f * vNorm));
        }
    }
}

// extractTracersKernel + launchExtractTracers, engine/sph_gravity.cu:1586-1668,
// 2163-2187 (40-byte records, layout of CrustTracerRecordPacked :1554-1567).
void oracle_extract_tracers(const AstraeaParticles* p, uint8_t* rec40, uint32_t tracerCount, float lx, float ly,
                            float lz, float sx, float sy, float sz) {
    if (tracerCount == 0 || rec40 == nullptr) return;
    std::memset(rec40, 0, 40u * static_cast<size_t>(tracerCount));
    for (uint32_t i = 0; i < p->count; ++i) {
        const int32_t t = p->tracerIndex[i];
        if (t < 0 || static_cast<uint32_t>(t) >= tracerCount) continue;
        const float px = p->posX[i], py = p->posY[i], pz = p->posZ[i];
        const float dx = px - lx, dy = py - ly, dz = pz - lz;
        const float r = std::sqrt(dx * dx + dy * dy + dz * dz);
        const float rRest = p->tracerRestRadiusPsu[i];
        const float dispKm = (r - rRest) * 1000.0f;
        float normalDelta = 0.0f;
        if (r > 1.0e-9f) {
            const float invR = 1.0f / r;
            const float nx = dx * invR, ny = dy * invR, nz = dz * invR;
            const float dot = std::fmin(1.0f, std::fmax(-1.0f, nx * p->tracerRestNormalX[i] +
                                                                   ny * p->tracerRestNormalY[i] +
                                                                   nz * p->tracerRestNormalZ[i]));
            normalDelta = std::acos(dot);
        }
        const float dam = std::fmin(1.0f, std::fmax(0.0f, finite0(p->damage[i])));
        const float tempK = std::fmax(3.0f, finite0(p->tempK[i]));
        const uint8_t phase = p->phaseId[i];
        const bool ocean = p->tracerIsOcean[i] != 0;
        const bool disrupted = dam >= 0.85f || phase == 2 || phase == 3 ||
                               std::fabs(r - rRest) > 0.5f * std::fmax(rRest, 1.0e-3f);
        const float dv = std::fmax(0.0f, -finite0(p->divV[i])) * std::fmax(p->h[i], 0.0f) * 1000.0f;
        const float over = std::fmax(0.0f, 1.225f * 340.0f * dv * 1.0e-3f);
        const float tsunami = ocean ? std::fmax(0.0f, finite0(dispKm) * 1000.0f) : 0.0f;
        uint8_t* d = rec40 + 40u * static_cast<size_t>(t);
        putU16(d + 0, static_cast<uint16_t>(t));
        putU16(d + 2, static_cast<uint16_t>((ocean ? 1u : 0u) | (disrupted ? 2u : 0u)));
        putF32(d + 4, finite0((px - sx) * 1000.0f));
        putF32(d + 8, finite0((py - sy) * 1000.0f));
        putF32(d + 12, finite0((pz - sz) * 1000.0f));
        putF32(d + 16, finite0(dispKm));
        putF32(d + 20, finite0(normalDelta));
        putF32(d + 24, tempK);
        putF32(d + 28, dam);
        putF32(d + 32, finite0(over));
        putF32(d + 36, finite0(tsunami));
    }
}

// Uncompressed PCLS frame: encodeHeader40 + buildBinaryFrame with
// compressZlib = false (server/binary_protocol.cpp:76-87, 155-217), records
// from the two functions above.  Returns the frame size (0 if cap too small).
size_t oracle_pcls_frame(const AstraeaParticles* p, const AstraeaPclsFrameInfo* info, uint8_t* out, size_t cap) {
    const size_t n = p->count, t = info->tracerCount;
    const bool hasSpeed = info->withSpeed != 0 && n > 0;
    const size_t payload = 20 * n + 40 * t + (hasSpeed ? n : 0);
    if (cap < 40 + payload) return 0;
    uint16_t flags = 0;
    if (t > 0) flags |= 2u;
    if (info->livingBodyPresent) flags |= 4u;
    if (hasSpeed) flags |= 8u;
    putU32(out + 0, 0x50434C53u);
    putU16(out + 4, 1u);
    putU16(out + 6, flags);
    uint64_t sb;
    std::memcpy(&sb, &info->simTimeSec, 8);
    putU32(out + 8, static_cast<uint32_t>(sb));
    putU32(out + 12, static_cast<uint32_t>(sb >> 32));
    putU32(out + 16, static_cast<uint32_t>(info->frameSeq & 0xffffffffull));
    putF32(out + 20, info->dtSec);
    putU32(out + 24, static_cast<uint32_t>(n));
    putU32(out + 28, static_cast<uint32_t>(t));
    putU32(out + 32, t > 0 ? info->tracerGridRes : 0u);
    putU32(out + 36, static_cast<uint32_t>(payload));
    uint8_t* recs = out + 40;
    uint8_t* trc = recs + 20 * n;
    uint8_t* spd = hasSpeed ? trc + 40 * t : nullptr;
    oracle_pack_render_records(p, recs, spd, info->sysCom[0], info->sysCom[1], info->sysCom[2]);
    oracle_extract_tracers(p, trc, static_cast<uint32_t>(t), info->livingCom[0], info->livingCom[1],
                           info->livingCom[2], info->sysCom[0], info->sysCom[1], info->sysCom[2]);
    return 40 + payload;
}

// ------------------------------------------------------- telemetry ----
// The O(N) loops of Simulation::Impl::computeTelemetryFromDevice
// (engine/simulation.cpp:948-1285) and sumDeviceRadPowerW (:567-582), serial
// and in FP64 like the engine's host code, on host copies of the fields.
// Parity unpinned by reference outputs: these loops run inside the engine's
// Simulation object, which needs the whole CUDA engine to construct.
void oracle_telemetry(const AstraeaParticles* p, const AstraeaTelemetryParams* prm, AstraeaTelemetry* o) {
    std::memset(o, 0, sizeof(*o));
    const uint32_t n = p->count;
    if (n == 0) return;
    const double G = kGPsuD;
    const double targetR = prm->targetRadiusPsu;
    double M = 0, sx = 0, sy = 0, sz = 0;
    double m0 = 0, x0 = 0, y0 = 0, z0 = 0, vx0 = 0, vy0 = 0, vz0 = 0;
    double m1 = 0, x1 = 0, y1 = 0, z1 = 0, vx1 = 0, vy1 = 0, vz1 = 0;
    double ke = 0, pe = 0, ie = 0, px = 0, py = 0, pz = 0, lx = 0, ly = 0, lz = 0, maxT = 0, maxP = 0, rad = 0;
    uint32_t seed = 0;
    double minPhi = HUGE_VAL;
    for (uint32_t i = 0; i < n; ++i) {                              // :982-1047
        const double m = p->mass[i], x = p->posX[i], y = p->posY[i], z = p->posZ[i];
        const double vx = p->velX[i], vy = p->velY[i], vz = p->velZ[i];
        const double phi = p->phiGrav[i], uv = p->u[i], T = p->tempK[i];
        const double PG = static_cast<double>(p->pressure[i]) * 1000.0;
        M += m; sx += m * x; sy += m * y; sz += m * z;
        if (p->bodyId[i] == 0) {
            m0 += m; x0 += m * x; y0 += m * y; z0 += m * z; vx0 += m * vx; vy0 += m * vy; vz0 += m * vz;
        } else {
            m1 += m; x1 += m * x; y1 += m * y; z1 += m * z; vx1 += m * vx; vy1 += m * vy; vz1 += m * vz;
        }
        ke += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        pe += 0.5 * m * phi;
        ie += m * uv;
        px += m * vx; py += m * vy; pz += m * vz;
        lx += m * (y * vz - z * vy); ly += m * (z * vx - x * vz); lz += m * (x * vy - y * vx);
        if (std::isfinite(T)) maxT = std::max(maxT, T);
        if (std::isfinite(PG)) maxP = std::max(maxP, PG);
        if (std::isfinite(phi) && phi < minPhi) { minPhi = phi; seed = i; }
        const double w = p->radPowerW[i];                             // :572-579
        if (std::isfinite(w) && w > 0.0) rad += w;
    }
    o->totalMassPsu = M;
    if (M > 0) { o->sysComPsu[0] = sx / M; o->sysComPsu[1] = sy / M; o->sysComPsu[2] = sz / M; }
    if (m0 > 0) { x0 /= m0; y0 /= m0; z0 /= m0; vx0 /= m0; vy0 /= m0; vz0 /= m0; }
    if (m1 > 0) { x1 /= m1; y1 /= m1; z1 /= m1; vx1 /= m1; vy1 /= m1; vz1 /= m1; }
    o->massBody0Psu = m0; o->massOtherPsu = m1;
    const double c0[6] = {x0, y0, z0, vx0, vy0, vz0}, c1[6] = {x1, y1, z1, vx1, vy1, vz1};
    for (int k = 0; k < 3; ++k) {
        o->comBody0Psu[k] = c0[k]; o->velBody0Psu[k] = c0[3 + k];
        o->comOtherPsu[k] = c1[k]; o->velOtherPsu[k] = c1[3 + k];
        o->livingComPsu[k] = m0 > 0 ? c0[k] : o->sysComPsu[k];
    }
    o->kineticPsu = ke; o->potentialPsu = pe; o->internalPsu = ie;
    o->momentumPsu[0] = px; o->momentumPsu[1] = py; o->momentumPsu[2] = pz;
    o->angularMomentumPsu[0] = lx; o->angularMomentumPsu[1] = ly; o->angularMomentumPsu[2] = lz;
    o->maxTempK = maxT; o->maxPressureGPa = maxP; o->radiatedPowerW = rad;
    o->remnantSeedIndex = seed;
    if (prm->livingBodyPresent) {                                   // :1092-1111
        double L = 0, I = 0;
        const double rLim2 = (1.5 * targetR) * (1.5 * targetR);
        for (uint32_t i = 0; i < n; ++i) {
            if (p->bodyId[i] != 0) continue;
            const double dx = static_cast<double>(p->posX[i]) - x0, dy = static_cast<double>(p->posY[i]) - y0,
                         dz = static_cast<double>(p->posZ[i]) - z0;
            if (dx * dx + dy * dy + dz * dz <= rLim2) {
                const double m = p->mass[i];
                const double dvx = static_cast<double>(p->velX[i]) - vx0, dvz = static_cast<double>(p->velZ[i]) - vz0;
                L += m * (dz * dvx - dx * dvz);
                I += m * (dx * dx + dz * dz);
            }
        }
        o->spinLPsu = L; o->spinIPsu = I;
    }
    double rX = p->posX[seed], rY = p->posY[seed], rZ = p->posZ[seed];   // :1121-1128
    double rVx = p->velX[seed], rVy = p->velY[seed], rVz = p->velZ[seed];
    double rM = std::max(m0, M * 0.5), rR = std::max(targetR, 0.25);
    int iters = 0;
    for (int it = 0; it < 5; ++it) {                                  // :1131-1174
        double nm = 0, nx = 0, ny = 0, nz = 0, nvx = 0, nvy = 0, nvz = 0, mr2 = 0;
        const double rSoft = std::max(0.5 * rR, 0.1);
        for (uint32_t i = 0; i < n; ++i) {
            const double dx = static_cast<double>(p->posX[i]) - rX, dy = static_cast<double>(p->posY[i]) - rY,
                         dz = static_cast<double>(p->posZ[i]) - rZ;
            const double r2 = dx * dx + dy * dy + dz * dz, r = std::sqrt(r2);
            const double dvx = static_cast<double>(p->velX[i]) - rVx, dvy = static_cast<double>(p->velY[i]) - rVy,
                         dvz = static_cast<double>(p->velZ[i]) - rVz;
            const double v2 = dvx * dvx + dvy * dvy + dvz * dvz;
            const double e = 0.5 * v2 + (-G * rM / std::max(r, rSoft));
            if (e < 0.0) {
                const double m = p->mass[i];
                nm += m; nx += m * p->posX[i]; ny += m * p->posY[i]; nz += m * p->posZ[i];
                nvx += m * p->velX[i]; nvy += m * p->velY[i]; nvz += m * p->velZ[i];
                mr2 += m * r2;
            }
        }
        if (!(nm > 0.0)) break;
        rM = nm; rX = nx / nm; rY = ny / nm; rZ = nz / nm; rVx = nvx / nm; rVy = nvy / nm; rVz = nvz / nm;
        rR = std::max(0.5 * targetR, std::sqrt(5.0 / 3.0) * std::sqrt(mr2 / nm));
        ++iters;
    }
    double bound = 0, disk = 0, ej = 0, impB = 0, maxD = 0;
    const double rSoftF = std::max(0.5 * rR, 0.1), mu = G * rM;
    for (uint32_t i = 0; i < n; ++i) {                                // :1183-1224
        const double m = p->mass[i];
        maxD = std::max(maxD, static_cast<double>(p->damage[i]));
        const double dx = static_cast<double>(p->posX[i]) - rX, dy = static_cast<double>(p->posY[i]) - rY,
                     dz = static_cast<double>(p->posZ[i]) - rZ;
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        const double dvx = static_cast<double>(p->velX[i]) - rVx, dvy = static_cast<double>(p->velY[i]) - rVy,
                     dvz = static_cast<double>(p->velZ[i]) - rVz;
        const double v2 = dvx * dvx + dvy * dvy + dvz * dvz;
        const double e = 0.5 * v2 + (-mu / std::max(r, rSoftF));
        if (e >= 0.0) { ej += m; continue; }
        if (p->bodyId[i] != 0) impB += m;
        bool isDisk = false;
        if (r > rR && mu > 0.0) {
            const double jx = dy * dvz - dz * dvy, jy = dz * dvx - dx * dvz, jz = dx * dvy - dy * dvx;
            const double j2 = jx * jx + jy * jy + jz * jz;
            const double ecc = std::sqrt(std::max(0.0, 1.0 + (2.0 * e * j2) / (mu * mu)));
            isDisk = j2 / (mu * (1.0 + ecc)) > rR;
        }
        (isDisk ? disk : bound) += m;
    }
    o->maxDamage = maxD;
    o->boundPlanetMassPsu = bound; o->diskMassPsu = disk; o->ejectaMassPsu = ej; o->impactorBoundMassPsu = impB;
    o->remnantPsu[0] = rX; o->remnantPsu[1] = rY; o->remnantPsu[2] = rZ;
    o->remnantVelPsu[0] = rVx; o->remnantVelPsu[1] = rVy; o->remnantVelPsu[2] = rVz;
    o->remnantMassPsu = rM; o->remnantRadiusPsu = rR;
    o->remnantIterations = iters;
}

int oracle_abi_version(void) { return ASTRAEA_GB300_ABI_VERSION; }
void oracle_set_group_stride(int k) { g_groupStride = k < 1 ? 1 : k; }
void oracle_set_r2_form(int k) { g_r2Form = (k >= 0 && k <= 2) ? k : 0; }

}  // extern "C"

// ======================================================== planet builder ===
// Restates engine/planet_builder.cpp (PlanetBuilder::solveHydrostatic1D and
// ::buildPlanet) with the archetype table of engine/presets.cpp:9-88 and the
// host EOS helpers of engine/eos.cu:390-535, in the reference's own order of
// operations.  Writes the body into HOST particle arrays the way the engine's
// upload writes it (engine/simulation.cpp:468-523, 852-880).
namespace {

constexpr double kLUnitD = 1.0e6, kMUnitD = 1.0e24, kTUnitD = 1.0e3;
constexpr double kRhoUnitD = kMUnitD / (kLUnitD * kLUnitD * kLUnitD);
constexpr double kPUnitD = kMUnitD / (kLUnitD * kTUnitD * kTUnitD);
constexpr double kUUnitD = (kLUnitD * kLUnitD) / (kTUnitD * kTUnitD);
constexpr double kGSiD = 6.67430e-11;

struct Layers { uint32_t count; int mat[3]; double frac[3]; };
const Layers kArchLayers[6] = {
    {3, {0, 1, 2}, {0.320, 0.675, 0.005}}, {2, {0, 1, 1}, {0.680, 0.320, 0.0}},
    {3, {0, 1, 2}, {0.150, 0.450, 0.400}}, {2, {0, 1, 1}, {0.250, 0.750, 0.0}},
    {3, {0, 1, 3}, {0.050, 0.100, 0.850}}, {3, {0, 1, 4}, {0.220, 0.580, 0.200}},
};
const Layers& archLayers(uint32_t a) { return kArchLayers[a > 5 ? 0 : a]; }   // presets.cpp:92-98

inline double mxD(double a, double b) { return a > b ? a : b; }
inline double clD(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// engine/eos.cu:390-442
void fromRhoTempSI(int mat, double rhoKgM3, double tempK, double& uSi, double& pSi) {
    const MatParams& p = kMat[matIndex(mat)];
    const double rho = mxD(rhoKgM3, 1.0e-12);
    const double tc = mxD(tempK, 0.0);
    if (mat == kHH) {
        const double uColdSi = p.kH2 * rho;
        const double uThSi = p.cv * tc;
        uSi = uColdSi + uThSi;
        pSi = p.kH2 * rho * rho + (p.gamma - 1.0) * rho * uThSi;
        return;
    }
    const double rhoPsu = rho / kRhoUnitD;
    const double uColdPsu = coldEnergy(mat, rhoPsu);
    const double uColdSi = uColdPsu * kUUnitD;
    uSi = uColdSi + p.cv * tc;
    const double uThExcess = mxD(0.0, uSi - uColdSi - p.cv * p.tRef);
    const double uEosPsu = uColdPsu + uThExcess / kUUnitD;
    const double rho0Psu = p.rho0 / kRhoUnitD;
    const double eta = rhoPsu / rho0Psu;
    const double mu = eta - 1.0;
    const double Eiv = p.Eiv / kUUnitD, Ecv = p.Ecv / kUUnitD;
    double pr;
    if (eta >= 1.0 || uEosPsu < Eiv) {
        pr = tillotsonCompressed(p, rhoPsu, rho0Psu, eta, mu, uEosPsu, 0.0).p;
    } else if (uEosPsu >= Ecv) {
        pr = tillotsonExpanded(p, rhoPsu, rho0Psu, eta, mu, uEosPsu).p;
    } else {
        const double pc = tillotsonCompressed(p, rhoPsu, rho0Psu, eta, mu, uEosPsu, 0.0).p;
        const double pe = tillotsonExpanded(p, rhoPsu, rho0Psu, eta, mu, uEosPsu).p;
        const double f = clD((uEosPsu - Eiv) / mxD(1.0e-30, Ecv - Eiv), 0.0, 1.0);
        pr = (1.0 - f) * pc + f * pe;
    }
    pSi = pr * kPUnitD;
}

// engine/eos.cu:444-535
double invertDensity(int mat, double targetPSi, double tempK, double rhoGuess) {
    const MatParams& p = kMat[matIndex(mat)];
    if (mat == kHH) {
        if (targetPSi <= 0.0) return 1.0e-6;
        const double bLin = (p.gamma - 1.0) * p.cv * mxD(tempK, 0.0);
        const double disc = std::sqrt(bLin * bLin + 4.0 * p.kH2 * targetPSi);
        return (2.0 * targetPSi) / mxD(1.0e-30, bLin + disc);
    }
    auto evalP = [&](double rho) {
        double u = 0.0, pp = 0.0;
        fromRhoTempSI(mat, rho, tempK, u, pp);
        return pp;
    };
    double rhoStart = (rhoGuess > 0.0) ? rhoGuess : p.rho0;
    rhoStart = clD(rhoStart, 0.05 * p.rho0, 50.0 * p.rho0);
    double rhoLow = rhoStart, rhoHigh = rhoStart;
    const double pStart = evalP(rhoStart);
    if (pStart > targetPSi) {
        for (int i = 0; i < 64; ++i) {
            rhoLow *= (i < 12) ? 0.85 : 0.5;
            if (rhoLow < 1.0e-6) rhoLow = 1.0e-6;
            if (evalP(rhoLow) <= targetPSi || rhoLow <= 1.0e-6) break;
        }
    } else if (pStart < targetPSi) {
        for (int i = 0; i < 64; ++i) {
            rhoHigh *= (i < 12) ? 1.25 : 2.0;
            if (evalP(rhoHigh) >= targetPSi || rhoHigh > 1.0e8) break;
        }
    } else {
        return rhoStart;
    }
    double fLow = evalP(rhoLow) - targetPSi;
    double fHigh = evalP(rhoHigh) - targetPSi;
    if (fLow >= 0.0) return rhoLow;
    if (fHigh <= 0.0) return rhoHigh;
    double rho = 0.5 * (rhoLow + rhoHigh);
    for (int iter = 0; iter < 64; ++iter) {
        const double fMid = evalP(rho) - targetPSi;
        if (std::abs(fMid) <= 1.0e-9 * mxD(1.0, std::abs(targetPSi))) return rho;
        if (fMid < 0.0) { rhoLow = rho; fLow = fMid; } else { rhoHigh = rho; fHigh = fMid; }
        if (rhoHigh - rhoLow <= 1.0e-12 * mxD(1.0, rho)) return 0.5 * (rhoLow + rhoHigh);
        double nextRho = 0.5 * (rhoLow + rhoHigh);
        const double denom = fHigh - fLow;
        if (std::abs(denom) > 1.0e-30) {
            const double secant = rhoLow - fLow * (rhoHigh - rhoLow) / denom;
            if (secant > rhoLow && secant < rhoHigh) nextRho = secant;
        }
        rho = nextRho;
    }
    return 0.5 * (rhoLow + rhoHigh);
}

struct PSample { double r, rho, P, M, T; int mat; };

// planet_builder.cpp:21-46
double densityOnGeotherm(const AstraeaBodySpec& s, int mat, double P, double pc, double pSurf, double guess,
                         double& outT) {
    const double denom = std::max(pc - pSurf, 1.0);
    const double pFrac = std::clamp((P - pSurf) / denom, 0.0, 1.0);
    outT = s.surfaceTempK + (s.coreTempK - s.surfaceTempK) * pFrac;
    double rho = invertDensity(mat, std::max(P, 0.0), outT, guess);
    if (mat == kHH) rho = std::max(rho, 1.0e-3);
    return rho;
}

struct ShootRes { double radius = 0.0, mass = 0.0; bool cap = false; std::vector<PSample> prof; };

// planet_builder.cpp:55-264
ShootRes shootOutward(const AstraeaBodySpec& s, double pc, double pSurf, double drM, bool rec) {
    ShootRes res;
    const Layers& comp = archLayers(s.archetype);
    const double target = s.massKg;
    const double bail = 20.0 * target;
    double layerEnd[3] = {};
    double cum = 0.0;
    for (uint32_t i = 0; i < comp.count; ++i) {
        cum += comp.frac[i];
        layerEnd[i] = (i + 1 == comp.count) ? std::numeric_limits<double>::infinity() : (cum * target);
    }
    uint32_t li = 0;
    double r = 0.0, P = pc, M = 0.0;
    const int mat0 = comp.mat[0];
    double t0 = s.coreTempK;
    double guess = kMat[matIndex(mat0)].rho0;
    double rho = densityOnGeotherm(s, mat0, P, pc, pSurf, guess, t0);
    guess = rho;
    if (rec) res.prof.push_back({0.0, rho, P, 0.0, t0, mat0});
    auto deriv = [&](int mat, double rv, double pv, double mv, double hint, double& dP, double& dM) {
        double tk = t0;
        const double rl = densityOnGeotherm(s, mat, pv, pc, pSurf, hint, tk);
        dM = 4.0 * kPiD * rv * rv * rl;
        if (rv <= 1.0e-9) dP = -(4.0 / 3.0) * kPiD * kGSiD * rl * rl * rv;
        else dP = -kGSiD * mv * rl / (rv * rv);
        return rl;
    };
    auto rk4 = [&](int mat, double r0, double p0, double m0, double h, double hint, double& oP, double& oM) {
        double k1P = 0, k1M = 0, k2P = 0, k2M = 0, k3P = 0, k3M = 0, k4P = 0, k4M = 0;
        const double r1 = deriv(mat, r0, p0, m0, hint, k1P, k1M);
        const double r2 = deriv(mat, r0 + 0.5 * h, std::max(pSurf, p0 + 0.5 * h * k1P), m0 + 0.5 * h * k1M, r1, k2P, k2M);
        const double r3 = deriv(mat, r0 + 0.5 * h, std::max(pSurf, p0 + 0.5 * h * k2P), m0 + 0.5 * h * k2M, r2, k3P, k3M);
        deriv(mat, r0 + h, std::max(pSurf, p0 + h * k3P), m0 + h * k3M, r3, k4P, k4M);
        oP = p0 + (h / 6.0) * (k1P + 2.0 * k2P + 2.0 * k3P + k4P);
        oM = m0 + (h / 6.0) * (k1M + 2.0 * k2M + 2.0 * k3M + k4M);
    };
    for (int step = 0; step < 12000; ++step) {
        const int mat = comp.mat[li];
        const double h = (s.archetype == 4 && li + 1 < comp.count) ? (0.25 * drM) : drM;
        double nP = P, nM = M;
        if (r == 0.0) {
            nP = P - (2.0 / 3.0) * kPiD * kGSiD * rho * rho * h * h;
            nM = (4.0 / 3.0) * kPiD * rho * h * h * h;
        } else {
            rk4(mat, r, P, M, h, guess, nP, nM);
        }
        const bool cS = nP <= pSurf;
        const bool cL = (li + 1 < comp.count) && (nM >= layerEnd[li]);
        const double fP = cS ? ((P - nP > 1.0e-30) ? std::clamp((P - pSurf) / (P - nP), 0.0, 1.0) : 1.0) : 2.0;
        const double fM = cL ? ((nM - M > 1.0e-30) ? std::clamp((layerEnd[li] - M) / (nM - M), 0.0, 1.0) : 1.0) : 2.0;
        if (cS && (!cL || fP <= fM)) {
            double rS = r + fP * h, mS = M;
            if (r == 0.0) {
                const double dp = std::max(0.0, P - pSurf);
                const double rA = std::sqrt(dp / ((2.0 / 3.0) * kPiD * kGSiD * rho * rho));
                rS = std::min(h, rA);
                mS = (4.0 / 3.0) * kPiD * rho * rS * rS * rS;
            } else {
                double d = 0.0;
                rk4(mat, r, P, M, fP * h, guess, d, mS);
            }
            if (rec) {
                double tS = s.surfaceTempK;
                const double rhoS = densityOnGeotherm(s, mat, pSurf, pc, pSurf, guess, tS);
                res.prof.push_back({rS, rhoS, pSurf, mS, tS, mat});
            }
            res.radius = rS; res.mass = mS;
            return res;
        }
        if (cL) {
            const double mB = layerEnd[li];
            double sub = 0.0;
            if (r == 0.0) {
                sub = std::cbrt((3.0 * mB) / (4.0 * kPiD * rho));
                sub = std::clamp(sub, 0.0, h);
                nP = P - (2.0 / 3.0) * kPiD * kGSiD * rho * rho * sub * sub;
                nM = mB;
            } else {
                double lo = 0.0, hi = h;
                sub = fM * h;
                for (int it = 0; it < 4; ++it) {
                    rk4(mat, r, P, M, sub, guess, nP, nM);
                    if (std::abs(nM - mB) <= 1.0e-10 * target) break;
                    if (nM < mB) lo = sub; else hi = sub;
                    sub = 0.5 * (lo + hi);
                }
                rk4(mat, r, P, M, sub, guess, nP, nM);
            }
            if (nP <= pSurf) {
                const double den = P - nP;
                const double sf = (den > 1.0e-30) ? std::clamp((P - pSurf) / den, 0.0, 1.0) : 1.0;
                const double rS = r + sf * sub;
                double d = 0.0, mS = M;
                rk4(mat, r, P, M, sf * sub, guess, d, mS);
                if (rec) {
                    double tS = s.surfaceTempK;
                    const double rhoS = densityOnGeotherm(s, mat, pSurf, pc, pSurf, guess, tS);
                    res.prof.push_back({rS, rhoS, pSurf, mS, tS, mat});
                }
                res.radius = rS; res.mass = mS;
                return res;
            }
            r += sub; P = nP; M = mB;
            if (rec) {
                double tE = 0.0;
                const double rhoE = densityOnGeotherm(s, mat, P, pc, pSurf, guess, tE);
                res.prof.push_back({r, rhoE, P, M, tE, mat});
            }
            ++li;
            const int nm = comp.mat[li];
            double tN = 0.0;
            guess = kMat[matIndex(nm)].rho0;
            rho = densityOnGeotherm(s, nm, P, pc, pSurf, guess, tN);
            guess = rho;
            if (rec) res.prof.push_back({r, rho, P, M, tN, nm});
            continue;
        }
        r += h; P = nP; M = nM;
        double tC = s.coreTempK;
        rho = densityOnGeotherm(s, mat, P, pc, pSurf, guess, tC);
        guess = rho;
        if (rec) res.prof.push_back({r, rho, P, M, tC, mat});
        if (M > bail) { res.radius = r; res.mass = M; res.cap = true; return res; }
    }
    res.radius = r; res.mass = M;
    return res;
}

// planet_builder.cpp:398-473
bool solveHydrostatic(const AstraeaBodySpec& s, std::vector<PSample>& prof, double& radius, double& pcOut) {
    if (!(s.massKg > 0.0) || s.archetype > 5) return false;
    const Layers& comp = archLayers(s.archetype);
    const double pSurf = (s.archetype == 4) ? 1.0e5 : 0.0;
    double invRho = 0.0;
    for (uint32_t i = 0; i < comp.count; ++i) {
        double rho0 = kMat[matIndex(comp.mat[i])].rho0;
        if (comp.mat[i] == kHH) rho0 = 600.0;
        invRho += comp.frac[i] / std::max(rho0, 1.0);
    }
    const double rhoEst = 1.0 / std::max(invRho, 1.0e-6);
    double rEst = std::cbrt((3.0 * s.massKg) / (4.0 * kPiD * rhoEst));
    if (s.archetype == 4) rEst = std::max(rEst, 6.5e7);
    const double drM = std::max(rEst / 800.0, 1.0e2);
    const double pEst = (3.0 * kGSiD * s.massKg * s.massKg) / (8.0 * kPiD * rEst * rEst * rEst * rEst);
    double lo = std::log(std::max(pSurf + 1.0e4, 1.0e-3 * pEst));
    double hi = std::log(std::max(pSurf + 1.0e6, 1.0e3 * pEst));
    for (int i = 0; i < 20; ++i) {
        const ShootRes r = shootOutward(s, std::exp(lo), pSurf, drM, false);
        if (!r.cap && r.mass <= s.massKg) break;
        lo -= 2.0;
    }
    for (int i = 0; i < 20; ++i) {
        const ShootRes r = shootOutward(s, std::exp(hi), pSurf, drM, false);
        if (r.cap || r.mass >= s.massKg) break;
        hi += 2.0;
    }
    double mid = 0.5 * (lo + hi);
    for (int it = 0; it < 60; ++it) {
        mid = 0.5 * (lo + hi);
        const ShootRes r = shootOutward(s, std::exp(mid), pSurf, drM, false);
        const double rel = (r.mass - s.massKg) / s.massKg;
        if (!r.cap && std::abs(rel) <= 1.0e-6) break;
        if (r.cap || r.mass > s.massKg) hi = mid; else lo = mid;
        if (hi - lo < 1.0e-12) break;
    }
    pcOut = std::exp(mid);
    ShootRes fin = shootOutward(s, pcOut, pSurf, drM, true);
    radius = fin.radius;
    prof = std::move(fin.prof);
    return !prof.empty();
}

// planet_builder.cpp:267-300
PSample atMass(const std::vector<PSample>& prof, double m) {
    if (prof.empty()) return PSample{0, 0, 0, 0, 0, 1};
    if (m <= prof.front().M) return prof.front();
    if (m >= prof.back().M) return prof.back();
    auto it = std::lower_bound(prof.begin(), prof.end(), m, [](const PSample& a, double v) { return a.M < v; });
    if (it == prof.begin()) return *it;
    const PSample& h = *it;
    const PSample& l = *(it - 1);
    const double dm = h.M - l.M;
    const double t = (dm > 1.0e-30) ? std::clamp((m - l.M) / dm, 0.0, 1.0) : 0.0;
    PSample o;
    o.r = l.r + t * (h.r - l.r);
    o.rho = l.rho + t * (h.rho - l.rho);
    o.P = l.P + t * (h.P - l.P);
    o.M = m;
    o.T = l.T + t * (h.T - l.T);
    o.mat = (t < 0.5) ? l.mat : h.mat;
    return o;
}

// planet_builder.cpp:329-396
void faceUvToNormal(uint32_t face, float u, float v, float& nx, float& ny, float& nz) {
    const float sx = 2.0f * u - 1.0f, sy = 2.0f * v - 1.0f;
    float vx = 0.0f, vy = 0.0f, vz = 0.0f;
    switch (face % 6u) {
        case 0: vx = 1.0f; vy = sy; vz = -sx; break;
        case 1: vx = -1.0f; vy = sy; vz = sx; break;
        case 2: vx = sx; vy = 1.0f; vz = -sy; break;
        case 3: vx = sx; vy = -1.0f; vz = sy; break;
        case 4: vx = sx; vy = sy; vz = 1.0f; break;
        case 5: vx = -sx; vy = sy; vz = -1.0f; break;
    }
    const float inv = 1.0f / std::sqrt(vx * vx + vy * vy + vz * vz);
    nx = vx * inv; ny = vy * inv; nz = vz * inv;
}

void normalToFaceUv(float nx, float ny, float nz, uint32_t& face, float& u, float& v) {
    const float ax = std::abs(nx), ay = std::abs(ny), az = std::abs(nz);
    float sx = 0.0f, sy = 0.0f;
    if (ax >= ay && ax >= az) {
        const float d = std::max(ax, 1.0e-12f);
        if (nx >= 0.0f) { face = 0; sx = -nz / d; sy = ny / d; } else { face = 1; sx = nz / d; sy = ny / d; }
    } else if (ay >= ax && ay >= az) {
        const float d = std::max(ay, 1.0e-12f);
        if (ny >= 0.0f) { face = 2; sx = nx / d; sy = -nz / d; } else { face = 3; sx = nx / d; sy = nz / d; }
    } else {
        const float d = std::max(az, 1.0e-12f);
        if (nz >= 0.0f) { face = 4; sx = nx / d; sy = ny / d; } else { face = 5; sx = -nx / d; sy = ny / d; }
    }
    u = std::clamp(0.5f * (sx + 1.0f), 0.0f, 1.0f);
    v = std::clamp(0.5f * (sy + 1.0f), 0.0f, 1.0f);
}

}  // namespace

extern "C" {

int oracle_solve_hydrostatic(const AstraeaBodySpec* s, AstraeaRadialSample* out, uint32_t cap, uint32_t* count,
                             double* radius, double* pc) {
    std::vector<PSample> prof;
    if (!solveHydrostatic(*s, prof, *radius, *pc)) return ASTRAEA_ERR_INVALID;
    *count = static_cast<uint32_t>(prof.size());
    if (out == nullptr || cap < prof.size()) return ASTRAEA_ERR_CAPACITY;
    for (size_t i = 0; i < prof.size(); ++i)
        out[i] = AstraeaRadialSample{prof[i].r, prof[i].rho, prof[i].P, prof[i].M, prof[i].T,
                                     static_cast<uint32_t>(prof[i].mat), 0u};
    return ASTRAEA_OK;
}

// planet_builder.cpp:475-905 into HOST arrays [offset, offset + n) of p.
// stableTies = 0 orders tracer candidates with std::sort as the engine does;
// 1 keeps particle order among equal radii (std::stable_sort).
int oracle_build_planet(const AstraeaBodySpec* spec, uint32_t n, uint32_t bodyId, uint32_t grid, uint64_t seed,
                        int stableTies, AstraeaParticles* p, uint32_t offset, AstraeaPlanetInfo* info) {
    if (n == 0) return ASTRAEA_ERR_INVALID;
    std::vector<PSample> prof;
    double radius = 0.0, pcPa = 0.0;
    if (!solveHydrostatic(*spec, prof, radius, pcPa)) return ASTRAEA_ERR_INVALID;
    const double actualMass = prof.back().M;
    const Layers& comp = archLayers(spec->archetype);
    const uint32_t L = comp.count;
    uint32_t layerN[3] = {};
    double cumEnd[3] = {};
    double cumFrac = 0.0;
    uint32_t given = 0;
    for (uint32_t k = 0; k < L; ++k) {
        cumFrac += comp.frac[k];
        cumEnd[k] = (k + 1 == L) ? actualMass : (cumFrac * actualMass);
        if (k + 1 == L) {
            layerN[k] = n - given;
        } else {
            uint32_t c = static_cast<uint32_t>(std::llround(comp.frac[k] * n));
            if (n >= L && c == 0) c = 1;
            const uint32_t maxAvail = n - given - ((n >= L) ? (L - 1 - k) : 0u);
            c = std::min(c, maxAvail);
            layerN[k] = c;
            given += c;
        }
    }
    std::mt19937_64 rng(seed ^ (static_cast<uint64_t>(static_cast<uint8_t>(bodyId)) * 0x9e3779b97f4a7c15ULL));
    std::uniform_real_distribution<double> u01(1.0e-6, 1.0 - 1.0e-6);
    const double nominalMass = actualMass / static_cast<double>(n);
    const double golden = kPiD * (3.0 - std::sqrt(5.0));
    uint32_t g = 0, shellsPlaced = 0;
    double mStart = 0.0;
    for (uint32_t k = 0; k < L; ++k) {
        const uint32_t nk = layerN[k];
        const double mEnd = cumEnd[k];
        if (nk == 0) { mStart = mEnd; continue; }
        const double layerTotal = std::max(mEnd - mStart, 0.0);
        const double pMassKg = layerTotal / static_cast<double>(nk);
        const double pMassPsu = pMassKg / kMUnitD;
        const int mat = comp.mat[k];
        const MatParams& ep = kMat[matIndex(mat)];
        const PSample sIn = atMass(prof, mStart);
        const PSample sOut = atMass(prof, mEnd);
        std::vector<double> bounds{mStart};
        double curM = mStart, curR = sIn.r;
        if (k == 0 && nk >= 2 && sOut.r > 0.0) {
            const double cM = std::min(mStart + pMassKg, mEnd);
            const double cR = std::cbrt((3.0 * cM) / (4.0 * kPiD * std::max(sIn.rho, 1.0e-3)));
            if (cM < mEnd && cR < sOut.r) { bounds.push_back(cM); curM = cM; curR = cR; }
        }
        auto massAtR = [&](double rT) {
            auto it = std::lower_bound(prof.begin(), prof.end(), rT, [](const PSample& a, double v) { return a.r < v; });
            double mv = mEnd;
            if (it != prof.end() && it != prof.begin()) {
                const PSample& h = *it;
                const PSample& l = *(it - 1);
                const double dr = h.r - l.r;
                const double t = (dr > 1.0e-30) ? std::clamp((rT - l.r) / dr, 0.0, 1.0) : 0.0;
                mv = l.M + t * (h.M - l.M);
            }
            return std::clamp(mv, curM + 1.0e-9 * layerTotal, mEnd);
        };
        while (curM < mEnd) {
            const PSample sc = atMass(prof, curM);
            const double spacing = std::cbrt(nominalMass / std::max(sc.rho, 1.0e-3));
            const double stepR = (k == 0 && nk >= 64 && curR < 3.5 * spacing) ? (0.62 * spacing) : spacing;
            const double nextR = curR + stepR;
            if (nextR >= sOut.r - 0.35 * stepR) { bounds.push_back(mEnd); break; }
            const double nextM = massAtR(nextR);
            bounds.push_back(nextM);
            if (nextM >= mEnd) break;
            curM = nextM; curR = nextR;
        }
        if (bounds.size() < 2) bounds.push_back(mEnd);
        if (bounds.size() == 2 && nk >= 128 && sOut.r > sIn.r) {
            const double avgRho = std::max(0.5 * (sIn.rho + sOut.rho), 1.0e-3);
            const double lsp = std::cbrt(nominalMass / avgRho);
            if ((sOut.r - sIn.r) > 0.25 * lsp) {
                bounds.clear();
                bounds.push_back(mStart);
                curM = mStart;
                for (size_t sub = 1; sub < 3; ++sub) {
                    const double fr = static_cast<double>(sub) / static_cast<double>(3);
                    const double nextM = massAtR(sIn.r + fr * (sOut.r - sIn.r));
                    if (nextM > curM && nextM < mEnd) { bounds.push_back(nextM); curM = nextM; }
                }
                bounds.push_back(mEnd);
            }
        }
        const size_t S = bounds.size() - 1;
        std::vector<uint32_t> cnt(S, 0);
        std::vector<double> rem(S, 0.0);
        uint32_t sum = 0;
        for (size_t s = 0; s < S; ++s) {
            const double dm = bounds[s + 1] - bounds[s];
            const double ex = (layerTotal > 0.0) ? (static_cast<double>(nk) * (dm / layerTotal)) : 0.0;
            const uint32_t fl = static_cast<uint32_t>(std::floor(ex));
            cnt[s] = fl; rem[s] = ex - static_cast<double>(fl); sum += fl;
        }
        if (sum < nk) {
            std::vector<size_t> idx(S);
            std::iota(idx.begin(), idx.end(), 0);
            std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return rem[a] > rem[b]; });
            for (uint32_t r = 0; r < nk - sum; ++r) cnt[idx[r % S]] += 1;
        }
        for (size_t s = 0; s < S; ++s) {
            const uint32_t ns = cnt[s];
            if (ns == 0) continue;
            ++shellsPlaced;
            const double mMid = 0.5 * (bounds[s] + bounds[s + 1]);
            const PSample smp = atMass(prof, mMid);
            const double rShell = (s == 0 && k == 0 && ns == 1) ? 0.0 : smp.r;
            const double rho = std::max(smp.rho, 1.0e-3);
            const double tK = smp.T;
            double uSi = 0.0, pSi = 0.0;
            fromRhoTempSI(mat, rho, tK, uSi, pSi);
            const double rPsu = rShell / kLUnitD;
            const double rhoPsu = rho / kRhoUnitD;
            const double uPsu = uSi / kUUnitD;
            const double h0Psu = 1.2 * std::cbrt(pMassPsu / rhoPsu);
            // Shoemake rotation, planet_builder.cpp:303-326
            std::uniform_real_distribution<double> r01(0.0, 1.0);
            const double q1 = r01(rng);
            const double q2 = 2.0 * kPiD * r01(rng);
            const double q3 = 2.0 * kPiD * r01(rng);
            const double s1 = std::sqrt(std::max(0.0, 1.0 - q1)), s2 = std::sqrt(std::max(0.0, q1));
            const double qx = s1 * std::sin(q2), qy = s1 * std::cos(q2), qz = s2 * std::sin(q3), qw = s2 * std::cos(q3);
            const double xx = qx * qx, yy = qy * qy, zz = qz * qz, xy = qx * qy, xz = qx * qz, yz = qy * qz;
            const double wx = qw * qx, wy = qw * qy, wz = qw * qz;
            const double rot[9] = {1.0 - 2.0 * (yy + zz), 2.0 * (xy - wz), 2.0 * (xz + wy),
                                   2.0 * (xy + wz), 1.0 - 2.0 * (xx + zz), 2.0 * (yz - wx),
                                   2.0 * (xz - wy), 2.0 * (yz + wx), 1.0 - 2.0 * (xx + yy)};
            for (uint32_t q = 0; q < ns; ++q) {
                double px = 0.0, py = 0.0, pz = 0.0;
                if (rPsu > 0.0) {
                    const double zl = (ns == 1) ? 1.0 : (1.0 - 2.0 * (static_cast<double>(q) + 0.5) / static_cast<double>(ns));
                    const double rxy = std::sqrt(std::max(0.0, 1.0 - zl * zl));
                    const double th = golden * static_cast<double>(q);
                    const double ux = rxy * std::cos(th), uy = rxy * std::sin(th), uz = zl;
                    px = rPsu * (rot[0] * ux + rot[1] * uy + rot[2] * uz);
                    py = rPsu * (rot[3] * ux + rot[4] * uy + rot[5] * uz);
                    pz = rPsu * (rot[6] * ux + rot[7] * uy + rot[8] * uz);
                }
                const double vx = spec->spinOmegaRadS * kTUnitD * pz;
                const double vz = -spec->spinOmegaRadS * kTUnitD * px;
                const double wDraw = -std::log(u01(rng));
                const double ws = std::clamp(std::pow(std::max(wDraw, 1.0e-6), 1.0 / 9.0), 1.0, 3.0);
                const uint32_t o = offset + g++;
                p->posX[o] = static_cast<float>(px); p->posY[o] = static_cast<float>(py); p->posZ[o] = static_cast<float>(pz);
                p->velX[o] = static_cast<float>(vx); p->velY[o] = 0.0f; p->velZ[o] = static_cast<float>(vz);
                p->velHalfX[o] = p->velX[o]; p->velHalfY[o] = 0.0f; p->velHalfZ[o] = p->velZ[o];
                p->mass[o] = static_cast<float>(pMassPsu);
                p->h0[o] = static_cast<float>(h0Psu); p->h[o] = p->h0[o];
                p->rho[o] = static_cast<float>(rhoPsu);
                p->u[o] = static_cast<float>(uPsu);
                p->tempK[o] = static_cast<float>(tK);
                p->epsFail[o] = static_cast<float>(ep.epsFailMin * ws);
                p->sXX[o] = p->sYY[o] = p->sZZ[o] = p->sXY[o] = p->sXZ[o] = p->sYZ[o] = 0.0f;
                p->damage[o] = 0.0f; p->damageCbrt[o] = 0.0f;
                p->pressure[o] = 0.0f; p->soundSpeed[o] = 0.0f; p->phaseId[o] = 0;
                p->materialId[o] = static_cast<uint8_t>(mat);
                p->bodyId[o] = static_cast<uint8_t>(bodyId);
                p->originalId[o] = o;
                p->tracerIndex[o] = -1;
                p->tracerRestRadiusPsu[o] = 0.0f;
                p->tracerRestNormalX[o] = p->tracerRestNormalY[o] = p->tracerRestNormalZ[o] = 0.0f;
                p->tracerIsOcean[o] = 0;
            }
        }
        mStart = mEnd;
    }
    if (g != n) return ASTRAEA_ERR_INVALID;

    // surface tracers, planet_builder.cpp:735-902
    uint32_t tracerCount = 0;
    const uint32_t T = 6u * grid * grid;
    if (spec->archetype == 0 && grid > 0 && n >= T) {
        std::vector<uint32_t> cand;
        std::vector<float> radii(n);
        for (uint32_t i = 0; i < n; ++i) {
            const float x = p->posX[offset + i], y = p->posY[offset + i], z = p->posZ[offset + i];
            radii[i] = std::sqrt(x * x + y * y + z * z);
            if (radii[i] > 1.0e-6f) cand.push_back(i);
        }
        auto byRadius = [&](uint32_t a, uint32_t b) { return radii[a] > radii[b]; };
        if (stableTies) std::stable_sort(cand.begin(), cand.end(), byRadius);
        else std::sort(cand.begin(), cand.end(), byRadius);
        if (cand.size() < T)
            for (uint32_t i = 0; i < n && cand.size() < T; ++i)
                if (radii[i] <= 1.0e-6f) cand.push_back(i);
        if (!cand.empty()) {
            const float rMax = radii[cand.front()];
            const float drSurf = p->h0[offset + cand.front()];
            size_t pool = 0;
            const size_t minPool = std::min(cand.size(), static_cast<size_t>(T) * 3u);
            for (; pool < cand.size(); ++pool) {
                const uint32_t pid = cand[pool];
                const bool inShell = (radii[pid] >= rMax - 1.8f * drSurf) || (p->materialId[offset + pid] == 2);
                if (!inShell && pool >= minPool) break;
            }
            if (pool < T) pool = std::min(cand.size(), static_cast<size_t>(T));
            cand.resize(pool);
            std::vector<float> cx(pool), cy(pool), cz(pool), tx(T), ty(T), tz(T);
            std::vector<uint8_t> used(pool, 0), filled(T, 0);
            std::vector<std::vector<uint32_t>> bins(T);
            for (size_t c = 0; c < pool; ++c) {
                const uint32_t pid = cand[c];
                if (radii[pid] > 1.0e-6f) {
                    const float inv = 1.0f / radii[pid];
                    cx[c] = p->posX[offset + pid] * inv; cy[c] = p->posY[offset + pid] * inv; cz[c] = p->posZ[offset + pid] * inv;
                } else {
                    cx[c] = 0.0f; cy[c] = 0.0f; cz[c] = 1.0f;
                }
                uint32_t face = 0;
                float u = 0.0f, v = 0.0f;
                normalToFaceUv(cx[c], cy[c], cz[c], face, u, v);
                const uint32_t gx = std::min(grid - 1u, static_cast<uint32_t>(u * static_cast<float>(grid)));
                const uint32_t gy = std::min(grid - 1u, static_cast<uint32_t>(v * static_cast<float>(grid)));
                bins[face * grid * grid + gy * grid + gx].push_back(static_cast<uint32_t>(c));
            }
            auto assign = [&](uint32_t b, size_t c) {
                const uint32_t o = offset + cand[c];
                used[c] = 1; filled[b] = 1; ++tracerCount;
                p->tracerIndex[o] = static_cast<int32_t>(b);
                p->tracerRestRadiusPsu[o] = radii[cand[c]];
                p->tracerRestNormalX[o] = cx[c]; p->tracerRestNormalY[o] = cy[c]; p->tracerRestNormalZ[o] = cz[c];
                p->tracerIsOcean[o] = (p->materialId[o] == 2) ? 1 : 0;
            };
            for (uint32_t face = 0; face < 6; ++face)
                for (uint32_t gy = 0; gy < grid; ++gy)
                    for (uint32_t gx = 0; gx < grid; ++gx) {
                        const uint32_t b = face * grid * grid + gy * grid + gx;
                        faceUvToNormal(face, (static_cast<float>(gx) + 0.5f) / static_cast<float>(grid),
                                       (static_cast<float>(gy) + 0.5f) / static_cast<float>(grid), tx[b], ty[b], tz[b]);
                        float best = -2.0f;
                        size_t bc = SIZE_MAX;
                        for (uint32_t c : bins[b]) {
                            if (used[c]) continue;
                            const float d = cx[c] * tx[b] + cy[c] * ty[b] + cz[c] * tz[b];
                            if (d > best) { best = d; bc = c; }
                        }
                        if (bc != SIZE_MAX) assign(b, bc);
                    }
            for (uint32_t b = 0; b < T; ++b) {
                if (filled[b]) continue;
                float best = -2.0f;
                size_t bc = SIZE_MAX;
                for (size_t c = 0; c < pool; ++c) {
                    if (used[c]) continue;
                    const float d = cx[c] * tx[b] + cy[c] * ty[b] + cz[c] * tz[b];
                    if (d > best) { best = d; bc = c; }
                }
                if (bc != SIZE_MAX) assign(b, bc);
            }
            if (tracerCount < T) {
                int32_t next = 0;
                for (uint32_t i = 0; i < n; ++i)
                    if (p->tracerIndex[offset + i] >= 0) p->tracerIndex[offset + i] = next++;
            }
        }
    }
    *info = AstraeaPlanetInfo{radius, actualMass, pcPa, tracerCount, static_cast<uint32_t>(prof.size()),
                              shellsPlaced, 0u};
    return ASTRAEA_OK;
}

}  // extern "C"
