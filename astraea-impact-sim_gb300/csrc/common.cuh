// common.cuh -- shared device definitions of the GB300 ASTRAEA physics path.
//
// Constants and small device functions used by every kernel.  Formulas cite
// the reference kernel they restate (engine/sph_gravity.cu, engine/eos.cu of
// Ananasjik/astraea-impact-sim).  Data layout (HBM, per particle / per node):
//
//   leaf    [N]   32-byte record {x, y, z, Hs}, {vx, vy, vz, m / max(rho, 1e-9)}   sorted positions,
//                 search radius, velocity, volume (rounded as pass 1 rounds it per pair)
//   leafAux [N]   float4 {Hs, eps, 2h, m}        Hs = search radius (below)
//   drift   [N]   32-byte record {x, y, z, H}, {vx, vy, vz, rho}   the next drift's neighbour record
//   rec2    [6N]  float4 x6 per particle          pass-2 neighbour record
//   node    [4(N-1)] float4 x4 per internal node:
//        r0 {comX, comY, comZ, mass}
//        r1 {dNode^2 (dNode = largest box side), left (int bits), right (int bits), maxHs}
//        r2 {minX, minY, minZ, maxH}             maxH = max 2h (engine field)
//        r3 {maxX, maxY, maxZ, 0}
//   nodeRange [N-1] uint2 {first, last} sorted leaf range of the node (refit)
//
// Search radius: pass 1 (engine/sph_gravity.cu:713) needs r < 2 h_old,
// pass 2 and the next drift (:1071, :1439) need r < max(2 h_i, 2 h_j) with
// h_new = clamp(h_old * f, 0.35 h0, 6 h0), f in [0.92, 1.08] (:785-787).
// Hs = 2 max(1.09 h_old, 0.351 h0) bounds every one of those radii, so one
// neighbour list per step, built against r < max(Hs_i, Hs_j), holds the
// exact neighbour set of all three passes (each pass re-applies its own
// exact test in FP32, in the reference's order of operations).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace astraea_gb300 {

constexpr float kPiF = 3.14159265358979323846f;
constexpr float kGPsuF = 66.7430f;        // engine/units.hpp:27
constexpr int kWarp = 32;
constexpr int kTreeStack = 128;           // per-thread DFS fallback stack

// Device status word flags (mirrors include/astraea_gb300.h).
constexpr uint32_t kFlagLookbackTimeout = 0x1u;
constexpr uint32_t kFlagNeighborOverflow = 0x2u;
constexpr uint32_t kFlagStackOverflow = 0x4u;

// Counters in DevStatus::counters.
enum Counter : int {
    kCntGravityInteractions = 0,   // particle-node + particle-particle evaluations
    kCntGravityNodeTests = 1,      // internal nodes tested by the group walk
    kCntNeighborEntries = 2,       // neighbour-list entries written
    kCntGravityRounds = 3,         // gravity walk rounds (up to 32 pending entries each)
    kCntGravityStackPeak = 4,      // deepest gravity walk stack (maximum, not a sum)
    kCntFallbackWalks = 5,         // particles served by the per-thread walk
    kCntNeighborCandidates = 6,    // leaves tested by the neighbour build (after the group-box filter)
    kCntGravityUndecided = 7,      // nodes the whole group had to test in the gravity walk
    kCntPass1Pairs = 8,            // pairs inside pass 1's radius (r < 2 h_i)
    kCntPass2Pairs = 9,            // pairs inside pass 2's radius (r < max(2 h_i, 2 h_j))
    kCntDriftPairs = 10,           // pairs inside the drift's radius
    kCntGravityGroupEvals = 11,    // far nodes taken by a group's expansion (far-field mode 3)
    kCntGravityBucketLeaves = 12,  // particle-particle terms from leaf buckets (far-field mode 3)
    kCntCount = 13
};

struct DevStatus {
    unsigned int flags;
    unsigned int dtBits;     // raw dt minimum of launchReduceDtPsu
    unsigned long long counters[kCntCount];
};

// ------------------------------------------------------------------ bits ---
__device__ __forceinline__ uint32_t orderedFromFloat(float f) {   // sph_gravity.cu:140-144
    const uint32_t u = __float_as_uint(f);
    return u ^ (static_cast<uint32_t>(-static_cast<int32_t>(u >> 31)) | 0x80000000u);
}
__device__ __forceinline__ float floatFromOrdered(uint32_t u) {   // sph_gravity.cu:146-149
    return __uint_as_float(u ^ (((u >> 31) - 1u) | 0x80000000u));
}
// Interleave the low 21 bits of v two zero bits apart (Morton spreading).
__device__ __forceinline__ uint64_t spreadBits21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x001f00000000ffffULL;
    v = (v | (v << 16)) & 0x001f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

// 32-byte read-only load (the 256-bit vector load of sm_100 and later): the
// two float4 halves of a 32-byte aligned record.  The SPH pair loops are
// bound by the L1 data pipe, which works per 32-byte sector per lane: one
// 32-byte load costs what a 16-byte load costs, so a record read in 32-byte
// pieces moves half the sectors of the same record read in 16-byte pieces.
struct F8 { float4 a, b; };
__device__ __forceinline__ F8 ldg256(const float4* p) {
    F8 r;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
    return r;
}

// Packed FP32 pairs for the f32x2 pipes (add/sub/mul/fma.rn.f32x2): lo and
// hi are two independent operands, each rounded as the scalar operation.
typedef unsigned long long f2;
__device__ __forceinline__ f2 pack2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) { f2 r; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { f2 r; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { f2 r; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b)); return r; }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Squared length with explicit IEEE rounding and no multiply-add fusion:
// ((dx*dx + dy*dy) + dz*dz).  Range and acceptance tests use this form so a
// pair's in/out decision is bit-identical to the oracle.
// |d|^2 rounded as the engine's compiled kernels round dx*dx + dy*dy + dz*dz:
// nvcc contracts that expression into fma(dz, dz, fma(dx, dx, dy*dy)) (the
// reference kernels' gravity on the 1M impact takes exactly the opening
// decisions of this form, and not those of the unfused sum, on the groups
// where the two differ).  Used wherever the engine decides with it: the
// gravity member test, the SPH range tests, the dt candidate.
__device__ __forceinline__ float len2Engine(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
}
__device__ __forceinline__ float len2Exact(float dx, float dy, float dz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
__device__ __forceinline__ float pointBoxDist2(float px, float py, float pz, float mnx, float mny, float mnz,
                                               float mxx, float mxy, float mxz) {
    const float dx = fmaxf(0.0f, fmaxf(__fsub_rn(mnx, px), __fsub_rn(px, mxx)));
    const float dy = fmaxf(0.0f, fmaxf(__fsub_rn(mny, py), __fsub_rn(py, mxy)));
    const float dz = fmaxf(0.0f, fmaxf(__fsub_rn(mnz, pz), __fsub_rn(pz, mxz)));
    return len2Exact(dx, dy, dz);
}

// ---------------------------------------------------------- SPH kernels ---
// Wendland C2 in 3-D with support H (sph_gravity.cu:199-208), its norm
// 21 / (2 pi H^3) computed once per particle with the engine's expression.
__device__ __forceinline__ float wendlandC2N(float r, float H, float norm) {   // norm = 21 / (2 pi H^3)
    if (r >= H || H <= 0.0f) return 0.0f;
    const float q = r / H;
    const float omq = 1.0f - q;
    const float omq2 = omq * omq;
    return norm * omq2 * omq2 * (1.0f + 4.0f * q);
}
__device__ __forceinline__ float wendlandNorm(float H) { return 21.0f / (2.0f * kPiF * H * H * H); }

// Pair-loop forms of the Wendland C2 kernel and of its gradient factor g,
// grad_i W(r_i - r_j, H) = g (r_i - r_j) (sph_gravity.cu:211-220, norm
// 210 / (pi H^5) computed once per particle).  The neighbour loops evaluate them
// once per pair; the IEEE quotient r / H (a dozen instructions with its
// special-case path) becomes three operations with y = 1 / H taken once per
// particle (or stored in its record): q0 = r y, the exact residual
// e = fma(-q0, H, r), q = fma(e, y, q0).  With y the correctly rounded
// reciprocal this one correction step returns the correctly rounded quotient
// (Markstein's theorem: P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119;
// J.-M. Muller et al., Handbook of Floating-Point Arithmetic, ch. 4), so the
// kernel values are the ones the engine's division gives; it holds while no
// operand or residual is subnormal (r, H >= 2e-6 here, r = 0 gives q = 0).
__device__ __forceinline__ float quotRN(float r, float H, float invH) {
    const float q0 = __fmul_rn(r, invH);
    return __fmaf_rn(__fmaf_rn(-q0, H, r), invH, q0);
}
__device__ __forceinline__ float wendlandC2I(float r, float H, float invH, float norm) {
    if (r >= H) return 0.0f;
    const float q = quotRN(r, H, invH);
    const float omq = 1.0f - q;
    const float omq2 = omq * omq;
    return norm * omq2 * omq2 * (1.0f + 4.0f * q);
}
__device__ __forceinline__ float wendlandC2GradI(float r, float H, float invH, float norm) {
    if (r >= H) return 0.0f;
    const float omq = 1.0f - quotRN(r, H, invH);
    return -norm * omq * omq * omq;
}
// Balsara switch (sph_gravity.cu:222-228).
__device__ __forceinline__ float balsaraSwitch(float divV, float cx, float cy, float cz, float cs, float h) {
    const float ad = fabsf(divV);
    const float ac = sqrtf(cx * cx + cy * cy + cz * cz);
    const float den = ad + ac + 1.0e-4f * fmaxf(cs, 0.05f) / fmaxf(h, 1.0e-6f);
    return ad / fmaxf(den, 1.0e-30f);
}
// Largest principal stress of (-P I + S), S traceless (sph_gravity.cu:230-254):
// trigonometric solution of the deviatoric cubic.
__device__ __forceinline__ float maxPrincipalStress(float P, float xx, float yy, float zz, float xy, float xz,
                                                    float yz) {
    const float p2 = xx * xx + yy * yy + zz * zz + 2.0f * (xy * xy + xz * xz + yz * yz);
    if (p2 <= 1.0e-24f) return -P;
    const float q = sqrtf(p2 * (1.0f / 6.0f));
    const float iq = 1.0f / q;
    const float bxx = xx * iq, byy = yy * iq, bzz = zz * iq, bxy = xy * iq, bxz = xz * iq, byz = yz * iq;
    const float det = bxx * (byy * bzz - byz * byz) - bxy * (bxy * bzz - byz * bxz) + bxz * (bxy * byz - byy * bxz);
    const float r = fminf(1.0f, fmaxf(-1.0f, 0.5f * det));
    const float phi = acosf(r) * (1.0f / 3.0f);
    return -P + 2.0f * q * cosf(phi);
}
__device__ __forceinline__ float effectivePressure(float P, uint8_t phase) {   // sph_gravity.cu:965-969
    return (phase != 0u) ? fmaxf(P, 0.0f) : P;
}

// ------------------------------------------------------ material tables ---
// Strength constants (sph_gravity.cu:35-73) and EOS parameters
// (eos.cu:10-116) in PSU (P in TPa, u in MJ/kg, rho in 1e6 kg/m^3).
struct MatConst {
    // strength
    float muShear, tMelt, bulkK, yieldY0;
    // EOS (FP32 path)
    float rho0, a, b, A, B, E0, Eiv, Ecv, alpha, beta;
    float rho0Lo;          // rho0 (double) - rho0 (float): the pair carries rho0 exactly
    float cv;              // MJ/(kg K)
    float cvTrefHi, cvTrefLo;   // cv * tRef as a float pair (hi + lo)
    float cMinCondensed;   // max(0.05, sqrt(A / rho0))
    float u0Ref;           // cv * 300 K (sph_gravity.cu:27-33)
    float kH2, gamma;      // HydrogenHelium polytrope + ideal gas
};

// Compile-time construction of the table from the published SI constants of
// engine/eos.cu:10-116 and engine/sph_gravity.cu:35-73.
constexpr double cxSqrt(double x) {
    double r = x > 1.0 ? x : 1.0;
    for (int i = 0; i < 200; ++i) r = 0.5 * (r + x / r);
    return r;
}
constexpr MatConst makeMat(double rho0Kg, double a, double b, double APa, double BPa, double E0, double Eiv,
                           double Ecv, double alpha, double beta, double cvSI, double tMelt, double tRef,
                           double muPa, double bulkPa, double y0Pa, double kH2, double gamma) {
    const double cv = cvSI / 1.0e6;
    const double cvTref = cv * tRef;
    const float hi = static_cast<float>(cvTref);
    const double rho0 = rho0Kg / 1.0e6;
    const double A = APa / 1.0e12;
    const double cMin = (A > 0.0) ? cxSqrt(A / rho0) : 0.0;
    return MatConst{static_cast<float>(muPa / 1.0e12), static_cast<float>(tMelt), static_cast<float>(bulkPa / 1.0e12),
                    static_cast<float>(y0Pa / 1.0e12), static_cast<float>(rho0), static_cast<float>(a),
                    static_cast<float>(b), static_cast<float>(A), static_cast<float>(BPa / 1.0e12),
                    static_cast<float>(E0 / 1.0e6), static_cast<float>(Eiv / 1.0e6), static_cast<float>(Ecv / 1.0e6),
                    static_cast<float>(alpha), static_cast<float>(beta),
                    static_cast<float>(rho0 - static_cast<double>(static_cast<float>(rho0))), static_cast<float>(cv), hi,
                    static_cast<float>(cvTref - static_cast<double>(hi)),
                    static_cast<float>(cMin > 0.05 ? cMin : 0.05),
                    static_cast<float>((cvSI * 300.0) / 1.0e6), static_cast<float>(kH2), static_cast<float>(gamma)};
}
// Strength columns (mu, T_melt, K, Y0) of the HydrogenHelium row are zero in
// engine/sph_gravity.cu:64-65, which disables the strength model for gas.
static __constant__ MatConst c_mat[5] = {
    makeMat(7800.0, 0.5, 1.5, 1.28e11, 1.05e11, 9.50e6, 2.40e6, 8.67e6, 5.0, 5.0, 449.0, 1811.0, 293.0, 7.70e10,
            1.28e11, 6.80e8, 0.0, 1.0),
    makeMat(2680.0, 0.5, 1.3, 1.80e10, 1.80e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 790.0, 1600.0, 293.0, 2.20e10,
            1.80e10, 3.50e9, 0.0, 1.0),
    makeMat(1000.0, 0.7, 0.15, 2.18e9, 1.325e10, 7.00e6, 4.19e5, 2.68e6, 10.0, 5.0, 4184.0, 273.15, 273.15, 3.50e9,
            2.18e9, 1.00e7, 0.0, 1.0),
    makeMat(0.178, 0.4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 8260.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2.08e5, 1.4),
    makeMat(2000.0, 0.5, 1.3, 1.20e10, 1.20e10, 1.60e7, 3.50e6, 1.80e7, 5.0, 5.0, 800.0, 1500.0, 293.0, 8.00e9,
            1.20e10, 5.00e7, 0.0, 1.0),
};

__device__ __forceinline__ int matIndex(uint8_t m) { return (m <= 4u) ? static_cast<int>(m) : 1; }

// FP64 constants of the engine's FP64 temperature and phase classification
// (eos.cu:229-266, 283-318, 320-350), formed as the engine forms them: PSU
// values by one division by the unit, 0.8 rho0 in kg/m^3 by one product.
// Each float threshold is the smallest float x for which the engine's FP64
// test on x passes, so the FP32 test of a float input decides exactly as the
// engine's FP64 test does.
struct MatConstD {
    double rho0, A, B, kH2, cv, tMelt;
    float ecvUp;        // smallest float u with (double)u >= E_cv (PSU)
    float rhoVapUp;     // smallest float rho with rho * 1e6 >= 0.8 rho0 [kg/m^3]
};
constexpr double cxUlpOfFloat(double f) {   // spacing of the floats in [2^e, 2^(e+1)) that holds f > 0
    double p = 1.0;
    while (p > f) p *= 0.5;
    while (p * 2.0 <= f) p *= 2.0;
    return p * (1.0 / 8388608.0);
}
constexpr float cxFloatNext(float f) { return static_cast<float>(static_cast<double>(f) + cxUlpOfFloat(f)); }
constexpr float cxFloatPrev(float f) {       // largest float below f > 0 (half the spacing below a power of two)
    const double u = cxUlpOfFloat(f);
    const bool pow2 = static_cast<double>(f) == u * 8388608.0;
    return static_cast<float>(static_cast<double>(f) - (pow2 ? 0.5 * u : u));
}
constexpr float cxFloatUp(double x) {       // smallest float >= x, x > 0 normal
    const float f = static_cast<float>(x);   // the nearest float: the next one up is >= x
    return (static_cast<double>(f) < x) ? cxFloatNext(f) : f;
}
constexpr float cxRhoUp(double kgPerM3) {   // smallest float rho with rho * 1e6 >= kgPerM3 (exact product)
    float f = cxFloatUp(kgPerM3 / 1.0e6);
    while (static_cast<double>(f) * 1.0e6 < kgPerM3) f = cxFloatNext(f);
    while (static_cast<double>(cxFloatPrev(f)) * 1.0e6 >= kgPerM3) f = cxFloatPrev(f);
    return f;
}
constexpr MatConstD makeMatD(double rho0Kg, double APa, double BPa, double Ecv, double cvSI, double tMelt, double kH2) {
    return MatConstD{rho0Kg / 1.0e6, APa / 1.0e12, BPa / 1.0e12, kH2, cvSI / 1.0e6, tMelt,
                     Ecv > 0.0 ? cxFloatUp(Ecv / 1.0e6) : 0.0f, rho0Kg > 0.0 ? cxRhoUp(0.8 * rho0Kg) : 0.0f};
}
static __constant__ MatConstD c_matD[5] = {
    makeMatD(7800.0, 1.28e11, 1.05e11, 8.67e6, 449.0, 1811.0, 0.0),     // Iron
    makeMatD(2680.0, 1.80e10, 1.80e10, 1.80e7, 790.0, 1600.0, 0.0),     // Granite
    makeMatD(1000.0, 2.18e9, 1.325e10, 2.68e6, 4184.0, 273.15, 0.0),    // WaterIce
    makeMatD(0.178, 0.0, 0.0, 0.0, 8260.0, 0.0, 2.08e5),                // HydrogenHelium
    makeMatD(2000.0, 1.20e10, 1.20e10, 1.80e7, 800.0, 1500.0, 0.0),     // Regolith
};
constexpr float kRhoWaterVapUp = cxRhoUp(322.0);   // eos.cu:247: rho [kg/m^3] < 322

// computeColdEnergyPsu (eos.cu:283-318) in FP64, in the engine's operation order.
__device__ __forceinline__ double coldEnergyF64(int mat, double rho) {
    const MatConstD& c = c_matD[mat];
    rho = rho > 0.0 ? rho : 0.0;
    if (mat == 3) return c.kH2 * rho;
    const double eta = rho / c.rho0;
    if (eta <= 1.0) return 0.0;
    const double mu = eta - 1.0;
    double ta, tb;
    if (mu < 1.0e-5) {
        const double m2 = mu * mu, m3 = m2 * mu, m4 = m3 * mu, m5 = m4 * mu;
        ta = 0.5 * m2 - (2.0 / 3.0) * m3 + 0.75 * m4 - 0.8 * m5;
        tb = (1.0 / 3.0) * m3 - 0.5 * m4 + 0.6 * m5;
    } else {
        const double le = log1p(mu);
        ta = le - (mu / eta);
        tb = (mu * (2.0 + mu)) / eta - 2.0 * le;
    }
    return (c.A * ta + c.B * tb) / c.rho0;
}

// The engine's FP64 temperature (eos.cu:320-330, 342).
static __device__ __noinline__ double temperatureF64(int mi, float rhoIn, float uIn) {
    const MatConstD& c = c_matD[mi];
    const double rho = fmax(static_cast<double>(rhoIn), 1.0e-12);
    const double u = static_cast<double>(uIn);
    const double uCold = coldEnergyF64(mi, rho);
    if (mi == 3) return fmax(3.0, fmax(0.0, u - uCold) / c.cv);
    return fmax(3.0, (u - uCold) / c.cv);
}

// ---------------------------------------------------------------- EOS -----
// FP32 evaluation of engine/eos.cu:283-388.  The reference evaluates in FP64;
// here every cancellation-prone quantity is formed without loss:
//   mu = ((rho - rho0_hi) - rho0_lo)/rho0 with rho0 = rho0_hi + rho0_lo the
//     FP64 reference density split into two floats (the difference is exact
//     when rho is within 2x of rho0, and the float rounding of rho0 itself,
//     ~3e-8 relative, does not leak into mu),
//   cold energy by its Taylor series for mu < 0.1,
//   the thermal excess u - cv T_ref with cv T_ref split into a float pair.
struct EosOut { float P, cs, T; uint8_t phase; };

__device__ __forceinline__ float coldEnergyF32(int mi, float rho) {
    const MatConst& c = c_mat[mi];
    rho = fmaxf(rho, 0.0f);
    if (mi == 3) return c.kH2 * rho;
    const float mu = ((rho - c.rho0) - c.rho0Lo) / c.rho0;
    if (!(mu > 0.0f)) return 0.0f;
    float ta, tb;
    if (mu < 0.1f) {
        // termA = sum_{k>=2} (-1)^k (k-1)/k mu^k ; termB = sum_{k>=3} (-1)^(k+1) (k-2)/k mu^k
        float sa = 0.0f, sb = 0.0f;
#pragma unroll
        for (int k = 16; k >= 2; --k) {
            const float ca = ((k & 1) ? -1.0f : 1.0f) * static_cast<float>(k - 1) / static_cast<float>(k);
            const float cb = (k >= 3) ? (((k & 1) ? 1.0f : -1.0f) * static_cast<float>(k - 2) / static_cast<float>(k)) : 0.0f;
            sa = sa * mu + ca;
            sb = sb * mu + cb;
        }
        ta = sa * mu * mu;
        tb = sb * mu * mu;
    } else {
        const float eta = 1.0f + mu;
        const float le = log1pf(mu);
        ta = le - (mu / eta);
        tb = (mu * (2.0f + mu)) / eta - 2.0f * le;
    }
    return (c.A * ta + c.B * tb) / c.rho0;
}

struct PD { float p, dpr, dpu; bool tension; };

__device__ __forceinline__ PD tillotsonCompressedF32(const MatConst& c, float rho, float eta, float mu, float uE,
                                                     float dmg) {
    const float bEff = (mu >= 0.0f) ? c.B : 0.0f;
    const float den = c.E0 * eta * eta;
    const float ratio = (den > 1.0e-30f) ? (uE / den) : 1.0e30f;
    const float iw = 1.0f / (ratio + 1.0f);
    const float wm1w2 = (ratio > 1.0e15f) ? 0.0f : (ratio * iw * iw);
    PD r;
    r.p = (c.a + c.b * iw) * rho * uE + c.A * mu + bEff * mu * mu;
    r.dpr = (c.a + c.b * iw) * uE + 2.0f * c.b * uE * wm1w2 + (c.A + 2.0f * bEff * mu) / c.rho0;
    r.dpu = (c.a + c.b * iw * iw) * rho;
    r.tension = false;
    if (r.p < 0.0f && dmg > 0.0f) {
        const float keep = 1.0f - dmg;
        r.p *= keep; r.dpr *= keep; r.dpu *= keep;
        r.tension = true;
    }
    return r;
}

__device__ __forceinline__ PD tillotsonExpandedF32(const MatConst& c, float rho, float eta, float mu, float uE) {
    const float x = -mu / eta;                     // 1/eta - 1, formed without cancellation
    const float ax2 = c.alpha * x * x;
    const float bx = c.beta * x;
    const float eA = (ax2 < 700.0f) ? expf(-ax2) : 0.0f;
    PD r;
    r.tension = false;
    if (eA == 0.0f) {
        r.p = c.a * rho * uE; r.dpr = c.a * uE; r.dpu = c.a * rho;
        return r;
    }
    const float eB = (bx < 700.0f) ? expf(-bx) : 0.0f;
    const float den = c.E0 * eta * eta;
    const float ratio = (den > 1.0e-30f) ? (uE / den) : 1.0e30f;
    const float iw = 1.0f / (ratio + 1.0f);
    const float wm1w2 = (ratio > 1.0e15f) ? 0.0f : (ratio * iw * iw);
    const float ideal = c.a * rho * uE;
    const float inner = (c.b * rho * uE * iw) + c.A * mu * eB;
    const float pe = ideal + inner * eA;
    const float r0r2 = c.rho0 / (rho * rho);
    const float expDrho = (eB > 0.0f) ? ((c.A / c.rho0 + c.A * mu * c.beta * r0r2) * eB) : 0.0f;
    r.p = pe;
    r.dpr = c.a * uE + eA * (c.b * uE * iw + 2.0f * c.b * uE * wm1w2 + expDrho) + 2.0f * c.alpha * x * r0r2 * (pe - ideal);
    r.dpu = (c.a + c.b * eA * iw * iw) * rho;
    return r;
}

// classifyPhase (eos.cu:229-266) on the engine's FP64 temperature T: the
// density and energy tests compare the float inputs with exact float
// thresholds (c_matD), the temperature tests are FP64.
__device__ __forceinline__ uint8_t classifyPhaseExact(int mi, float rho, float u, double T) {
    if (mi == 3) return (T > 10000.0) ? 3u : 5u;                  // eos.cu:235-238
    const MatConstD& d = c_matD[mi];
    if (mi == 2) {                                               // eos.cu:243-254
        if (T > 15000.0) return 3u;
        if (u >= d.ecvUp || (T > 647.0 && rho < kRhoWaterVapUp)) return 2u;
        if (T >= 273.15) return 4u;
        return 0u;
    }
    if (T > 12000.0) return 3u;                                  // eos.cu:257-266
    if (u >= d.ecvUp && rho < d.rhoVapUp) return 2u;
    if (T >= d.tMelt) return 1u;
    return 0u;
}

// True when the FP32 temperature T (from u and an FP32 cold energy uCold)
// may lie on the other side of a phase threshold than the engine's FP64 one:
// within 1e-5 T plus 4e-6 (|u| + |uCold|) / c_v of a threshold of the
// material (the FP32 T is within about a tenth of that of the FP64 T).
__device__ __forceinline__ bool nearPhaseTemperature(int mi, float T, float u, float uCold, float cv) {
    const float tol = 1.0e-5f * T + 4.0e-6f * (fabsf(u) + fabsf(uCold)) / cv;
    if (mi == 3) return fabsf(T - 10000.0f) <= tol;
    if (mi == 2)
        return fabsf(T - 15000.0f) <= tol || fabsf(T - 647.0f) <= tol || fabsf(T - 273.15f) <= tol;
    return fabsf(T - 12000.0f) <= tol || fabsf(T - static_cast<float>(c_matD[mi].tMelt)) <= tol;
}

// Phase and stored temperature: far from every threshold the FP32 T decides
// as the FP64 one would; near one, the engine's FP64 T is formed and both
// the phase and the stored temperature (float(T)) are the engine's.
__device__ __forceinline__ void phaseAndTemperature(int mi, float rhoIn, float u, float uCold, float cv, EosOut& o) {
    double T = static_cast<double>(o.T);
    if (nearPhaseTemperature(mi, o.T, u, uCold, cv)) {
        T = temperatureF64(mi, rhoIn, u);
        o.T = static_cast<float>(T);
    }
    o.phase = classifyPhaseExact(mi, rhoIn < 1.0e-12f ? 1.0e-12f : rhoIn, u, T);
}

__device__ __forceinline__ EosOut evaluateEosF32(uint8_t matRaw, float rhoIn, float u, float dIn) {
    const int mi = matIndex(matRaw);
    const MatConst& c = c_mat[mi];
    const float rho = fmaxf(rhoIn, 1.0e-12f);
    const float dmg = fminf(fmaxf(dIn, 0.0f), 1.0f);
    EosOut o;
    if (mi == 3) {                                               // eos.cu:328-340
        const float uTh = fmaxf(0.0f, u - c.kH2 * rho);
        const float T = fmaxf(3.0f, uTh / c.cv);
        const float P = c.kH2 * rho * rho + (c.gamma - 1.0f) * rho * uTh;
        const float cs2 = 2.0f * c.kH2 * rho + c.gamma * (c.gamma - 1.0f) * uTh;
        o.P = P; o.cs = fmaxf(0.05f, sqrtf(fmaxf(0.0f, cs2))); o.T = T;
        phaseAndTemperature(mi, rhoIn, u, c.kH2 * rho, c.cv, o);
        return o;
    }
    const float mu = ((rho - c.rho0) - c.rho0Lo) / c.rho0;   // additive uses
    const float eta = rho / c.rho0;                           // multiplicative uses
    const float uCold = coldEnergyF32(mi, rho);
    const float T = fmaxf(3.0f, (u - uCold) / c.cv);
    const float excess = ((u - c.cvTrefHi) - c.cvTrefLo) - uCold;
    const float uE = uCold + fmaxf(0.0f, excess);
    PD r;
    if (mu >= 0.0f || uE < c.Eiv) {
        r = tillotsonCompressedF32(c, rho, eta, mu, uE, dmg);
    } else if (uE >= c.Ecv) {
        r = tillotsonExpandedF32(c, rho, eta, mu, uE);
    } else {
        const PD pc = tillotsonCompressedF32(c, rho, eta, mu, uE, dmg);
        const PD pe = tillotsonExpandedF32(c, rho, eta, mu, uE);
        const float den = fmaxf(1.0e-30f, c.Ecv - c.Eiv);
        const float f = fminf(fmaxf((uE - c.Eiv) / den, 0.0f), 1.0f);
        r.p = (1.0f - f) * pc.p + f * pe.p;
        r.dpr = (1.0f - f) * pc.dpr + f * pe.dpr;
        r.dpu = (1.0f - f) * pc.dpu + f * pe.dpu + (pe.p - pc.p) / den;
        r.tension = pc.tension;
    }
    const float cs2 = r.dpr + (r.p / (rho * rho)) * r.dpu;
    const bool condensed = (mu >= 0.0f) || (uE < c.Eiv && rho >= 0.9f * c.rho0 && !r.tension);
    const float cMin = condensed ? c.cMinCondensed : 0.05f;
    o.P = r.p;
    o.cs = fmaxf(cMin, sqrtf(fmaxf(0.0f, cs2)));
    o.T = T;
    phaseAndTemperature(mi, rhoIn, u, uCold, c.cv, o);
    return o;
}

constexpr int kRec2Width = 6;   // float4 per pass-2 record

// Two float4 of one particle in one 32-byte aligned record, read whole by
// ldg256 in the SPH pair loops.
struct __align__(32) Rec32 {
    float4 a, b;
};

// ----------------------------------------------------------- workspace ---
// Device pointers of the library-owned scratch of one BVH (see capi.cu).
struct Work {
    uint32_t capacity;
    uint32_t maxNbr;
    Rec32* leaf;           // sorted order: a {x, y, z, Hs}, b {vx, vy, vz, m / max(rho, 1e-9)} (permutation / leaf refresh)
    float4* leafAux;
    float4* rec2;          // kRec2Width float4 per particle: the pass-2 record
    float4* node;          // 4 x float4 per internal node
    uint2* nodeRange;      // [N-1] {first, last}: the sorted leaf range of each internal node
    float4* leafScan;      // [4N] per leaf: block prefix and block suffix {min xyz, max 2h}, {max xyz, max Hs}
    long long* momScan;    // [10N] per leaf: inclusive block prefix of m, m x (3), m x x^T (6), fixed point
    float4* blockTable;    // [2 levels nb] sparse table of block extremes (level 0: the blocks)
    long long* blockMom;   // [10 nb] block totals, then exclusive block offsets
    float4* nodeQuad;      // 2 x float4 per internal node: central second moments
                           // {Sxx, Syy, Szz, Sxy}, {Sxz, Syz, 0, 0} (far-field mode 1)
    float4* driftPos;      // {x, y, z, 0} after the drift
    Rec32* drift;          // for the next drift: a {x, y, z, H = 2 max(h, 1e-6)} (pass 1 / leaf refresh),
                           // b {vx, vy, vz, rho} (opening kick / leaf refresh)
    float2* driftAux;      // {m, 21 / (2 pi H^3)} (the Wendland norm of H)
    uint32_t* nbrCount;
    uint32_t* nbrList;     // group-interleaved: entry k of particle i at ((i/32) maxNbr + k) 32 + i%32
    uint32_t* words;       // small words, see WordIndex
    uint32_t* sortScratch; // histograms + look-back + tile counters
    size_t sortScratchWords;
    uint32_t sortMaxTiles;
    DevStatus* status;
    uint32_t* groupCounts; // null, or [groups]: each group's gravity interaction count (diagnostic)
    int32_t* traceList;    // null, or {count, entries...}: the nodes (>= 0) and leaves (~j) the group
    uint32_t traceGroup;   //   traceGroup accepts in the gravity walk, appended in walk order (diagnostic)
    uint32_t traceCap;
    const uint32_t* runIf; // null, or a device word: the gravity kernel returns at once while it is 0
    uint32_t leafBucket;   // far-field mode 3: opened nodes of at most this many particles are evaluated P-P
    float expandGamma2;    // far-field mode 3: gamma^2 of the group-expansion test
};

// Indices into Work::words.
enum WordIndex : int {
    kWBounds = 0,        // 6 ordered-uint bounds (min xyz, max xyz)
    kWLiving = 6,        // 2 living flags
    kWDtMin = 8,         // 2 dt-min bit words (step parity)
    kWDtState = 10,      // 2 float dt slots (step parity)
    kWGroupCounter = 12, // persistent-grid work counter (gravity)
    kWNbrCounter = 13,   // persistent-grid work counter (neighbour build)
    kWMassMax = 14,      // bits of the largest |mass| (set by the permutation, read by the refit)
    kWBoundsF = 16,      // 6 floats: decoded bounds
    kWCount = 32
};

}  // namespace astraea_gb300
