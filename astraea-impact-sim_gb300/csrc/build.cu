// build.cu -- scene bounds, SoA permutation + leaf records + Karras LBVH, and
// the bottom-up refit, for sm_103a.
//
// Restates engine/sph_gravity.cu:258-333 (AABB), 363-430 (permutation),
// 173-187 + 432-529 (leaf init + Karras 2012 radix tree) and 531-620
// (bottom-up refit).  GB300 layout choices:
//   * permutation, leaf records and the Karras internal-node build run in one
//     pass over the sorted index range (one launch instead of two);
//   * the tree walks read 64-byte AoS node records (common.cuh) instead of
//     eleven SoA arrays; the engine's SoA / packed node arrays are still
//     written when the caller's descriptor has them;
//   * node mass and centre of mass come from exact 64-bit fixed-point sums
//     (sum m, sum m x) over the node's leaf range, rounded to FP32 once
//     per node.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

// ------------------------------------------------------------- bounds ----
__global__ void initBoundsKernel(uint32_t* words) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const uint32_t hi = orderedFromFloat(1.0e30f), lo = orderedFromFloat(-1.0e30f);
        words[kWBounds + 0] = hi; words[kWBounds + 1] = hi; words[kWBounds + 2] = hi;
        words[kWBounds + 3] = lo; words[kWBounds + 4] = lo; words[kWBounds + 5] = lo;
        words[kWLiving + 0] = 0u; words[kWLiving + 1] = 0u; words[kWMassMax] = 0u;
    }
}

__global__ void __launch_bounds__(256) boundsKernel(const float* __restrict__ x, const float* __restrict__ y,
                                                    const float* __restrict__ z, uint32_t n, uint32_t* words) {
    float mn[3] = {1.0e30f, 1.0e30f, 1.0e30f}, mx[3] = {-1.0e30f, -1.0e30f, -1.0e30f};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float a = __ldg(&x[i]), b = __ldg(&y[i]), c = __ldg(&z[i]);
        mn[0] = fminf(mn[0], a); mx[0] = fmaxf(mx[0], a);
        mn[1] = fminf(mn[1], b); mx[1] = fmaxf(mx[1], b);
        mn[2] = fminf(mn[2], c); mx[2] = fmaxf(mx[2], c);
    }
    blockBoundsToWords(mn, mx, words);
}

// ------------------------------------- permutation + leaves + Karras ----
__device__ __forceinline__ int karrasDelta(const uint64_t* __restrict__ codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t ci = __ldg(&codes[i]), cj = __ldg(&codes[j]);
    if (ci != cj) return __clzll(static_cast<long long>(ci ^ cj));
    return 64 + __clz(static_cast<int>(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j)));
}

#define AG_LIVE_F32(X)                                                                                         \
    X(velX) X(velY) X(velZ) X(mass) X(h) X(h0) X(rho) X(u) X(sXX) X(sYY) X(sZZ) X(sXY) X(sXZ) X(sYZ) X(damage) \
        X(damageCbrt) X(epsFail) X(tracerRestRadiusPsu) X(tracerRestNormalX) X(tracerRestNormalY)            \
            X(tracerRestNormalZ)
#define AG_LIVE_OTHER(X) X(materialId) X(bodyId) X(originalId) X(tracerIndex) X(tracerIsOcean)
// Fields recomputed by the step before anything reads them (the fused step
// skips them; the stage-by-stage call moves them like the engine does).
#define AG_DEAD_F32(X)                                                                                          \
    X(velHalfX) X(velHalfY) X(velHalfZ) X(accX) X(accY) X(accZ) X(drhoDt) X(pressure) X(soundSpeed) X(duDt)    \
        X(tempK) X(radPowerW) X(dSXX) X(dSYY) X(dSZZ) X(dSXY) X(dSXZ) X(dSYZ) X(dDamageCbrtDt) X(divV) X(curlVX) \
            X(curlVY) X(curlVZ) X(shepardC) X(surfFactor) X(phiGrav)
#define AG_DEAD_OTHER(X) X(phaseId)

template <bool kAllFields>
__global__ void __launch_bounds__(256) permuteLeavesKarrasKernel(AstraeaParticles p, AstraeaParticles alt,
                                                                 AstraeaRadixBvh bvh, const float4* __restrict__ posSrc,
                                                                 Work w, uint32_t n, uint32_t* livingFlags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tracer = false, intact = false;
    uint32_t massBits = 0u;                         // |m| as bits: ordered like the values
    if (i < n) {
        // min(): keeps the gather in bounds even if a failed sort (look-back
        // timeout, flagged in the status word) left a non-permutation here.
        const uint32_t s = min(__ldg(&bvh.indicesSorted[i]), n - 1u);
        float x, y, z;
        if (posSrc != nullptr) {
            const float4 q = posSrc[s];
            x = q.x; y = q.y; z = q.z;
        } else {
            x = __ldg(&p.posX[s]); y = __ldg(&p.posY[s]); z = __ldg(&p.posZ[s]);
        }
        alt.posX[i] = x; alt.posY[i] = y; alt.posZ[i] = z;
#define AG_GATHER(f) alt.f[i] = __ldg(&p.f[s]);
        AG_LIVE_F32(AG_GATHER)
        AG_LIVE_OTHER(AG_GATHER)
        if (kAllFields) {
            AG_DEAD_F32(AG_GATHER)
            AG_DEAD_OTHER(AG_GATHER)
        }
#undef AG_GATHER
        const float m = __ldg(&p.mass[s]);
        massBits = __float_as_uint(fabsf(m));
        const float hRaw = __ldg(&p.h[s]);
        const float hI = fmaxf(hRaw, 1.0e-6f);
        const float h0I = fmaxf(__ldg(&p.h0[s]), 1.0e-6f);
        const float Href = 2.0f * hRaw;     // engine leaf nodeMaxH (sph_gravity.cu:446)
        const float Hs = 2.0f * fmaxf(1.09f * hI, 0.351f * h0I);
        w.leaf[i].a = make_float4(x, y, z, Hs);
        w.leafAux[i] = make_float4(Hs, 0.8f * h0I, Href, m);
        w.leaf[i].b = make_float4(__ldg(&p.velX[s]), __ldg(&p.velY[s]), __ldg(&p.velZ[s]),
                                  __fdividef(m, fmaxf(__ldg(&p.rho[s]), 1.0e-9f)));
        const uint32_t leaf = (n - 1u) + i;
        if (bvh.aabbMinX != nullptr) {
            bvh.aabbMinX[leaf] = x; bvh.aabbMinY[leaf] = y; bvh.aabbMinZ[leaf] = z;
            bvh.aabbMaxX[leaf] = x; bvh.aabbMaxY[leaf] = y; bvh.aabbMaxZ[leaf] = z;
            bvh.nodeMass[leaf] = m;
            bvh.comX[leaf] = x; bvh.comY[leaf] = y; bvh.comZ[leaf] = z;
            bvh.nodeMaxH[leaf] = Href;
        }
        if (bvh.nodeComMass != nullptr) {
            bvh.nodeComMass[leaf] = AstraeaFloat4{x, y, z, m};
            bvh.nodeMinExtent[leaf] = AstraeaFloat4{x, y, z, 0.0f};
            bvh.nodeMaxHPacked[leaf] = AstraeaFloat4{x, y, z, Href};
        }
        if (__ldg(&p.tracerIndex[s]) >= 0) {       // sph_gravity.cu:466-471
            tracer = true;
            intact = __ldg(&p.damage[s]) < 0.8f;
        }
        if (n == 1u) bvh.parent[0] = -1;
    }
    const unsigned anyTracer = __ballot_sync(0xffffffffu, tracer);
    const unsigned anyIntact = __ballot_sync(0xffffffffu, intact);
    const uint32_t warpMassBits = __reduce_max_sync(0xffffffffu, massBits);
    if ((threadIdx.x & 31) == 0) {
        if (anyTracer) atomicOr(&livingFlags[0], 1u);
        if (anyIntact) atomicOr(&livingFlags[1], 1u);
        // scale of the refit's sums; the word only grows, so a stale read costs one extra atomic at most
        if (warpMassBits > __ldcg(&w.words[kWMassMax])) atomicMax(&w.words[kWMassMax], warpMassBits);
    }
    if (i + 1u < n) {                               // internal node i (Karras 2012)
        const int ii = static_cast<int>(i);
        const int nn = static_cast<int>(n);
        const uint64_t* codes = bvh.mortonCodesSorted;
        const int d = (karrasDelta(codes, nn, ii, ii + 1) - karrasDelta(codes, nn, ii, ii - 1) >= 0) ? 1 : -1;
        const int dMin = karrasDelta(codes, nn, ii, ii - d);
        int lmax = 2;
        while (karrasDelta(codes, nn, ii, ii + lmax * d) > dMin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (karrasDelta(codes, nn, ii, ii + (l + t) * d) > dMin) l += t;
        const int j = ii + l * d;
        const int dNode = karrasDelta(codes, nn, ii, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (karrasDelta(codes, nn, ii, ii + (s + t) * d) > dNode) s += t;
        } while (t > 1);
        const int g = ii + s * d + ((d < 0) ? d : 0);
        const int first = min(ii, j), last = max(ii, j);
        w.nodeRange[ii] = make_uint2(static_cast<uint32_t>(first), static_cast<uint32_t>(last));
        bvh.leftChild[ii] = (first == g) ? ~g : g;
        bvh.rightChild[ii] = (last == g + 1) ? ~(g + 1) : (g + 1);
        bvh.parent[(first == g) ? (nn - 1 + g) : g] = ii;
        bvh.parent[(last == g + 1) ? (nn - 1 + g + 1) : (g + 1)] = ii;
        bvh.atomicVisited[ii] = 0u;
        if (ii == 0) bvh.parent[0] = -1;
    }
}

// Leaf records from the caller's current SoA (used before tree walks that are
// not preceded by this library's own permutation).
__global__ void __launch_bounds__(256) refreshLeavesKernel(AstraeaParticles p, Work w, uint32_t n, bool withVelRho) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hI = fmaxf(__ldg(&p.h[i]), 1.0e-6f);
    const float h0I = fmaxf(__ldg(&p.h0[i]), 1.0e-6f);
    const float m = __ldg(&p.mass[i]);
    const float Hs = 2.0f * fmaxf(1.09f * hI, 0.351f * h0I);
    w.leaf[i].a = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), Hs);
    w.leafAux[i] = make_float4(Hs, 0.8f * h0I, 2.0f * __ldg(&p.h[i]), m);
    const float H = 2.0f * hI;                                      // the drift's 2 max(h, 1e-6)
    w.drift[i].a = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), H);
    w.driftAux[i] = make_float2(__ldg(&p.mass[i]), wendlandNorm(H));
    if (withVelRho) {
        const float4 vr = make_float4(__ldg(&p.velX[i]), __ldg(&p.velY[i]), __ldg(&p.velZ[i]), __ldg(&p.rho[i]));
        w.leaf[i].b = make_float4(vr.x, vr.y, vr.z, __fdividef(m, fmaxf(vr.w, 1.0e-9f)));
        w.drift[i].b = vr;
    }
}

// ------------------------------------------------------------- refit ----
// Replaces bottomUpBvhMomentsKernel (engine/sph_gravity.cu:531-620).  Every
// internal node of a Karras tree covers a contiguous range [first, last] of
// sorted leaves (stored by the build), so a node's box, maxH and mass
// moments are reductions over that range and need no climb through the
// tree, no arrival counters and no fences:
//   1. per block of 256 leaves: prefix and suffix min/max of the box and h
//      values, inclusive prefix sums of the moments, the block's totals;
//      then every node whose range lies inside the block, from shared memory;
//   2. one block: exclusive scan of the block totals; a sparse table of
//      block extremes;
//   3. per node spanning blocks: box = suffix (first's block) + prefix
//      (last's block) + one table query over the blocks between; moments =
//      difference of two global prefix sums.
// Min/max are exact in any order, so boxes, dNode and maxH equal the
// engine's.  The moments are summed as 64-bit fixed-point integers: with
// |m| < 2^em (the largest mass, reduced by the permutation), |x| < 2^ex (the
// scene bounds) and n <= 2^lg, the unit of m x is 2^(em + ex + lg - 61), so
// no partial sum reaches 2^62.  Integer sums are exact in any order and a
// node's sum is the exact difference of two prefix sums (FP64 prefix sums
// lose a small node's digits to the cancellation), and they take the
// integer pipes instead of the FP64 pipe, which runs at 1/64 of the FP32
// rate on this GPU.  A leaf term m x is the exact product (24 x 24-bit
// integer mantissa product) rounded once to the unit, so each sum is at
// least as precise as an FP64 accumulation; the node COM is the quotient of
// two sums in FP32 with one correction step, the mass the sum rounded to
// float once.  kMoments (the quadrupole
// far field) forms its terms m, m x, m x_a x_b in FP64 and the central
// second moments S = sum m x x^T - M c c^T in FP64 from the exact sums.
constexpr int kRefitBlock = 256;
constexpr int kMomW = 10;     // m, mx, my, mz, mxx, myy, mzz, mxy, mxz, myz

__device__ __forceinline__ float pow2f(int e) {           // 2^e, e clamped to the normal range
    return __int_as_float((max(-126, min(127, e)) + 127) << 23);
}
__device__ __forceinline__ double pow2d(int e) {          // 2^e for |e| < 1000
    return __longlong_as_double(static_cast<long long>(e + 1023) << 52);
}
__device__ __forceinline__ int expAbove(float v) {        // least e with |v| < 2^e; -126 for 0 and subnormals
    const int b = static_cast<int>((__float_as_uint(v) >> 23) & 0xffu);
    return b == 0 ? -126 : b - 126;
}

// Units of one build's fixed-point sums; every thread derives the same
// values from the bounds and largest-mass words.
struct MomScale {
    int em, ex, lg;           // |m| < 2^em, |x| < 2^ex, n <= 2^lg
    float mIn, xIn;           // leaf term of m x: (m 2^(61 - lg - em)) (x 2^-ex)
};
__device__ __forceinline__ MomScale momScale(const Work& w, uint32_t n) {
    float X = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) X = fmaxf(X, fabsf(floatFromOrdered(__ldcg(&w.words[kWBounds + k]))));
    MomScale s;
    s.em = min(expAbove(__uint_as_float(__ldcg(&w.words[kWMassMax]))), 127);
    s.ex = min(expAbove(X), 127);
    s.lg = n > 1u ? 32 - __clz(static_cast<int>(n - 1u)) : 0;
    s.mIn = pow2f(61 - s.lg - s.em);
    s.xIn = pow2f(-s.ex);
    return s;
}

// a b rounded to the nearest integer (ties away from zero), exact before
// that rounding: the product of the two 24-bit significands is formed in a
// 64-bit integer.  |a b| < 2^62 by the choice of units.
__device__ __forceinline__ long long fixProd(float a, float b) {
    const uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
    const int ea = static_cast<int>((ua >> 23) & 0xffu), eb = static_cast<int>((ub >> 23) & 0xffu);
    const uint64_t ma = (ua & 0x7fffffu) | (ea != 0 ? 0x800000u : 0u);
    const uint64_t mb = (ub & 0x7fffffu) | (eb != 0 ? 0x800000u : 0u);
    const uint64_t P = ma * mb;                                    // < 2^48
    const int sh = max(ea, 1) + max(eb, 1) - 300;                  // a b = P 2^sh
    uint64_t q;
    if (sh >= 0) q = P << min(sh, 15);
    else if (sh > -60) q = (P + (1ull << (-sh - 1))) >> (-sh);
    else q = 0u;
    return ((ua ^ ub) >> 31) != 0u ? -static_cast<long long>(q) : static_cast<long long>(q);
}

template <bool kMoments>
__device__ __forceinline__ void leafTerms(const float4& pm, const MomScale& S, long long* v) {
    if constexpr (kMoments) {
        const double m = pm.w, x = pm.x, y = pm.y, z = pm.z;
        const double u0 = pow2d(61 - S.lg - S.em), u1 = pow2d(61 - S.lg - S.em - S.ex),
                     u2 = pow2d(61 - S.lg - S.em - 2 * S.ex);
        v[0] = __double2ll_rn(m * u0);
        v[1] = __double2ll_rn(m * x * u1);
        v[2] = __double2ll_rn(m * y * u1);
        v[3] = __double2ll_rn(m * z * u1);
        v[4] = __double2ll_rn(m * x * x * u2);
        v[5] = __double2ll_rn(m * y * y * u2);
        v[6] = __double2ll_rn(m * z * z * u2);
        v[7] = __double2ll_rn(m * x * y * u2);
        v[8] = __double2ll_rn(m * x * z * u2);
        v[9] = __double2ll_rn(m * y * z * u2);
    } else {
        const float ms = pm.w * S.mIn;                      // the scalings by 2^k are exact
        v[0] = __float2ll_rn(ms);
        v[1] = fixProd(ms, pm.x * S.xIn);
        v[2] = fixProd(ms, pm.y * S.xIn);
        v[3] = fixProd(ms, pm.z * S.xIn);
    }
}

// a / b with b = bh + bl (bh = RN(b), r = RN(1 / bh)): the quotient ah r
// and one correction step from the FMA residual (Markstein, IBM J. Res.
// Dev. 34 (1990)), a split into two floats the same way.
__device__ __forceinline__ float llQuot(long long a, float bh, float bl, float r) {
    const float ah = __ll2float_rn(a);
    const float al = __ll2float_rn(a - __float2ll_rz(ah));
    const float q0 = ah * r;
    float res = fmaf(-q0, bh, ah);
    res = fmaf(-q0, bl, res + al);
    return fmaf(res, r, q0);
}

struct Ext8 {                 // min x y z, max x y z, max 2h, max Hs
    float mnx, mny, mnz, mxx, mxy, mxz, h, hs;
};
__device__ __forceinline__ Ext8 extEmpty() {
    return Ext8{3.0e38f, 3.0e38f, 3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};
}
__device__ __forceinline__ Ext8 extJoin(const Ext8& a, const Ext8& b) {
    return Ext8{fminf(a.mnx, b.mnx), fminf(a.mny, b.mny), fminf(a.mnz, b.mnz), fmaxf(a.mxx, b.mxx),
                fmaxf(a.mxy, b.mxy), fmaxf(a.mxz, b.mxz), fmaxf(a.h, b.h), fmaxf(a.hs, b.hs)};
}
__device__ __forceinline__ void extStore(float4* dst, const Ext8& e) {
    dst[0] = make_float4(e.mnx, e.mny, e.mnz, e.h);
    dst[1] = make_float4(e.mxx, e.mxy, e.mxz, e.hs);
}
__device__ __forceinline__ Ext8 extLoad(const float4* src) {
    const float4 a = __ldcg(&src[0]), b = __ldcg(&src[1]);
    return Ext8{a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w};
}
__device__ __forceinline__ Ext8 extShfl(const Ext8& e, int delta, bool up) {
    Ext8 o;
    float* d = reinterpret_cast<float*>(&o);
    const float* s = reinterpret_cast<const float*>(&e);
#pragma unroll
    for (int k = 0; k < 8; ++k)
        d[k] = up ? __shfl_up_sync(0xffffffffu, s[k], delta) : __shfl_down_sync(0xffffffffu, s[k], delta);
    return o;
}

// Node records from a node's box, h extremes and fixed-point moment sums.
template <bool kMoments>
__device__ void writeNode(const AstraeaRadixBvh& bvh, const Work& w, int node, const Ext8& e, const long long* Q,
                          const MomScale& S) {
    const int lc = __ldg(&bvh.leftChild[node]), rc = __ldg(&bvh.rightChild[node]);
    float cx, cy, cz, mSum;
    double M[kMomW];
    if constexpr (kMoments) {
        const double u1 = pow2d(S.em + S.ex + S.lg - 61), u2 = pow2d(S.em + 2 * S.ex + S.lg - 61);
        M[0] = static_cast<double>(Q[0]) * pow2d(S.em + S.lg - 61);
#pragma unroll
        for (int k = 1; k < 4; ++k) M[k] = static_cast<double>(Q[k]) * u1;
#pragma unroll
        for (int k = 4; k < kMomW; ++k) M[k] = static_cast<double>(Q[k]) * u2;
        mSum = static_cast<float>(M[0]);
    } else {
        mSum = (__ll2float_rn(Q[0]) * pow2f(S.lg - 61)) * pow2f(S.em);
    }
    if (Q[0] > 0) {
        if constexpr (kMoments) {
            const double im = 1.0 / M[0];
            cx = static_cast<float>(M[1] * im);
            cy = static_cast<float>(M[2] * im);
            cz = static_cast<float>(M[3] * im);
        } else {                                   // c = (Q_x / Q_m) 2^ex
            const float bh = __ll2float_rn(Q[0]);
            const float bl = __ll2float_rn(Q[0] - __float2ll_rz(bh));
            const float r = __frcp_rn(bh), sc = pow2f(S.ex);
            cx = llQuot(Q[1], bh, bl, r) * sc;
            cy = llQuot(Q[2], bh, bl, r) * sc;
            cz = llQuot(Q[3], bh, bl, r) * sc;
        }
    } else {                                       // massless subtree: the box centre
        cx = 0.5f * (e.mnx + e.mxx);
        cy = 0.5f * (e.mny + e.mxy);
        cz = 0.5f * (e.mnz + e.mxz);
    }
    const float dNode = fmaxf(e.mxx - e.mnx, fmaxf(e.mxy - e.mny, e.mxz - e.mnz));
    float4* rec = w.node + 4 * static_cast<size_t>(node);
    __stcg(&rec[0], make_float4(cx, cy, cz, mSum));
    __stcg(&rec[1], make_float4(__fmul_rn(dNode, dNode), __int_as_float(lc), __int_as_float(rc), e.hs));
    __stcg(&rec[2], make_float4(e.mnx, e.mny, e.mnz, e.h));
    __stcg(&rec[3], make_float4(e.mxx, e.mxy, e.mxz, 0.0f));
    if constexpr (kMoments) {
        float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (Q[0] > 0) {
            const double c[3] = {M[1] / M[0], M[2] / M[0], M[3] / M[0]};
            s[0] = static_cast<float>(fmax(0.0, M[4] - M[0] * c[0] * c[0]));
            s[1] = static_cast<float>(fmax(0.0, M[5] - M[0] * c[1] * c[1]));
            s[2] = static_cast<float>(fmax(0.0, M[6] - M[0] * c[2] * c[2]));
            s[3] = static_cast<float>(M[7] - M[0] * c[0] * c[1]);
            s[4] = static_cast<float>(M[8] - M[0] * c[0] * c[2]);
            s[5] = static_cast<float>(M[9] - M[0] * c[1] * c[2]);
        }
        __stcg(&w.nodeQuad[2 * static_cast<size_t>(node)], make_float4(s[0], s[1], s[2], s[3]));
        __stcg(&w.nodeQuad[2 * static_cast<size_t>(node) + 1], make_float4(s[4], s[5], 0.0f, 0.0f));
    }
    if (bvh.aabbMinX != nullptr) {
        bvh.aabbMinX[node] = e.mnx; bvh.aabbMinY[node] = e.mny; bvh.aabbMinZ[node] = e.mnz;
        bvh.aabbMaxX[node] = e.mxx; bvh.aabbMaxY[node] = e.mxy; bvh.aabbMaxZ[node] = e.mxz;
        bvh.nodeMaxH[node] = e.h; bvh.nodeMass[node] = mSum;
        bvh.comX[node] = cx; bvh.comY[node] = cy; bvh.comZ[node] = cz;
    }
    if (bvh.nodeComMass != nullptr) {
        bvh.nodeComMass[node] = AstraeaFloat4{cx, cy, cz, mSum};
        bvh.nodeMinExtent[node] = AstraeaFloat4{e.mnx, e.mny, e.mnz, dNode};
        bvh.nodeMaxHPacked[node] = AstraeaFloat4{e.mxx, e.mxy, e.mxz, e.h};
    }
}

template <bool kMoments>
__global__ void __launch_bounds__(kRefitBlock) refitBlockKernel(AstraeaRadixBvh bvh, Work w, uint32_t n) {
    constexpr int kW = kMoments ? kMomW : 4;
    constexpr int kWarps = kRefitBlock / 32;
    __shared__ Ext8 wPre[kRefitBlock], wSuf[kRefitBlock];   // warp-inclusive prefix / suffix extremes
    __shared__ Ext8 warpAgg[kWarps];
    __shared__ Ext8 sLeaf[kRefitBlock];                     // each leaf's own extremes
    __shared__ long long sP[kW][kRefitBlock];               // inclusive block prefix of the moments
    __shared__ long long warpOff[kW][kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t b0 = blockIdx.x * kRefitBlock;
    const uint32_t i = b0 + static_cast<uint32_t>(t);
    const bool valid = i < n;
    const MomScale S = momScale(w, n);
    Ext8 e = extEmpty();
    long long v[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) v[k] = 0;
    if (valid) {
        const float4 pa = __ldg(&w.leaf[i].a);
        const float4 ax = __ldg(&w.leafAux[i]);
        const float4 pm = make_float4(pa.x, pa.y, pa.z, ax.w);
        e = Ext8{pm.x, pm.y, pm.z, pm.x, pm.y, pm.z, ax.z, ax.x};
        leafTerms<kMoments>(pm, S, v);
    }
    // warp-inclusive scans: prefix (up), suffix (down), moments (up)
    Ext8 pre = e, suf = e;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Ext8 u = extShfl(pre, d, true);
        if (lane >= d) pre = extJoin(pre, u);
        const Ext8 q = extShfl(suf, d, false);
        if (lane + d < 32) suf = extJoin(suf, q);
#pragma unroll
        for (int k = 0; k < kW; ++k) {
            const long long o = __shfl_up_sync(0xffffffffu, v[k], d);
            if (lane >= d) v[k] += o;
        }
    }
    sLeaf[t] = e;
    wPre[t] = pre;
    wSuf[t] = suf;
    if (lane == 31) {
        warpAgg[warp] = pre;
#pragma unroll
        for (int k = 0; k < kW; ++k) warpOff[k][warp] = v[k];
    }
    __syncthreads();
    if (t == 0) {                                   // exclusive offsets of the warps' moment sums
#pragma unroll
        for (int k = 0; k < kW; ++k) {
            long long run = 0;
            for (int q = 0; q < kWarps; ++q) {
                const long long x = warpOff[k][q];
                warpOff[k][q] = run;
                run += x;
            }
        }
    }
    __syncthreads();
    for (int q = 0; q < warp; ++q) pre = extJoin(pre, warpAgg[q]);
    for (int q = warp + 1; q < kWarps; ++q) suf = extJoin(suf, warpAgg[q]);
#pragma unroll
    for (int k = 0; k < kW; ++k) {
        v[k] += warpOff[k][warp];
        sP[k][t] = v[k];
    }
    if (valid) {
        float4* ls = w.leafScan + 4 * static_cast<size_t>(i);
        extStore(ls, pre);
        extStore(ls + 2, suf);
        long long* ms = w.momScan + static_cast<size_t>(kMomW) * i;
#pragma unroll
        for (int k = 0; k < kW; ++k) ms[k] = v[k];
    }
    if (t == kRefitBlock - 1) {                    // block totals (level 0 of the table)
        extStore(w.blockTable + 2 * static_cast<size_t>(blockIdx.x), pre);
#pragma unroll
        for (int k = 0; k < kW; ++k) w.blockMom[static_cast<size_t>(kMomW) * blockIdx.x + k] = v[k];
    }
    __syncthreads();
    // internal nodes whose range lies inside this block
    if (i + 1u < n) {
        const uint2 r = __ldg(&w.nodeRange[i]);
        if (r.x >= b0 && r.y < b0 + kRefitBlock && r.x <= r.y) {
            const int f = static_cast<int>(r.x - b0), l = static_cast<int>(r.y - b0);
            const int wf = f >> 5, wl = l >> 5;
            Ext8 a;
            if (wf != wl) {                         // suffix + prefix + whole warps between
                a = extJoin(wSuf[f], wPre[l]);
                for (int q = wf + 1; q < wl; ++q) a = extJoin(a, warpAgg[q]);
            } else if ((f & 31) == 0) {
                a = wPre[l];
            } else if ((l & 31) == 31) {
                a = wSuf[f];
            } else {                                // inside one warp, off both ends: <= 30 leaves
                a = extEmpty();
                for (int k = f; k <= l; ++k) a = extJoin(a, sLeaf[k]);
            }
            long long Q[kW];
#pragma unroll
            for (int k = 0; k < kW; ++k) Q[k] = sP[k][l] - (f > 0 ? sP[k][f - 1] : 0);
            writeNode<kMoments>(bvh, w, static_cast<int>(i), a, Q, S);
        }
    }
}

// Block offsets: exclusive scan of the block totals, in place; one block of
// 1024 threads over chunks of 1024 blocks (coalesced), the next chunk's
// loads in flight while the current one is scanned.
template <bool kMoments>
__global__ void __launch_bounds__(1024) refitScanKernel(Work w, uint32_t nb) {
    constexpr int kW = kMoments ? kMomW : 4;
    __shared__ long long warpSum[kW][32];
    __shared__ long long carry[kW];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    if (t < static_cast<uint32_t>(kW)) carry[t] = 0;
    long long cur[kW], nxt[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) cur[k] = t < nb ? __ldcg(&w.blockMom[static_cast<size_t>(kMomW) * t + k]) : 0;
    __syncthreads();
    for (uint32_t base = 0; base < nb; base += 1024u) {
        const uint32_t bn = base + 1024u + t;
#pragma unroll
        for (int k = 0; k < kW; ++k) nxt[k] = bn < nb ? __ldcg(&w.blockMom[static_cast<size_t>(kMomW) * bn + k]) : 0;
        long long inc[kW];
#pragma unroll
        for (int k = 0; k < kW; ++k) inc[k] = cur[k];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
#pragma unroll
            for (int k = 0; k < kW; ++k) {
                const long long o = __shfl_up_sync(0xffffffffu, inc[k], d);
                if (lane >= static_cast<uint32_t>(d)) inc[k] += o;
            }
        if (lane == 31u)
#pragma unroll
            for (int k = 0; k < kW; ++k) warpSum[k][warp] = inc[k];
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int k = 0; k < kW; ++k) {
                long long x = warpSum[k][lane];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const long long o = __shfl_up_sync(0xffffffffu, x, d);
                    if (lane >= static_cast<uint32_t>(d)) x += o;
                }
                warpSum[k][lane] = x;              // inclusive over warps
            }
        }
        __syncthreads();
        const uint32_t b = base + t;
        if (b < nb)
#pragma unroll
            for (int k = 0; k < kW; ++k)
                w.blockMom[static_cast<size_t>(kMomW) * b + k] =
                    carry[k] + (warp > 0 ? warpSum[k][warp - 1] : 0) + inc[k] - cur[k];
        __syncthreads();                           // carry and warpSum read by all
        if (t < static_cast<uint32_t>(kW)) carry[t] += warpSum[t][31];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kW; ++k) cur[k] = nxt[k];
    }
}

// Up to three levels of the sparse table of block extremes per launch
// (the levels are latency-bound, so the extra loads are cheap): with
// s = 2^(lev-1) and A_k = T[lev-1][b + k s], T[lev-1+j][b] joins
// A_0 .. A_(2^j - 1) (it covers blocks b .. b + 2^j s - 1), j = 1 .. count.
__global__ void __launch_bounds__(256) refitLevelKernel(Work w, uint32_t nb, uint32_t lev, uint32_t count) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = 1u << (lev - 1);
    if (b + 2u * s > nb) return;
    const float4* src = w.blockTable + 2 * static_cast<size_t>(lev - 1) * nb;
    Ext8 a[8];
#pragma unroll
    for (uint32_t k = 0; k < 8u; ++k)
        a[k] = (k < (2u << (count - 1)) && b + (k + 1u) * s <= nb) ? extLoad(src + 2 * (b + k * s)) : extEmpty();
    Ext8 acc = a[0];
#pragma unroll
    for (uint32_t j = 1; j <= 3u; ++j) {
        const uint32_t width = 1u << j;
        if (j > count || b + width * s > nb) break;
        for (uint32_t k = width >> 1; k < width; ++k) acc = extJoin(acc, a[k]);
        extStore(w.blockTable + 2 * (static_cast<size_t>(lev - 1 + j) * nb + b), acc);
    }
}

// Nodes whose range spans blocks.
template <bool kMoments>
__global__ void __launch_bounds__(256) refitCrossKernel(AstraeaRadixBvh bvh, Work w, uint32_t n, uint32_t nb) {
    constexpr int kW = kMoments ? kMomW : 4;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1u >= n) return;
    const uint2 r = __ldg(&w.nodeRange[i]);
    const uint32_t bf = r.x / kRefitBlock, bl = r.y / kRefitBlock;
    if (bf == bl || r.y >= n || r.x > r.y) return;
    Ext8 e = extJoin(extLoad(w.leafScan + 4 * static_cast<size_t>(r.x) + 2),   // suffix in first's block
                     extLoad(w.leafScan + 4 * static_cast<size_t>(r.y)));      // prefix in last's block
    if (bl > bf + 1u) {
        const uint32_t lo = bf + 1u, hi = bl - 1u, len = hi - lo + 1u;
        const uint32_t lev = 31u - static_cast<uint32_t>(__clz(len));
        const float4* tab = w.blockTable + 2 * static_cast<size_t>(lev) * nb;
        e = extJoin(e, extJoin(extLoad(tab + 2 * lo), extLoad(tab + 2 * (hi + 1u - (1u << lev)))));
    }
    long long Q[kW];
    const long long* ml = w.momScan + static_cast<size_t>(kMomW) * r.y;
    const long long* ol = w.blockMom + static_cast<size_t>(kMomW) * bl;
#pragma unroll
    for (int k = 0; k < kW; ++k) Q[k] = __ldcg(&ol[k]) + __ldcg(&ml[k]);
    if (r.x > 0u) {
        const uint32_t f1 = r.x - 1u;
        const long long* mf = w.momScan + static_cast<size_t>(kMomW) * f1;
        const long long* of = w.blockMom + static_cast<size_t>(kMomW) * (f1 / kRefitBlock);
#pragma unroll
        for (int k = 0; k < kW; ++k) Q[k] -= __ldcg(&of[k]) + __ldcg(&mf[k]);
    }
    writeNode<kMoments>(bvh, w, static_cast<int>(i), e, Q, momScale(w, n));
}

inline unsigned gridFor(uint32_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

cudaError_t launchInitBounds(uint32_t* words, cudaStream_t st) {
    initBoundsKernel<<<1, 32, 0, st>>>(words);
    return cudaGetLastError();
}

cudaError_t launchBounds(const AstraeaParticles& p, uint32_t n, uint32_t* words, int sms, cudaStream_t st) {
    const unsigned blocks = min(gridFor(n, 256), static_cast<unsigned>(sms * 4));
    boundsKernel<<<blocks, 256, 0, st>>>(p.posX, p.posY, p.posZ, n, words);
    return cudaGetLastError();
}

cudaError_t launchPermuteLeavesKarras(const AstraeaParticles& p, const AstraeaParticles& alt,
                                      const AstraeaRadixBvh& bvh, const float4* posSrc, const Work& w, uint32_t n,
                                      uint32_t* livingFlags, bool allFields, cudaStream_t st) {
    if (allFields)
        permuteLeavesKarrasKernel<true><<<gridFor(n, 256), 256, 0, st>>>(p, alt, bvh, posSrc, w, n, livingFlags);
    else
        permuteLeavesKarrasKernel<false><<<gridFor(n, 256), 256, 0, st>>>(p, alt, bvh, posSrc, w, n, livingFlags);
    return cudaGetLastError();
}

cudaError_t launchRefreshLeaves(const AstraeaParticles& p, const Work& w, uint32_t n, bool withVelRho,
                                cudaStream_t st) {
    refreshLeavesKernel<<<gridFor(n, 256), 256, 0, st>>>(p, w, n, withVelRho);
    return cudaGetLastError();
}

uint32_t refitBlocks(uint32_t n) { return (n + kRefitBlock - 1) / kRefitBlock; }
uint32_t refitLevels(uint32_t nb) {
    uint32_t lev = 1;
    while ((2u << (lev - 1)) <= nb) ++lev;      // levels 0 .. floor(log2 nb)
    return lev;
}

// Node masses and COMs rounded as the engine rounds them (node rounding 1):
// the engine's bottom-up FP32 combination (bottomUpBvhMomentsKernel,
// engine/sph_gravity.cu:531-621) -- m = m_L + m_R, c = (m_L c_L + m_R c_R)
// (1 / m) with the sum contracted as nvcc contracts it, fma(m_L, c_L, m_R c_R)
// (on the reference kernels' own build this gives their COMs bit for bit),
// c = (c_L + c_R) / 2 for a massless pair.  One thread per leaf climbs
// towards the root; the second child to arrive at a node combines it (the
// arrival counters were zeroed by the Karras kernel of this build).  Only
// the mass and COM of the node records and of the descriptor's arrays are
// replaced; boxes, h extremes and the quadrupole moments stay the refit's.
__global__ void __launch_bounds__(256) engineNodeMomentsKernel(AstraeaParticles p, AstraeaRadixBvh bvh, Work w,
                                                                uint32_t n) {
    const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n || n < 2u) return;
    auto childRec = [&](int c) {
        if (c < 0) {
            const uint32_t j = static_cast<uint32_t>(~c);
            return make_float4(p.posX[j], p.posY[j], p.posZ[j], p.mass[j]);
        }
        return __ldcg(&w.node[4 * static_cast<size_t>(c)]);
    };
    int pNode = __ldcg(&bvh.parent[n - 1u + leaf]);
    __threadfence();
    uint32_t climbs = 0;
    while (pNode >= 0 && pNode < static_cast<int>(n) - 1 && ++climbs < 4096u) {
        if (atomicAdd(&bvh.atomicVisited[pNode], 1u) == 0u) return;   // the sibling's thread combines
        const float4 L = childRec(__ldcg(&bvh.leftChild[pNode]));
        const float4 R = childRec(__ldcg(&bvh.rightChild[pNode]));
        const float m = __fadd_rn(L.w, R.w);
        float cx, cy, cz;
        if (m > 0.0f) {
            const float inv = __fdiv_rn(1.0f, m);
            cx = __fmul_rn(__fmaf_rn(L.w, L.x, __fmul_rn(R.w, R.x)), inv);
            cy = __fmul_rn(__fmaf_rn(L.w, L.y, __fmul_rn(R.w, R.y)), inv);
            cz = __fmul_rn(__fmaf_rn(L.w, L.z, __fmul_rn(R.w, R.z)), inv);
        } else {
            cx = __fmul_rn(0.5f, __fadd_rn(L.x, R.x));
            cy = __fmul_rn(0.5f, __fadd_rn(L.y, R.y));
            cz = __fmul_rn(0.5f, __fadd_rn(L.z, R.z));
        }
        __stcg(&w.node[4 * static_cast<size_t>(pNode)], make_float4(cx, cy, cz, m));
        if (bvh.aabbMinX != nullptr) {
            bvh.nodeMass[pNode] = m;
            bvh.comX[pNode] = cx; bvh.comY[pNode] = cy; bvh.comZ[pNode] = cz;
        }
        if (bvh.nodeComMass != nullptr) bvh.nodeComMass[pNode] = AstraeaFloat4{cx, cy, cz, m};
        __threadfence();
        pNode = __ldcg(&bvh.parent[pNode]);
    }
}

cudaError_t launchEngineNodeMoments(const AstraeaParticles& p, const AstraeaRadixBvh& bvh, const Work& w, uint32_t n,
                                    cudaStream_t st) {
    if (n < 2u) return cudaSuccess;
    engineNodeMomentsKernel<<<gridFor(n, 256), 256, 0, st>>>(p, bvh, w, n);
    return cudaGetLastError();
}

cudaError_t launchRefit(const AstraeaRadixBvh& bvh, const Work& w, uint32_t n, bool moments, cudaStream_t st) {
    if (n < 2u) return cudaSuccess;
    const uint32_t nb = refitBlocks(n);
    const uint32_t levels = refitLevels(nb);
    if (moments) {
        refitBlockKernel<true><<<nb, kRefitBlock, 0, st>>>(bvh, w, n);
        refitScanKernel<true><<<1, 1024, 0, st>>>(w, nb);
    } else {
        refitBlockKernel<false><<<nb, kRefitBlock, 0, st>>>(bvh, w, n);
        refitScanKernel<false><<<1, 1024, 0, st>>>(w, nb);
    }
    for (uint32_t lev = 1; lev < levels; lev += 3)
        refitLevelKernel<<<gridFor(nb, 256), 256, 0, st>>>(w, nb, lev, std::min(3u, levels - lev));
    if (moments)
        refitCrossKernel<true><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n, nb);
    else
        refitCrossKernel<false><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n, nb);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
