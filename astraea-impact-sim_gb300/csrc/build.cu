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
//   * node mass and centre of mass are accumulated as FP64 moments
//     (sum m, sum m x) and rounded to FP32 once per node.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

// ------------------------------------------------------------- bounds ----
__global__ void initBoundsKernel(uint32_t* words) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const uint32_t hi = orderedFromFloat(1.0e30f), lo = orderedFromFloat(-1.0e30f);
        words[kWBounds + 0] = hi; words[kWBounds + 1] = hi; words[kWBounds + 2] = hi;
        words[kWBounds + 3] = lo; words[kWBounds + 4] = lo; words[kWBounds + 5] = lo;
        words[kWLiving + 0] = 0u; words[kWLiving + 1] = 0u;
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
        const float hRaw = __ldg(&p.h[s]);
        const float hI = fmaxf(hRaw, 1.0e-6f);
        const float h0I = fmaxf(__ldg(&p.h0[s]), 1.0e-6f);
        const float Href = 2.0f * hRaw;     // engine leaf nodeMaxH (sph_gravity.cu:446)
        const float Hs = 2.0f * fmaxf(1.09f * hI, 0.351f * h0I);
        w.leaf[i].a = make_float4(x, y, z, m);
        w.leafAux[i] = make_float4(Hs, 0.8f * h0I, Href, 0.0f);
        w.leaf[i].b = make_float4(__ldg(&p.velX[s]), __ldg(&p.velY[s]), __ldg(&p.velZ[s]), __ldg(&p.rho[s]));
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
    if ((threadIdx.x & 31) == 0) {
        if (anyTracer) atomicOr(&livingFlags[0], 1u);
        if (anyIntact) atomicOr(&livingFlags[1], 1u);
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
    w.leaf[i].a = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), __ldg(&p.mass[i]));
    w.leafAux[i] = make_float4(2.0f * fmaxf(1.09f * hI, 0.351f * h0I), 0.8f * h0I, 2.0f * __ldg(&p.h[i]), 0.0f);
    const float H = 2.0f * hI;                                      // the drift's 2 max(h, 1e-6)
    w.drift[i].a = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), H);
    w.driftAux[i] = make_float2(__ldg(&p.mass[i]), wendlandNorm(H));
    if (withVelRho) {
        const float4 vr = make_float4(__ldg(&p.velX[i]), __ldg(&p.velY[i]), __ldg(&p.velZ[i]), __ldg(&p.rho[i]));
        w.leaf[i].b = vr;
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
//      values, inclusive FP64 prefix sums of the moments, the block's
//      totals; then every node whose range lies inside the block, from
//      shared memory;
//   2. one block: exclusive FP64 scan of the block totals and a sparse table
//      of block extremes;
//   3. per node spanning blocks: box = suffix (first's block) + prefix
//      (last's block) + one table query over the blocks between; moments =
//      difference of two global prefix sums.
// Min/max are exact in any order, so boxes, dNode and maxH equal the
// engine's; COM and mass come from FP64 sums (as before, rounded to float
// once).  kMoments adds the central second moments S = sum m x x^T - M c c^T
// from FP64 sums of m x_a x_b.
constexpr int kRefitBlock = 256;
constexpr int kMomW = 10;     // m, mx, my, mz, mxx, myy, mzz, mxy, mxz, myz

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

// Node records from a node's box, h extremes and FP64 moments.
template <bool kMoments>
__device__ void writeNode(const AstraeaRadixBvh& bvh, const Work& w, int node, const Ext8& e, const double* M) {
    const int lc = __ldg(&bvh.leftChild[node]), rc = __ldg(&bvh.rightChild[node]);
    float cx, cy, cz;
    if (M[0] > 0.0) {
        const double im = 1.0 / M[0];
        cx = static_cast<float>(M[1] * im);
        cy = static_cast<float>(M[2] * im);
        cz = static_cast<float>(M[3] * im);
    } else {                                       // massless subtree: the box centre
        cx = 0.5f * (e.mnx + e.mxx);
        cy = 0.5f * (e.mny + e.mxy);
        cz = 0.5f * (e.mnz + e.mxz);
    }
    const float mSum = static_cast<float>(M[0]);
    const float dNode = fmaxf(e.mxx - e.mnx, fmaxf(e.mxy - e.mny, e.mxz - e.mnz));
    float4* rec = w.node + 4 * static_cast<size_t>(node);
    __stcg(&rec[0], make_float4(cx, cy, cz, mSum));
    __stcg(&rec[1], make_float4(__fmul_rn(dNode, dNode), __int_as_float(lc), __int_as_float(rc), e.hs));
    __stcg(&rec[2], make_float4(e.mnx, e.mny, e.mnz, e.h));
    __stcg(&rec[3], make_float4(e.mxx, e.mxy, e.mxz, 0.0f));
    if (kMoments) {
        float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (M[0] > 0.0) {
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
    __shared__ double sP[kW][kRefitBlock];                  // inclusive block prefix of the moments
    __shared__ double warpOff[kW][kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t b0 = blockIdx.x * kRefitBlock;
    const uint32_t i = b0 + static_cast<uint32_t>(t);
    const bool valid = i < n;
    Ext8 e = extEmpty();
    double v[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) v[k] = 0.0;
    if (valid) {
        const float4 pm = __ldg(&w.leaf[i].a);
        const float4 ax = __ldg(&w.leafAux[i]);
        e = Ext8{pm.x, pm.y, pm.z, pm.x, pm.y, pm.z, ax.z, ax.x};
        const double m = pm.w, x = pm.x, y = pm.y, z = pm.z;
        v[0] = m; v[1] = m * x; v[2] = m * y; v[3] = m * z;
        if constexpr (kMoments) {
            v[4] = m * x * x; v[5] = m * y * y; v[6] = m * z * z;
            v[7] = m * x * y; v[8] = m * x * z; v[9] = m * y * z;
        }
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
            const double o = __shfl_up_sync(0xffffffffu, v[k], d);
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
            double run = 0.0;
            for (int q = 0; q < kWarps; ++q) {
                const double x = warpOff[k][q];
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
        double* ms = w.momScan + static_cast<size_t>(kMomW) * i;
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
            double M[kMomW];
#pragma unroll
            for (int k = 0; k < kW; ++k) M[k] = sP[k][l] - (f > 0 ? sP[k][f - 1] : 0.0);
#pragma unroll
            for (int k = kW; k < kMomW; ++k) M[k] = 0.0;
            writeNode<kMoments>(bvh, w, static_cast<int>(i), a, M);
        }
    }
}

// Block offsets: exclusive FP64 scan of the block totals, in place; one
// block of 1024 threads.
template <bool kMoments>
__global__ void __launch_bounds__(1024) refitScanKernel(Work w, uint32_t nb) {
    constexpr int kW = kMoments ? kMomW : 4;
    __shared__ double warpSum[kW][32];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint32_t per = (nb + 1023u) / 1024u;
    const uint32_t lo = min(nb, t * per), hi = min(nb, lo + per);
    double acc[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) acc[k] = 0.0;
    for (uint32_t b = lo; b < hi; ++b)
#pragma unroll
        for (int k = 0; k < kW; ++k) acc[k] += w.blockMom[static_cast<size_t>(kMomW) * b + k];
    double inc[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) inc[k] = acc[k];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
#pragma unroll
        for (int k = 0; k < kW; ++k) {
            const double o = __shfl_up_sync(0xffffffffu, inc[k], d);
            if (lane >= static_cast<uint32_t>(d)) inc[k] += o;
        }
    if (lane == 31u)
#pragma unroll
        for (int k = 0; k < kW; ++k) warpSum[k][warp] = inc[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < kW; ++k) {
            double x = warpSum[k][lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const double o = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= static_cast<uint32_t>(d)) x += o;
            }
            warpSum[k][lane] = x;                  // inclusive over warps
        }
    }
    __syncthreads();
    double run[kW];
#pragma unroll
    for (int k = 0; k < kW; ++k) run[k] = inc[k] - acc[k] + (warp > 0 ? warpSum[k][warp - 1] : 0.0);
    for (uint32_t b = lo; b < hi; ++b)
#pragma unroll
        for (int k = 0; k < kW; ++k) {
            double* slot = &w.blockMom[static_cast<size_t>(kMomW) * b + k];
            const double x = *slot;
            *slot = run[k];
            run[k] += x;
        }
}

// One level of the sparse table of block extremes: T[lev][b] = T[lev-1][b]
// joined with T[lev-1][b + 2^(lev-1)].
__global__ void __launch_bounds__(256) refitLevelKernel(Work w, uint32_t nb, uint32_t lev) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t span = 1u << (lev - 1);
    if (b + 2u * span > nb) return;
    const float4* src = w.blockTable + 2 * static_cast<size_t>(lev - 1) * nb;
    extStore(w.blockTable + 2 * (static_cast<size_t>(lev) * nb + b),
             extJoin(extLoad(src + 2 * b), extLoad(src + 2 * (b + span))));
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
    double M[kMomW];
    const double* ml = w.momScan + static_cast<size_t>(kMomW) * r.y;
    const double* ol = w.blockMom + static_cast<size_t>(kMomW) * bl;
#pragma unroll
    for (int k = 0; k < kW; ++k) M[k] = __ldcg(&ol[k]) + __ldcg(&ml[k]);
    if (r.x > 0u) {
        const uint32_t f1 = r.x - 1u;
        const double* mf = w.momScan + static_cast<size_t>(kMomW) * f1;
        const double* of = w.blockMom + static_cast<size_t>(kMomW) * (f1 / kRefitBlock);
#pragma unroll
        for (int k = 0; k < kW; ++k) M[k] -= __ldcg(&of[k]) + __ldcg(&mf[k]);
    }
#pragma unroll
    for (int k = kW; k < kMomW; ++k) M[k] = 0.0;
    writeNode<kMoments>(bvh, w, static_cast<int>(i), e, M);
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
    for (uint32_t lev = 1; lev < levels; ++lev)
        refitLevelKernel<<<gridFor(nb, 256), 256, 0, st>>>(w, nb, lev);
    if (moments)
        refitCrossKernel<true><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n, nb);
    else
        refitCrossKernel<false><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n, nb);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
