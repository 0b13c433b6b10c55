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
        w.leafPM[i] = make_float4(x, y, z, m);
        w.leafAux[i] = make_float4(Hs, 0.8f * h0I, Href, 0.0f);
        w.velRho[i] = make_float4(__ldg(&p.velX[s]), __ldg(&p.velY[s]), __ldg(&p.velZ[s]), __ldg(&p.rho[s]));
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
    w.leafPM[i] = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), __ldg(&p.mass[i]));
    w.leafAux[i] = make_float4(2.0f * fmaxf(1.09f * hI, 0.351f * h0I), 0.8f * h0I, 2.0f * __ldg(&p.h[i]), 0.0f);
    const float H = 2.0f * hI;                                      // the drift's 2 max(h, 1e-6)
    w.driftRec[i] = make_float4(__ldg(&p.posX[i]), __ldg(&p.posY[i]), __ldg(&p.posZ[i]), H);
    w.driftAux[i] = make_float2(__ldg(&p.mass[i]), wendlandNorm(H));
    if (withVelRho)
        w.velRho[i] = make_float4(__ldg(&p.velX[i]), __ldg(&p.velY[i]), __ldg(&p.velZ[i]), __ldg(&p.rho[i]));
}

// ------------------------------------------------------------- refit ----
struct ChildData {
    float mnx, mny, mnz, mxx, mxy, mxz, maxH, maxHs;
    NodeMom mom;
    float cx, cy, cz;
    float s[6];            // central second moments xx yy zz xy xz yz (moments refit only)
};

template <bool kMoments>
__device__ __forceinline__ ChildData loadChild(const Work& w, int c, int n) {
    ChildData d;
#pragma unroll
    for (int k = 0; k < 6; ++k) d.s[k] = 0.0f;
    if (c < 0) {
        const int leaf = ~c;
        const float4 pm = __ldg(&w.leafPM[leaf]);
        const float4 ax = __ldg(&w.leafAux[leaf]);
        d.mnx = d.mxx = d.cx = pm.x;
        d.mny = d.mxy = d.cy = pm.y;
        d.mnz = d.mxz = d.cz = pm.z;
        d.maxH = ax.z;
        d.maxHs = ax.x;
        const double m = pm.w;
        d.mom = NodeMom{m * static_cast<double>(pm.x), m * static_cast<double>(pm.y), m * static_cast<double>(pm.z), m};
    } else {
        const float4* rec = w.node + 4 * static_cast<size_t>(c);
        const float4 r0 = __ldcg(&rec[0]);
        const float4 r1 = __ldcg(&rec[1]);
        const float4 r2 = __ldcg(&rec[2]);
        const float4 r3 = __ldcg(&rec[3]);
        d.cx = r0.x; d.cy = r0.y; d.cz = r0.z;
        d.maxHs = r1.w;
        d.mnx = r2.x; d.mny = r2.y; d.mnz = r2.z; d.maxH = r2.w;
        d.mxx = r3.x; d.mxy = r3.y; d.mxz = r3.z;
        const double2* mp = reinterpret_cast<const double2*>(w.nodeMom + c);
        const double2 a = __ldcg(&mp[0]);
        const double2 b = __ldcg(&mp[1]);
        d.mom = NodeMom{a.x, a.y, b.x, b.y};
        if (kMoments) {
            const float4 q0 = __ldcg(&w.nodeQuad[2 * static_cast<size_t>(c)]);
            const float4 q1 = __ldcg(&w.nodeQuad[2 * static_cast<size_t>(c) + 1]);
            d.s[0] = q0.x; d.s[1] = q0.y; d.s[2] = q0.z; d.s[3] = q0.w; d.s[4] = q1.x; d.s[5] = q1.y;
        }
    }
    (void)n;
    return d;
}

// kMoments: also the central second moments S = sum m (x - c)(x - c)^T of
// every node, combined with the parallel-axis rule
//   S = S_L + S_R + m_L d_L d_L^T + m_R d_R d_R^T,   d = c_child - c,
// in FP32 (no cancellation: every term is non-negative or a small offset).
template <bool kMoments>
__global__ void __launch_bounds__(256) refitKernel(AstraeaRadixBvh bvh, Work w, uint32_t n) {
    const uint32_t leafIdx = blockIdx.x * blockDim.x + threadIdx.x;
    if (leafIdx >= n || n < 2u) return;
    // The data of the node this thread just finished stays in registers; at
    // each level only the sibling is loaded (the engine reloads both children).
    int curr = ~static_cast<int>(leafIdx);          // child reference of the leaf
    ChildData mine = loadChild<kMoments>(w, curr, static_cast<int>(n));
    int pNode = __ldcg(&bvh.parent[(n - 1u) + leafIdx]);
    // A radix tree over 63-bit keys + 32-bit index ties is at most 96 deep;
    // the bound only matters for a tree built from a failed sort.
    for (int level = 0; pNode >= 0; ++level) {
        if (level >= 256 || pNode >= static_cast<int>(n) - 1) {
            atomicOr(&w.status->flags, kFlagStackOverflow);
            return;
        }
        // loads that do not depend on the arrival order, issued before the atomic
        const int lc = __ldcg(&bvh.leftChild[pNode]);
        const int rc = __ldcg(&bvh.rightChild[pNode]);
        const int grand = __ldcg(&bvh.parent[pNode]);
        // Arrival counter with release (this thread's node records, written
        // with st.cg, become visible to the second arrival) and acquire (the
        // sibling's records are read after it) in one atomic, instead of two
        // full fences.
        uint32_t before;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;"
                     : "=r"(before)
                     : "l"(&bvh.atomicVisited[pNode])
                     : "memory");
        if (before == 0u) return;   // first arrival stops
        const bool fromLeft = (lc == curr);
        const ChildData other = loadChild<kMoments>(w, fromLeft ? rc : lc, static_cast<int>(n));
        const ChildData& L = fromLeft ? mine : other;
        const ChildData& R = fromLeft ? other : mine;
        ChildData out;
        out.mnx = fminf(L.mnx, R.mnx); out.mny = fminf(L.mny, R.mny); out.mnz = fminf(L.mnz, R.mnz);
        out.mxx = fmaxf(L.mxx, R.mxx); out.mxy = fmaxf(L.mxy, R.mxy); out.mxz = fmaxf(L.mxz, R.mxz);
        out.maxH = fmaxf(L.maxH, R.maxH);
        out.maxHs = fmaxf(L.maxHs, R.maxHs);
        out.mom = NodeMom{L.mom.sx + R.mom.sx, L.mom.sy + R.mom.sy, L.mom.sz + R.mom.sz, L.mom.m + R.mom.m};
        if (out.mom.m > 0.0) {
            const double im = 1.0 / out.mom.m;
            out.cx = static_cast<float>(out.mom.sx * im);
            out.cy = static_cast<float>(out.mom.sy * im);
            out.cz = static_cast<float>(out.mom.sz * im);
        } else {                                   // massless subtree (sph_gravity.cu:591-595)
            out.cx = 0.5f * (L.cx + R.cx);
            out.cy = 0.5f * (L.cy + R.cy);
            out.cz = 0.5f * (L.cz + R.cz);
        }
        if (kMoments) {
            const float mL = static_cast<float>(L.mom.m), mR = static_cast<float>(R.mom.m);
            const float lx = L.cx - out.cx, ly = L.cy - out.cy, lz = L.cz - out.cz;
            const float rx = R.cx - out.cx, ry = R.cy - out.cy, rz = R.cz - out.cz;
            out.s[0] = L.s[0] + R.s[0] + mL * lx * lx + mR * rx * rx;
            out.s[1] = L.s[1] + R.s[1] + mL * ly * ly + mR * ry * ry;
            out.s[2] = L.s[2] + R.s[2] + mL * lz * lz + mR * rz * rz;
            out.s[3] = L.s[3] + R.s[3] + mL * lx * ly + mR * rx * ry;
            out.s[4] = L.s[4] + R.s[4] + mL * lx * lz + mR * rx * rz;
            out.s[5] = L.s[5] + R.s[5] + mL * ly * lz + mR * ry * rz;
            __stcg(&w.nodeQuad[2 * static_cast<size_t>(pNode)], make_float4(out.s[0], out.s[1], out.s[2], out.s[3]));
            __stcg(&w.nodeQuad[2 * static_cast<size_t>(pNode) + 1], make_float4(out.s[4], out.s[5], 0.0f, 0.0f));
        }
        const float mSum = static_cast<float>(out.mom.m);
        const float dNode = fmaxf(out.mxx - out.mnx, fmaxf(out.mxy - out.mny, out.mxz - out.mnz));
        float4* rec = w.node + 4 * static_cast<size_t>(pNode);
        __stcg(&rec[0], make_float4(out.cx, out.cy, out.cz, mSum));
        __stcg(&rec[1], make_float4(__fmul_rn(dNode, dNode), __int_as_float(lc), __int_as_float(rc), out.maxHs));
        __stcg(&rec[2], make_float4(out.mnx, out.mny, out.mnz, out.maxH));
        __stcg(&rec[3], make_float4(out.mxx, out.mxy, out.mxz, 0.0f));
        double2* mp = reinterpret_cast<double2*>(w.nodeMom + pNode);
        __stcg(&mp[0], make_double2(out.mom.sx, out.mom.sy));
        __stcg(&mp[1], make_double2(out.mom.sz, out.mom.m));
        if (bvh.aabbMinX != nullptr) {
            bvh.aabbMinX[pNode] = out.mnx; bvh.aabbMinY[pNode] = out.mny; bvh.aabbMinZ[pNode] = out.mnz;
            bvh.aabbMaxX[pNode] = out.mxx; bvh.aabbMaxY[pNode] = out.mxy; bvh.aabbMaxZ[pNode] = out.mxz;
            bvh.nodeMaxH[pNode] = out.maxH; bvh.nodeMass[pNode] = mSum;
            bvh.comX[pNode] = out.cx; bvh.comY[pNode] = out.cy; bvh.comZ[pNode] = out.cz;
        }
        if (bvh.nodeComMass != nullptr) {
            bvh.nodeComMass[pNode] = AstraeaFloat4{out.cx, out.cy, out.cz, mSum};
            bvh.nodeMinExtent[pNode] = AstraeaFloat4{out.mnx, out.mny, out.mnz, dNode};
            bvh.nodeMaxHPacked[pNode] = AstraeaFloat4{out.mxx, out.mxy, out.mxz, out.maxH};
        }
        mine = out;
        curr = pNode;
        pNode = grand;
    }
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

cudaError_t launchRefit(const AstraeaRadixBvh& bvh, const Work& w, uint32_t n, bool moments, cudaStream_t st) {
    if (n < 2u) return cudaSuccess;
    if (moments)
        refitKernel<true><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n);
    else
        refitKernel<false><<<gridFor(n, 256), 256, 0, st>>>(bvh, w, n);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
