// gravity.cu -- Barnes-Hut monopole gravity for sm_103a.
//
// Same interaction set as the engine kernel gravityBarnesHutKernel
// (engine/sph_gravity.cu:810-961): particles are taken in groups of 32
// consecutive sorted particles (one engine warp); every internal node reached
// is accepted as a monopole for the whole group iff every active member has
// dNode^2 < theta^2 r^2 and r^2 > 1e-20 (and, when theta^2 > 1/3, lies outside
// the node box), otherwise the group descends; leaves are evaluated
// particle-particle with eps_ij = (eps_i + eps_j)/2, monopoles with eps_i.
//
// GB300 restructuring (same sets, different schedule):
//   * the group walk is node-parallel: up to 32 pending nodes are loaded at
//     once, one per lane; a sound group-box bound accepts most far nodes, an
//     exact test of one representative member opens most near ones, and the
//     few undecided nodes are tested by all 32 members at once (one node per
//     warp iteration, one vote), so no lane loops over the group alone;
//   * accepted monopoles and reached leaves are appended to two per-warp
//     interaction lists in shared memory; every 32 entries the warp evaluates
//     them with each lane summing its own particle's force from broadcast
//     shared-memory reads (pure FP32 FMA + one rsqrt per pair);
//   * a persistent grid pulls groups from an atomic counter.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kGravWarps = 4;
constexpr int kGravStack = 1024;
constexpr int kGravList = 64;

struct GravWarpSmem {
    int stack[kGravStack];
    float4 mlist[kGravList];   // {comX, comY, comZ, G*mass}
    float4 plist[kGravList];   // {x, y, z, G*m}
    float2 paux[kGravList];    // {eps_j / 2, j (int bits)}
};

__device__ __forceinline__ uint32_t laneMaskLt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The engine's per-member acceptance test (sph_gravity.cu:914-929) with
// explicit IEEE rounding: dNode^2 < theta^2 r^2, r^2 > 1e-20 and, when
// checkInside, the member outside the node box.
__device__ __forceinline__ bool acceptsMember(float px, float py, float pz, float4 com, float dd, float theta2,
                                              bool checkInside, float4 bmin, float4 bmax) {
    const float r2 = len2Exact(__fsub_rn(px, com.x), __fsub_rn(py, com.y), __fsub_rn(pz, com.z));
    bool ok = (dd < __fmul_rn(theta2, r2)) && (r2 > 1.0e-20f);
    if (ok && checkInside && px >= bmin.x && px <= bmax.x && py >= bmin.y && py <= bmax.y && pz >= bmin.z &&
        pz <= bmax.z)
        ok = false;
    return ok;
}

struct Accum {
    float ax, ay, az, phi;
};

// Monopole terms: f = -G m / (r^2 + eps_i^2 + 1e-20)^(3/2) (sph_gravity.cu:935-942).
// epsI2 arrives with the 1e-20 already added: eps >= 8e-7, so 1e-20 is below
// half an ulp of eps^2 and both orders of the two additions round alike.
__device__ __forceinline__ void evalMonopoles(const float4* list, int cnt, float xi, float yi, float zi, float epsI2,
                                              Accum& a) {
#pragma unroll 4
    for (int e = 0; e < cnt; ++e) {
        const float4 q = list[e];
        const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float inv = rsqrtf(r2 + epsI2);
        const float inv3 = inv * inv * inv;
        const float f = -q.w * inv3;
        a.ax += f * dx;
        a.ay += f * dy;
        a.az += f * dz;
        a.phi -= q.w * inv;
    }
}

// Particle-particle terms with eps_ij = (eps_i + eps_j)/2 (sph_gravity.cu:875-889);
// the list carries eps_j/2.
__device__ __forceinline__ void evalParticles(const float4* list, const float2* aux, int cnt, float xi, float yi,
                                              float zi, float epsI, int self, Accum& a, uint32_t& nSelf) {
#pragma unroll 4
    for (int e = 0; e < cnt; ++e) {
        const float4 q = list[e];
        const float2 x2 = aux[e];
        const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float eij = fmaf(0.5f, epsI, x2.x);
        const float inv = rsqrtf(fmaf(eij, eij, r2));
        const float inv3 = inv * inv * inv;
        const bool isSelf = __float_as_int(x2.y) == self;
        const float gm = isSelf ? 0.0f : q.w;
        nSelf += isSelf ? 1u : 0u;
        const float f = -gm * inv3;
        a.ax += f * dx;
        a.ay += f * dy;
        a.az += f * dz;
        a.phi -= gm * inv;
    }
}

__global__ void __launch_bounds__(kGravWarps * 32) gravityKernel(AstraeaParticles p, Work w, uint32_t n,
                                                                 float theta2, bool checkInside, uint32_t numGroups,
                                                                 uint32_t* groupCounter) {
    __shared__ GravWarpSmem smem[kGravWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    GravWarpSmem& S = smem[warp];
    unsigned long long nInter = 0, nTests = 0, nUndecided = 0;
    bool overflowed = false;

    if (n == 1u) {                                   // sph_gravity.cu:824-832
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            p.accX[0] = 0.0f; p.accY[0] = 0.0f; p.accZ[0] = 0.0f; p.phiGrav[0] = 0.0f;
        }
        return;
    }
    const float4 rootR1 = __ldg(&w.node[1]);
    const int rootL = __float_as_int(rootR1.y), rootR = __float_as_int(rootR1.z);

    for (;;) {
        uint32_t g = 0;
        if (lane == 0) g = atomicAdd(groupCounter, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= numGroups) break;
        const uint32_t i = g * 32u + static_cast<uint32_t>(lane);
        const bool active = i < n;
        const int act = static_cast<int>(min(32u, n - g * 32u));
        float4 me = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float epsI = 0.8e-6f;
        if (active) {
            me = __ldg(&w.leafPM[i]);
            epsI = __ldg(&w.leafAux[i]).y;
        }
        const float xi = me.x, yi = me.y, zi = me.z;
        const float epsI2 = epsI * epsI + 1.0e-20f;
        const float gminx = warpMinF(active ? xi : 3.0e38f), gmaxx = warpMaxF(active ? xi : -3.0e38f);
        const float gminy = warpMinF(active ? yi : 3.0e38f), gmaxy = warpMaxF(active ? yi : -3.0e38f);
        const float gminz = warpMinF(active ? zi : 3.0e38f), gmaxz = warpMaxF(active ? zi : -3.0e38f);
        // representative member: the one nearest the group-box centre
        const float cxg = 0.5f * (gminx + gmaxx), cyg = 0.5f * (gminy + gmaxy), czg = 0.5f * (gminz + gmaxz);
        float dc = active ? (xi - cxg) * (xi - cxg) + (yi - cyg) * (yi - cyg) + (zi - czg) * (zi - czg) : 3.0e38f;
        int best = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, dc, o);
            const int ob = __shfl_xor_sync(0xffffffffu, best, o);
            if (od < dc || (od == dc && ob < best)) { dc = od; best = ob; }
        }
        const float repx = __shfl_sync(0xffffffffu, xi, best);
        const float repy = __shfl_sync(0xffffffffu, yi, best);
        const float repz = __shfl_sync(0xffffffffu, zi, best);
        if (lane == 0) { S.stack[0] = rootL; S.stack[1] = rootR; }
        int sp = 2, mCount = 0, pCount = 0;
        uint32_t rounds = 0;
        Accum acc{0.0f, 0.0f, 0.0f, 0.0f};
        uint32_t nSelf = 0;
        __syncwarp();

        while (sp > 0) {
            if (++rounds > 2u * n + 64u) {     // only reachable on a corrupted tree
                overflowed = true;
                break;
            }
            const int take = min(sp, 32);
            const int c = (lane < take) ? S.stack[sp - take + lane] : 0;
            sp -= take;
            __syncwarp();
            // child references outside [~(n-1), n-2] cannot come from a valid tree
            const bool has = lane < take && c >= -static_cast<int>(n) && c < static_cast<int>(n) - 1;
            const bool isLeaf = has && c < 0;
            const bool isNode = has && c >= 0;
            bool accept = false;
            float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            int cl = 0, cr = 0;
            bool undecided = false;
            float dd = 0.0f;
            float4 bmin = make_float4(0.f, 0.f, 0.f, 0.f), bmax = bmin;
            if (isNode) {
                const float4* rec = w.node + 4 * static_cast<size_t>(c);
                r0 = __ldg(&rec[0]);
                const float4 r1 = __ldg(&rec[1]);
                cl = __float_as_int(r1.y);
                cr = __float_as_int(r1.z);
                dd = __fmul_rn(r1.x, r1.x);
                bool disjoint = true;
                if (checkInside) {
                    bmin = __ldg(&rec[2]);
                    bmax = __ldg(&rec[3]);
                    disjoint = bmax.x < gminx || bmin.x > gmaxx || bmax.y < gminy || bmin.y > gmaxy ||
                               bmax.z < gminz || bmin.z > gmaxz;
                }
                // (1) Sound group test: every member lies in the group box, so
                // its distance to the COM is at least the box distance D; the
                // 1e-5 margin covers the rounding of both computations.
                const float bx = fmaxf(0.0f, fmaxf(gminx - r0.x, r0.x - gmaxx));
                const float by = fmaxf(0.0f, fmaxf(gminy - r0.y, r0.y - gmaxy));
                const float bz = fmaxf(0.0f, fmaxf(gminz - r0.z, r0.z - gmaxz));
                const float D2 = bx * bx + by * by + bz * bz;
                if (disjoint && D2 > 2.0e-20f && dd < theta2 * D2 * 0.99999f) {
                    accept = true;
                } else if (!acceptsMember(repx, repy, repz, r0, dd, theta2, checkInside, bmin, bmax)) {
                    accept = false;   // (2) one member (the representative) already opens it
                } else {
                    undecided = true; // (3) decided below by the whole group
                }
            }
            // (3) exact test of each undecided node by all members at once
            unsigned und = __ballot_sync(0xffffffffu, undecided);
            nUndecided += __popc(und);
            while (und) {
                const int k = __ffs(und) - 1;
                und &= und - 1;
                float4 q = make_float4(__shfl_sync(0xffffffffu, r0.x, k), __shfl_sync(0xffffffffu, r0.y, k),
                                       __shfl_sync(0xffffffffu, r0.z, k), 0.0f);
                const float ddk = __shfl_sync(0xffffffffu, dd, k);
                float4 mn = bmin, mx = bmax;
                if (checkInside) {
                    mn = make_float4(__shfl_sync(0xffffffffu, bmin.x, k), __shfl_sync(0xffffffffu, bmin.y, k),
                                     __shfl_sync(0xffffffffu, bmin.z, k), 0.0f);
                    mx = make_float4(__shfl_sync(0xffffffffu, bmax.x, k), __shfl_sync(0xffffffffu, bmax.y, k),
                                     __shfl_sync(0xffffffffu, bmax.z, k), 0.0f);
                }
                const bool ok = !active || acceptsMember(xi, yi, zi, q, ddk, theta2, checkInside, mn, mx);
                const bool all = __all_sync(0xffffffffu, ok);
                if (lane == k) accept = all;
            }
            bool open = isNode && !accept;
            unsigned openMask = __ballot_sync(0xffffffffu, open);
            if (sp + 2 * __popc(openMask) > kGravStack) {
                // Out of stack: the group takes these nodes as monopoles, the
                // rule of the engine kernel when its stack is full (:933).
                if (open) { open = false; accept = true; }
                openMask = 0u;
                overflowed = true;
            }
            if (open) {
                const int pos = sp + 2 * __popc(openMask & laneMaskLt());
                S.stack[pos] = cl;
                S.stack[pos + 1] = cr;
            }
            sp += 2 * __popc(openMask);
            const unsigned accMask = __ballot_sync(0xffffffffu, accept);
            if (accept) S.mlist[mCount + __popc(accMask & laneMaskLt())] = make_float4(r0.x, r0.y, r0.z, kGPsuF * r0.w);
            mCount += __popc(accMask);
            const unsigned leafMask = __ballot_sync(0xffffffffu, isLeaf);
            if (isLeaf) {
                const int j = ~c;
                const float4 pm = __ldg(&w.leafPM[j]);
                const float ej = __ldg(&w.leafAux[j]).y;
                const int slot = pCount + __popc(leafMask & laneMaskLt());
                S.plist[slot] = make_float4(pm.x, pm.y, pm.z, kGPsuF * pm.w);
                S.paux[slot] = make_float2(0.5f * ej, __int_as_float(j));
            }
            pCount += __popc(leafMask);
            nTests += __popc(__ballot_sync(0xffffffffu, isNode));
            __syncwarp();
            if (mCount >= 32) {
                mCount -= 32;
                if (active) evalMonopoles(S.mlist + mCount, 32, xi, yi, zi, epsI2, acc);
                nInter += static_cast<unsigned long long>(act) * 32u;
                __syncwarp();
            }
            if (pCount >= 32) {
                pCount -= 32;
                if (active) evalParticles(S.plist + pCount, S.paux + pCount, 32, xi, yi, zi, epsI, static_cast<int>(i), acc, nSelf);
                nInter += static_cast<unsigned long long>(act) * 32u;
                __syncwarp();
            }
        }
        if (active) {
            evalMonopoles(S.mlist, mCount, xi, yi, zi, epsI2, acc);
            evalParticles(S.plist, S.paux, pCount, xi, yi, zi, epsI, static_cast<int>(i), acc, nSelf);
            p.accX[i] = acc.ax;
            p.accY[i] = acc.ay;
            p.accZ[i] = acc.az;
            p.phiGrav[i] = acc.phi;
        }
        nInter += static_cast<unsigned long long>(act) * static_cast<unsigned>(mCount + pCount);
        // nSelf: every active lane met itself once among the leaves.
        const unsigned selfTotal = __reduce_add_sync(0xffffffffu, nSelf);
        if (lane == 0) nInter -= selfTotal;
        __syncwarp();
    }
    if (lane == 0) {
        DevStatus* st = reinterpret_cast<DevStatus*>(w.status);
        atomicAdd(&st->counters[kCntGravityInteractions], nInter);
        atomicAdd(&st->counters[kCntGravityNodeTests], nTests);
        atomicAdd(&st->counters[kCntGravityUndecided], nUndecided);
        if (overflowed) atomicOr(&st->flags, kFlagStackOverflow);
    }
}

}  // namespace

cudaError_t launchGravity(const AstraeaParticles& p, const Work& w, uint32_t n, float theta, int sms,
                          cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const float th = fmaxf(0.0f, theta);
    const float theta2 = th * th;
    const bool checkInside = theta2 > 0.333333f;
    const uint32_t groups = (n + 31u) / 32u;
    uint32_t* counter = w.words + kWGroupCounter;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    int perSm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, gravityKernel, kGravWarps * 32, 0);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = std::min<uint32_t>(static_cast<uint32_t>(std::max(1, perSm) * sms),
                                               (groups + kGravWarps - 1) / kGravWarps);
    gravityKernel<<<blocks, kGravWarps * 32, 0, st>>>(p, w, n, theta2, checkInside, groups, counter);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
