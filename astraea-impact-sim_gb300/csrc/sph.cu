// sph.cu -- neighbour lists, SPH pass 1 / pass 2 and the XSPH drift (sm_103a).
//
// Restates sphPass1Kernel (engine/sph_gravity.cu:645-788), sphPass2Kernel
// (:965-1287) and leapfrogDriftKernel (:1376-1489).  The engine walks the
// tree three times per step with one particle per lane; a lane's pair body
// only runs when that lane is in range, so most lanes idle.  Here:
//   * one group walk per step (buildNeighborsKernel) writes, for every
//     particle, the list of j with r_ij < max(Hs_i, Hs_j) -- a superset of the
//     pass-1, pass-2 and next-drift neighbour sets (see common.cuh);
//   * pass 1, pass 2 and the drift run one thread per particle over its own
//     list, re-applying the engine's exact FP32 range test, so every lane
//     works on its own pairs;
//   * neighbour data is read from packed records (pass 1: position + Hs
//     and velocity + volume m/rho in one 32-byte record; drift: position + H and
//     velocity + density; pass 2: a 96-byte record written by the EOS
//     kernel, read in three 32-byte pieces), one 256-bit load per piece
//     instead of one gather per field.
// A particle whose list overflowed the per-particle capacity is served by a
// per-thread depth-first walk with the same superset test (rare path).
#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kNbWarps = 4;
constexpr int kNbStack = 384;   // entries per warp (peak use: 80 at 1M, 88 at 16M)
constexpr int kNbList = 64;
constexpr uint32_t kNbExpand = 32;   // an opened node of at most this many particles is read as its leaf range

// dirMem[k] (k = 4 [sx > 0] + 2 [sy > 0] + [sz > 0], s in {-1, 1}^3, the
// octant diagonals): the member {x, y, z, Hs} with the largest projection
// on direction s (first member on ties); undMin/undMax: the undecided nodes of one walk round
// {box min, node maxHs} / {box max}; the member positions are staged in
// undMin while dirMem is computed.
struct NbWarpSmem {
    int stack[kNbStack];
    // candidate leaves, pair-interleaved for the f32x2 pipes:
    // cand[8k..8k+7] = {xA, xB, yA, yB, zA, zB, HsA, HsB} of entries 2k, 2k+1
    float cand[8 * (kNbList / 2)];
    int candIdx[kNbList];
    float4 dirMem[8];
    float4 undMin[32];
    float4 undMax[32];
};

__device__ __forceinline__ uint32_t laneMaskLt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// One global store, issued only where `pred` holds (a predicated st.global).
__device__ __forceinline__ void storeIf(uint32_t* p, uint32_t v, bool pred) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.u32 [%0], %1;\n\t}"
                 :: "l"(p), "r"(v), "r"(static_cast<uint32_t>(pred)));
}

template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32) buildNeighborsKernel(Work w, uint32_t n, uint32_t numGroups,
                                                                    uint32_t* groupCounter) {
    __shared__ NbWarpSmem smem[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    NbWarpSmem& S = smem[warp];
    unsigned long long nEntries = 0, nCand = 0;
    bool overflow = false, stackOverflow = false;
    const uint32_t maxNbr = w.maxNbr;

    if (n < 2u) {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            w.nbrCount[i] = 0u;
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
        float4 me = make_float4(0.f, 0.f, 0.f, 0.f);
        float Hs = 0.0f;
        if (active) {
            me = __ldg(&w.leaf[i].a);
            Hs = me.w;
        }
        const float gminx = warpMinF(active ? me.x : 3.0e38f), gmaxx = warpMaxF(active ? me.x : -3.0e38f);
        const float gminy = warpMinF(active ? me.y : 3.0e38f), gmaxy = warpMaxF(active ? me.y : -3.0e38f);
        const float gminz = warpMinF(active ? me.z : 3.0e38f), gmaxz = warpMaxF(active ? me.z : -3.0e38f);
        const float gHs = warpMaxF(Hs);
        // per-direction extreme members (dirMem); member data staged in undMin
        const float cxg = 0.5f * (gminx + gmaxx), cyg = 0.5f * (gminy + gmaxy), czg = 0.5f * (gminz + gmaxz);
        S.undMin[lane] = make_float4(me.x, me.y, me.z, Hs);
        __syncwarp();
        if (lane < 8) {
            const float sx = (lane & 4) ? 1.0f : -1.0f, sy = (lane & 2) ? 1.0f : -1.0f, sz = (lane & 1) ? 1.0f : -1.0f;
            float best = -3.0e38f;
            int bi = 0;
            for (int m = 0; m < act; ++m) {
                const float4 q = S.undMin[m];
                const float pr = sx * (q.x - cxg) + sy * (q.y - cyg) + sz * (q.z - czg);
                if (pr > best) { best = pr; bi = m; }
            }
            S.dirMem[lane] = S.undMin[bi];
        }
        __syncwarp();
        if (lane == 0) { S.stack[0] = rootL; S.stack[1] = rootR; }
        // candidates form a ring of 64 entries: a round appends at most 32
        // behind the pending ones (at most 31), a flush takes the 32 oldest,
        // which start at entry 0 or 32 (cHead toggles) -- nothing is moved
        int sp = 2, cCount = 0, cHead = 0;
        uint32_t cnt = 0, rounds = 0;
        uint32_t* myList = w.nbrList + static_cast<size_t>(g) * maxNbr * 32u + static_cast<uint32_t>(lane);
        __syncwarp();

        auto putCand = [&](int slot, float x, float y, float z, float hs, int j) {
            float* b = S.cand + 8 * (slot >> 1) + (slot & 1);
            b[0] = x; b[2] = y; b[4] = z; b[6] = hs;
            S.candIdx[slot] = j;
        };
        // Superset test r < max(Hs_i, Hs_j) in plain FMA arithmetic, two
        // candidates per instruction: every pass re-tests its own radius
        // exactly, and Hs exceeds those radii by 0.9 %, far more than any
        // rounding difference.  Tests candidates 0 .. 2 pairs - 1 in order.
        const f2 X2 = pack2(me.x, me.x), Y2 = pack2(me.y, me.y), Z2 = pack2(me.z, me.z);
        auto flush = [&](int pairs) {
            if (active) {
                for (int k = cHead >> 1; k < (cHead >> 1) + pairs; ++k) {
                    const float* b = S.cand + 8 * k;
                    const ulonglong2 u = *reinterpret_cast<const ulonglong2*>(b);       // (x), (y)
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(b + 4);   // (z), (Hs)
                    const int2 jj = *reinterpret_cast<const int2*>(S.candIdx + 2 * k);
                    const f2 dx = sub2(X2, u.x), dy = sub2(Y2, u.y), dz = sub2(Z2, v.x);
                    float r2a, r2b, ha, hb;
                    unpack2(fma2(dz, dz, fma2(dy, dy, mul2(dx, dx))), r2a, r2b);
                    unpack2(v.y, ha, hb);
                    const float Ra = fmaxf(Hs, ha), Rb = fmaxf(Hs, hb);
                    // appends as predicated stores: no branch per candidate
                    // (a branch per hit cost 6 % of the build at 1M)
                    const bool hA = r2a < Ra * Ra && jj.x != static_cast<int>(i);
                    storeIf(myList + static_cast<size_t>(cnt) * 32u, static_cast<uint32_t>(jj.x), hA && cnt < maxNbr);
                    cnt += hA ? 1u : 0u;
                    const bool hB = r2b < Rb * Rb && jj.y != static_cast<int>(i);
                    storeIf(myList + static_cast<size_t>(cnt) * 32u, static_cast<uint32_t>(jj.y), hB && cnt < maxNbr);
                    cnt += hB ? 1u : 0u;
                }
            }
        };
        while (sp > 0) {
            if (++rounds > 2u * n + 64u) {     // only reachable on a corrupted tree
                stackOverflow = true;
                break;
            }
            const int take = min(sp, 32);
            const int c = (lane < take) ? S.stack[sp - take + lane] : 0;
            sp -= take;
            __syncwarp();
            const bool has = lane < take && c >= -static_cast<int>(n) && c < static_cast<int>(n) - 1;
            const bool isLeaf = has && c < 0;
            bool open = false;
            int cl = 0, cr = 0;
            bool undecided = false;
            float4 bmin = make_float4(0.f, 0.f, 0.f, 0.f), bmax = bmin;
            float nodeHs = 0.0f;
            if (has && c >= 0) {
                const float4* rec = w.node + 4 * static_cast<size_t>(c);
                const float4 r1 = __ldg(&rec[1]);
                bmin = __ldg(&rec[2]);
                bmax = __ldg(&rec[3]);
                cl = __float_as_int(r1.y);
                cr = __float_as_int(r1.z);
                nodeHs = r1.w;
                // (1) box-box distance bounds every member's point-box distance
                const float dx = fmaxf(0.0f, fmaxf(bmin.x - gmaxx, gminx - bmax.x));
                const float dy = fmaxf(0.0f, fmaxf(bmin.y - gmaxy, gminy - bmax.y));
                const float dz = fmaxf(0.0f, fmaxf(bmin.z - gmaxz, gminz - bmax.z));
                const float Rg = fmaxf(gHs, nodeHs);
                if (dx * dx + dy * dy + dz * dz <= Rg * Rg * 1.00001f) {
                    // (2) the member furthest towards the node opens it when in range;
                    // (3) otherwise the whole group decides
                    const float ux = 0.5f * (bmin.x + bmax.x) - cxg, uy = 0.5f * (bmin.y + bmax.y) - cyg,
                                uz = 0.5f * (bmin.z + bmax.z) - czg;
                    const float4 dm = S.dirMem[(ux >= 0.0f ? 4 : 0) | (uy >= 0.0f ? 2 : 0) | (uz >= 0.0f ? 1 : 0)];
                    const float R = fmaxf(dm.w, nodeHs);
                    if (pointBoxDist2(dm.x, dm.y, dm.z, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z) <=
                        R * R * 1.00001f)
                        open = true;
                    else
                        undecided = true;
                }
            }
            const unsigned und = __ballot_sync(0xffffffffu, undecided);
            if (und) {
                const int nu = __popc(und);
                const int slot = __popc(und & laneMaskLt());
                if (undecided) {
                    S.undMin[slot] = make_float4(bmin.x, bmin.y, bmin.z, nodeHs);
                    S.undMax[slot] = make_float4(bmax.x, bmax.y, bmax.z, 0.0f);
                }
                __syncwarp();
                unsigned bits = 0u;
                for (int k = 0; k < nu; ++k) {
                    const float4 mn = S.undMin[k], mx = S.undMax[k];
                    const float R = fmaxf(Hs, mn.w);
                    const bool near = active && pointBoxDist2(me.x, me.y, me.z, mn.x, mn.y, mn.z, mx.x, mx.y, mx.z) <=
                                                    R * R * 1.00001f;
                    bits |= (__any_sync(0xffffffffu, near) ? 1u : 0u) << k;
                }
                if (undecided) open = (bits >> slot) & 1u;
                __syncwarp();
            }
            // An opened node of at most 32 particles is not descended: its
            // sorted leaf range is read whole below (one coalesced load).
            uint2 rng = make_uint2(1u, 0u);               // empty unless a small node is expanded
            if (open) {
                const uint2 r = __ldg(&w.nodeRange[c]);
                if (r.x <= r.y && r.y < n && r.y - r.x < kNbExpand) {
                    rng = r;
                    open = false;
                }
            }
            unsigned expandMask = __ballot_sync(0xffffffffu, rng.x <= rng.y);
            unsigned openMask = __ballot_sync(0xffffffffu, open);
            if (sp + 2 * __popc(openMask) > kNbStack) {
                stackOverflow = true;     // cannot happen for trees of depth < 32
                openMask = 0u;
                open = false;
            }
            if (open) {
                const int pos = sp + 2 * __popc(openMask & laneMaskLt());
                S.stack[pos] = cl;
                S.stack[pos + 1] = cr;
            }
            sp += 2 * __popc(openMask);
            // A leaf becomes a candidate only if it can reach the group box.
            float4 pm = make_float4(0.f, 0.f, 0.f, 0.f);
            float hsj = 0.0f;
            bool keep = false;
            if (isLeaf) {
                pm = __ldg(&w.leaf[~c].a);
                hsj = pm.w;
                const float dx = fmaxf(0.0f, fmaxf(gminx - pm.x, pm.x - gmaxx));
                const float dy = fmaxf(0.0f, fmaxf(gminy - pm.y, pm.y - gmaxy));
                const float dz = fmaxf(0.0f, fmaxf(gminz - pm.z, pm.z - gmaxz));
                const float R = fmaxf(gHs, hsj);
                keep = dx * dx + dy * dy + dz * dz <= R * R * 1.00001f;
            }
            const unsigned leafMask = __ballot_sync(0xffffffffu, keep);
            if (keep) putCand((cHead + cCount + __popc(leafMask & laneMaskLt())) & 63, pm.x, pm.y, pm.z, hsj, ~c);
            cCount += __popc(leafMask);
            nCand += __popc(leafMask);
            __syncwarp();
            if (cCount >= 32) {
                flush(16);
                __syncwarp();
                cCount -= 32;
                cHead ^= 32;
            }
            while (expandMask) {                // small opened nodes: their particles, lane by lane
                const int src = __ffs(expandMask) - 1;
                expandMask &= expandMask - 1u;
                const uint32_t first = __shfl_sync(0xffffffffu, rng.x, src);
                const uint32_t last = __shfl_sync(0xffffffffu, rng.y, src);
                for (uint32_t base = first; base <= last; base += 32u) {
                const uint32_t j = base + static_cast<uint32_t>(lane);
                bool keepJ = false;
                float4 pj = make_float4(0.f, 0.f, 0.f, 0.f);
                float hj = 0.0f;
                if (j <= last) {
                    pj = __ldg(&w.leaf[j].a);
                    hj = pj.w;
                    const float dx = fmaxf(0.0f, fmaxf(gminx - pj.x, pj.x - gmaxx));
                    const float dy = fmaxf(0.0f, fmaxf(gminy - pj.y, pj.y - gmaxy));
                    const float dz = fmaxf(0.0f, fmaxf(gminz - pj.z, pj.z - gmaxz));
                    const float R = fmaxf(gHs, hj);
                    keepJ = dx * dx + dy * dy + dz * dz <= R * R * 1.00001f;
                }
                const unsigned km = __ballot_sync(0xffffffffu, keepJ);
                if (keepJ) putCand((cHead + cCount + __popc(km & laneMaskLt())) & 63, pj.x, pj.y, pj.z, hj, static_cast<int>(j));
                cCount += __popc(km);
                nCand += __popc(km);
                __syncwarp();
                if (cCount >= 32) {
                    flush(16);
                    __syncwarp();
                    cCount -= 32;
                    cHead ^= 32;
                }
                }
            }
        }
        if (cCount & 1) {                  // odd tail: a pad entry no member can reach
            if (lane == 0) putCand(cHead + cCount, 3.0e38f, 3.0e38f, 3.0e38f, 0.0f, -1);
            __syncwarp();
        }
        flush((cCount + 1) >> 1);
        if (active) {
            w.nbrCount[i] = cnt;
            if (cnt > maxNbr) overflow = true;
        }
        nEntries += cnt;
        __syncwarp();
    }
    const unsigned long long tot = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(nEntries & 0xffffffffu));
    const bool anyOver = __any_sync(0xffffffffu, overflow);
    if (lane == 0) {
        atomicAdd(&w.status->counters[kCntNeighborEntries], tot);
        atomicAdd(&w.status->counters[kCntNeighborCandidates], nCand);
        if (anyOver) atomicOr(&w.status->flags, kFlagNeighborOverflow);
        if (stackOverflow) atomicOr(&w.status->flags, kFlagStackOverflow);
    }
}

// Neighbour lists are group-interleaved: entry k of particle i is word
// ((i / 32) maxNbr + k) 32 + i % 32, so the 32 particles of a group (the
// lanes of one warp in every pass) read their k-th entries as one 128-byte
// row and a lane's list never shares a sector with another lane's.
__device__ __forceinline__ const uint32_t* listOf(const Work& w, uint32_t i) {
    return w.nbrList + static_cast<size_t>(i >> 5) * w.maxNbr * 32u + (i & 31u);
}

// Visit every j of particle i's superset list; when the list overflowed,
// walk the tree depth-first with the same superset test instead.
template <class F>
__device__ __forceinline__ void forEachCandidate(const Work& w, uint32_t i, F&& f) {
    const uint32_t c = __ldg(&w.nbrCount[i]);
    if (c <= w.maxNbr) {
        const uint32_t* list = listOf(w, i);
        for (uint32_t k = 0; k < c; ++k) f(__ldg(&list[static_cast<size_t>(k) * 32u]));
        return;
    }
    atomicAdd(&w.status->counters[kCntFallbackWalks], 1ull);
    const float4 me = __ldg(&w.leaf[i].a);
    const float Hs = me.w;
    int stack[kTreeStack];
    int sp = 0;
    const float4 rootR1 = __ldg(&w.node[1]);
    stack[sp++] = __float_as_int(rootR1.y);
    stack[sp++] = __float_as_int(rootR1.z);
    const int nInt = static_cast<int>(w.capacity);
    uint32_t iters = 0;
    while (sp > 0) {
        const int c2 = stack[--sp];
        if (++iters > 4u * w.capacity + 64u || c2 < -nInt || c2 >= nInt - 1) {   // corrupted tree only
            atomicOr(&w.status->flags, kFlagStackOverflow);
            break;
        }
        if (c2 < 0) {
            const uint32_t j = static_cast<uint32_t>(~c2);
            if (j == i) continue;
            const float4 q = __ldg(&w.leaf[j].a);
            const float R = fmaxf(Hs, q.w);
            if (len2Engine(__fsub_rn(me.x, q.x), __fsub_rn(me.y, q.y), __fsub_rn(me.z, q.z)) < __fmul_rn(R, R)) f(j);
            continue;
        }
        const float4* rec = w.node + 4 * static_cast<size_t>(c2);
        const float4 r1 = __ldg(&rec[1]);
        const float4 bmin = __ldg(&rec[2]);
        const float4 bmax = __ldg(&rec[3]);
        const float R = fmaxf(Hs, r1.w);
        if (pointBoxDist2(me.x, me.y, me.z, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z) <= R * R * 1.00001f) {
            if (sp + 2 <= kTreeStack) {
                stack[sp++] = __float_as_int(r1.y);
                stack[sp++] = __float_as_int(r1.z);
            } else {
                atomicOr(&w.status->flags, kFlagStackOverflow);
            }
        }
    }
}

// List words are read once per pass and the lists (308 B per particle) do
// not fit in L1: read them without allocating in L1, which keeps L1 for the
// neighbour records.  Four consecutive entries of one particle (32 words
// apart in the group-interleaved layout).
__device__ __forceinline__ uint32_t ldWordNoL1(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint4 ldListNoL1(const uint32_t* list, uint32_t k) {
    const uint32_t* p = list + static_cast<size_t>(k) * 32u;
    return make_uint4(ldWordNoL1(p), ldWordNoL1(p + 32), ldWordNoL1(p + 64), ldWordNoL1(p + 96));
}

// Same candidate set as forEachCandidate, with each candidate's first record
// loaded by `load(j)` for four list entries before any `body(j, rec)` runs,
// so four independent gathers are in flight per thread, and the next four
// list entries loaded before those four bodies run.
template <class L, class B>
__device__ __forceinline__ void forEachCandidatePrefetched(const Work& w, uint32_t i, L&& load, B&& body) {
    const uint32_t c = __ldg(&w.nbrCount[i]);
    if (c <= w.maxNbr) {
        const uint32_t* list = listOf(w, i);
        uint32_t k = 0;
        uint4 q = c >= 4 ? ldListNoL1(list, 0u) : make_uint4(0u, 0u, 0u, 0u);
        for (; k + 4 <= c; k += 4) {
            const uint4 next = (k + 8 <= c) ? ldListNoL1(list, k + 4) : q;
            const auto r0 = load(q.x), r1 = load(q.y), r2 = load(q.z), r3 = load(q.w);
            body(q.x, r0); body(q.y, r1); body(q.z, r2); body(q.w, r3);
            q = next;
        }
        for (; k < c; ++k) {
            const uint32_t j = __ldg(&list[static_cast<size_t>(k) * 32u]);
            body(j, load(j));
        }
        return;
    }
    forEachCandidate(w, i, [&](uint32_t j) { body(j, load(j)); });
}

// Adds a per-thread count to a device counter with one atomic per group of
// threads that reach the call together (the running threads of a warp).
__device__ __forceinline__ void addCount(DevStatus* st, int which, uint32_t v) {
    const unsigned m = __activemask();
    const unsigned tot = __reduce_add_sync(m, v);
    if ((threadIdx.x & 31u) == static_cast<unsigned>(__ffs(m) - 1))
        atomicAdd(&st->counters[which], static_cast<unsigned long long>(tot));
}

// ---------------------------------------------------------------- pass 1 ---
// 6 blocks per SM (80 registers): no spills; 7 blocks (72) spilled and ran 1.6 % slower
__global__ void __launch_bounds__(128, 6) pass1Kernel(AstraeaParticles p, Work w, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const F8 rec = ldg256(&w.leaf[i].a);
    const float4 me = rec.a, vr = rec.b;
    const float mi = __ldg(&p.mass[i]);
    const float hi = fmaxf(__ldg(&p.h[i]), 1.0e-6f);
    const float h0i = fmaxf(__ldg(&p.h0[i]), 1.0e-6f);
    const float rhoI = fmaxf(__ldg(&p.rho[i]), 1.0e-9f);
    const float Hi = 2.0f * hi;
    const float Hi2 = __fmul_rn(Hi, Hi);
    const float w0 = 21.0f / (2.0f * kPiF * Hi * Hi * Hi);
    const float Hi5 = (Hi * Hi) * (Hi * Hi) * Hi;
    const float gNormI = 210.0f / (kPiF * Hi5);
    const float invHi = 1.0f / Hi;
    float shep = (mi / rhoI) * w0;
    int ngb = 1;
    float nsX = 0.f, nsY = 0.f, nsZ = 0.f;
    float gXX = 0.f, gXY = 0.f, gXZ = 0.f, gYX = 0.f, gYY = 0.f, gYZ = 0.f, gZX = 0.f, gZY = 0.f, gZZ = 0.f;
    if (n >= 2u) {
        // one 32-byte record per candidate: {x, y, z, Hs}, {vx, vy, vz, m / max(rho, 1e-9)}
        forEachCandidatePrefetched(w, i, [&](uint32_t j) { return ldg256(&w.leaf[j].a); }, [&](uint32_t j, const F8& rj) {
            const float4 q = rj.a;
            const float dx = __fsub_rn(me.x, q.x), dy = __fsub_rn(me.y, q.y), dz = __fsub_rn(me.z, q.z);
            const float r2 = len2Engine(dx, dy, dz);
            if (!(r2 < Hi2)) return;                       // sph_gravity.cu:713
            ++ngb;
            const float4 vj = rj.b;
            const float r = sqrtf(r2);
            const float volJ = vj.w;
            const float wij = wendlandC2I(r, Hi, invHi, w0);
            shep += volJ * wij;
            nsX -= volJ * dx * wij;
            nsY -= volJ * dy * wij;
            nsZ -= volJ * dz * wij;
            const float gc = wendlandC2GradI(r, Hi, invHi, gNormI);
            const float gx = gc * dx, gy = gc * dy, gz = gc * dz;
            const float dvx = vj.x - vr.x, dvy = vj.y - vr.y, dvz = vj.z - vr.z;
            gXX += volJ * dvx * gx; gXY += volJ * dvx * gy; gXZ += volJ * dvx * gz;
            gYX += volJ * dvy * gx; gYY += volJ * dvy * gy; gYZ += volJ * dvy * gz;
            gZX += volJ * dvz * gx; gZY += volJ * dvz * gy; gZZ += volJ * dvz * gz;
        });
    }
    addCount(w.status, kCntPass1Pairs, static_cast<uint32_t>(ngb - 1));
    p.shepardC[i] = shep;                                   // sph_gravity.cu:772-787
    const float normNs = sqrtf(nsX * nsX + nsY * nsY + nsZ * nsZ);
    float fs = fminf(1.0f, fmaxf(0.0f, 1.6f * fmaxf(1.0f - shep, normNs / hi) - 0.15f));
    if (ngb <= 2) fs = 1.0f;
    p.surfFactor[i] = fs;
    p.divV[i] = gXX + gYY + gZZ;
    p.curlVX[i] = gZY - gYZ;
    p.curlVY[i] = gXZ - gZX;
    p.curlVZ[i] = gYX - gXY;
    const float ratio = 56.0f / static_cast<float>(ngb);
    const float factor = fminf(1.08f, fmaxf(0.92f, cbrtf(ratio)));
    const float hNew = fminf(6.0f * h0i, fmaxf(0.35f * h0i, hi * factor));
    p.h[i] = hNew;
    // records of the next drift (positions and h do not change before it)
    const float Hd = 2.0f * fmaxf(hNew, 1.0e-6f);
    w.drift[i].a = make_float4(me.x, me.y, me.z, Hd);
    w.driftAux[i] = make_float2(mi, wendlandNorm(Hd));
}

// ---------------------------------------------------------------- pass 2 ---
// Reads the pass-2 records written by the EOS kernel (layout and derived
// values: integrate.cu, writePass2Record): one 256-bit load per 32-byte
// piece, and no per-pair division for quantities of the neighbour alone.
__global__ void __launch_bounds__(128, 4) pass2Kernel(AstraeaParticles p, Work w, uint32_t n,
                                                   const uint32_t* livingFlags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* R = w.rec2;
    const float4 a0 = __ldg(&R[kRec2Width * static_cast<size_t>(i) + 0]);
    const float4 a1 = __ldg(&R[kRec2Width * static_cast<size_t>(i) + 1]);
    const float4 a2 = __ldg(&R[kRec2Width * static_cast<size_t>(i) + 2]);
    const float4 a4 = __ldg(&R[kRec2Width * static_cast<size_t>(i) + 4]);
    const float4 a5 = __ldg(&R[kRec2Width * static_cast<size_t>(i) + 5]);
    const float xi = a0.x, yi = a0.y, zi = a0.z, hi = a0.w, Hi = 2.0f * hi;
    const float vxi = a1.x, vyi = a1.y, vzi = a1.z, mi = a1.w;
    const float rhoI = a2.x, pOverRho2I = a2.y, csI = a2.z, fBalI = a2.w;
    const float sXXi = __ldg(&p.sXX[i]), sYYi = __ldg(&p.sYY[i]), sZZi = __ldg(&p.sZZ[i]);
    const float sXYi = __ldg(&p.sXY[i]), sXZi = __ldg(&p.sXZ[i]), sYZi = __ldg(&p.sYZ[i]);
    const int matI = __float_as_int(a4.z);
    const float Ri = a4.w;
    const float gradNormI = a5.y, invRhoI2 = a5.z, invHi = a5.w;
    const float pI = effectivePressure(__ldg(&p.pressure[i]), __ldg(&p.phaseId[i]));   // the record's P_eff
    const float sXXr = sXXi * invRhoI2, sYYr = sYYi * invRhoI2, sZZr = sZZi * invRhoI2;
    const float sXYr = sXYi * invRhoI2, sXZr = sXZi * invRhoI2, sYZr = sYZi * invRhoI2;
    const float tempI = __ldg(&p.tempK[i]);
    const float damI = __ldg(&p.damage[i]);
    const float fSurf = __ldg(&p.surfFactor[i]);

    float axS = 0.f, ayS = 0.f, azS = 0.f, drC = 0.f, drD = 0.f, duP = 0.f, duAv = 0.f, duT = 0.f, duS = 0.f;
    float gXX = 0.f, gXY = 0.f, gXZ = 0.f, gYX = 0.f, gYY = 0.f, gYZ = 0.f, gZX = 0.f, gZY = 0.f, gZZ = 0.f;
    uint32_t nPairs = 0;
    if (n >= 2u) {
        // records in 32-byte pieces: {q0, q1} for every candidate (one sector),
        // {q2, q3} and {q4, q5} for the candidates in range
        forEachCandidatePrefetched(w, i, [&](uint32_t j) { return ldg256(&R[kRec2Width * static_cast<size_t>(j)]); },
                                   [&](uint32_t j, const F8& q01) {
            const float4 b0 = q01.a;
            const float dx = __fsub_rn(xi, b0.x), dy = __fsub_rn(yi, b0.y), dz = __fsub_rn(zi, b0.z);
            const float r2 = len2Engine(dx, dy, dz);
            const float hj = b0.w, Hj = 2.0f * hj;
            const float Hm = fmaxf(Hi, Hj);
            if (!(r2 < __fmul_rn(Hm, Hm))) return;          // sph_gravity.cu:1071
            ++nPairs;
            const F8 q23 = ldg256(&R[kRec2Width * static_cast<size_t>(j) + 2]);
            const F8 q45 = ldg256(&R[kRec2Width * static_cast<size_t>(j) + 4]);
            const float4 b1 = q01.b, b2 = q23.a, b3 = q23.b, b4 = q45.a, b5 = q45.b;
            const float mj = b1.w, rhoJ = b2.x, pOverRho2J = b2.y, csJ = b2.z, fBalJ = b2.w;
            const float volJ = b5.x;
            const float dvx = vxi - b1.x, dvy = vyi - b1.y, dvz = vzi - b1.z;
            const float vDotR = dvx * dx + dvy * dy + dvz * dz;
            const float r = sqrtf(r2);
            const float gI = wendlandC2GradI(r, Hi, invHi, gradNormI), gJ = wendlandC2GradI(r, Hj, b5.w, b5.y);
            const float gb = 0.5f * (gI + gJ);
            const float gx = gb * dx, gy = gb * dy, gz = gb * dz;
            const float vDotG = dvx * gx + dvy * gy + dvz * gz;
            drC += volJ * vDotG;                               // continuity (:1114)
            // The delta-SPH and viscosity terms are evaluated for every pair in
            // range and kept by a select (the engine's conditions, the same
            // values): as branches they cost pass 2 11 % at 1M.
            {                                                  // delta-SPH diffusion (:1115-1119)
                const float rDotG = -(dx * gx + dy * gy + dz * gz);
                const float dd = r2 + 0.01f * Hi * Hi;
                const float t = drD + volJ * (2.0f * (rhoJ - rhoI) / dd) * rDotG;
                drD = (__float_as_int(b4.z) == matI) ? t : drD;
            }
            float piIJ;                                        // Monaghan AV x Balsara (:1121-1128)
            {
                const float hB = 0.5f * (hi + hj), cB = 0.5f * (csI + csJ), rB = 0.5f * (rhoI + rhoJ);
                const float muIJ = __fdividef(hB * vDotR, r2 + 0.01f * hB * hB);
                const float t = __fdividef(-1.0f * cB * muIJ + 2.0f * muIJ * muIJ, rB) * (0.5f * (fBalI + fBalJ));
                piIJ = (vDotR < 0.0f) ? t : 0.0f;
            }
            float tens = 0.0f;                                 // tensile correction (:1130-1142)
            const float Rj = b4.w;
            if (Ri + Rj > 0.0f) {
                const float Hb = 0.5f * (Hi + Hj);
                if (r < Hb) {
                    const float qb = __fdividef(r, Hb), om = 1.0f - qb, om2 = om * om;
                    const float fr = (om2 * om2 * (1.0f + 4.0f * qb)) * (1.0f / 0.6328125f);
                    const float fr2 = fr * fr;
                    tens = (Ri + Rj) * (fr2 * fr2);
                }
            }
            const float iso = -mj * ((pOverRho2I + pOverRho2J) + piIJ + tens);
            axS += iso * gx; ayS += iso * gy; azS += iso * gz;
            duP += mj * vDotG;
            duAv += 0.5f * mj * piIJ * vDotG;
            duT += 0.5f * mj * tens * vDotG;
            const float tXX = sXXr + b3.x, tYY = sYYr + b3.y, tZZ = sZZr + b3.z, tXY = sXYr + b3.w;
            const float tXZ = sXZr + b4.x, tYZ = sYZr + b4.y;
            axS += mj * (tXX * gx + tXY * gy + tXZ * gz);      // deviatoric stress (:1161-1163)
            ayS += mj * (tXY * gx + tYY * gy + tYZ * gz);
            azS += mj * (tXZ * gx + tYZ * gy + tZZ * gz);
            const float wx = -dvx, wy = -dvy, wz = -dvz;
            duS += mj * ((sXXi * wx + sXYi * wy + sXZi * wz) * gx + (sXYi * wx + sYYi * wy + sYZi * wz) * gy +
                         (sXZi * wx + sYZi * wy + sZZi * wz) * gz);
            const float gxi = gI * dx, gyi = gI * dy, gzi = gI * dz;   // velocity gradient (:1173-1179)
            gXX += volJ * wx * gxi; gXY += volJ * wx * gyi; gXZ += volJ * wx * gzi;
            gYX += volJ * wy * gxi; gYY += volJ * wy * gyi; gYZ += volJ * wy * gzi;
            gZX += volJ * wz * gxi; gZY += volJ * wz * gyi; gZZ += volJ * wz * gzi;
        });
    }
    addCount(w.status, kCntPass2Pairs, nPairs);
    p.accX[i] += axS;                                          // sph_gravity.cu:1213-1218
    p.accY[i] += ayS;
    p.accZ[i] += azS;
    const float diffMask = (__ldg(&p.shepardC[i]) > 0.85f) ? (1.0f - fSurf) : 0.0f;
    p.drhoDt[i] = rhoI * drC + 0.05f * Hi * csI * diffMask * drD;
    const float duStress = invRhoI2 * duS;

    // Surface radiative cooling (sph_gravity.cu:1222-1235), in FP32: every
    // quantity stays far inside the float range (area <~1e13 m^2, T^4 <~1e20).
    const bool livingIntact = livingFlags[1] != 0u;
    const float tAmb = (livingIntact && __ldg(&p.bodyId[i]) == 0u && damI < 0.8f) ? 255.0f : 3.0f;
    const float mSi = fmaxf(mi * 1.0e24f, 1.0f);
    const float rhoSi = fmaxf(rhoI * 1.0e6f, 1.0e-3f);
    const float rP = cbrtf((3.0f * mSi) / (4.0f * kPiF * rhoSi));
    const float area = kPiF * rP * rP;
    const float T4 = tempI * tempI * tempI * tempI;
    const float Ta4 = tAmb * tAmb * tAmb * tAmb;
    const float dT4 = fmaxf(0.0f, T4 - Ta4);
    const float pRad = fSurf * 0.9f * 5.670374419e-8f * area * dT4;
    p.radPowerW[i] = pRad;
    const float duRad = -pRad / (fmaxf(mi, 1.0e-30f) * 1.0e27f);
    p.duDt[i] = pOverRho2I * duP + duAv + duT + duStress + duRad;

    // Jaumann stress rate + Grady-Kipp damage (sph_gravity.cu:1239-1286).
    const MatConst& st = c_mat[matIndex(static_cast<uint8_t>(matI))];
    if (st.muShear <= 0.0f || st.tMelt <= 0.0f) {
        p.dSXX[i] = 0.f; p.dSYY[i] = 0.f; p.dSZZ[i] = 0.f; p.dSXY[i] = 0.f; p.dSXZ[i] = 0.f; p.dSYZ[i] = 0.f;
        p.dDamageCbrtDt[i] = 0.0f;
        return;
    }
    const float tNorm = tempI / st.tMelt;
    const float soft = fmaxf(0.0f, 1.0f - tNorm * tNorm);
    const float muEff = (1.0f - damI) * st.muShear * soft;
    const float tr3 = (gXX + gYY + gZZ) * (1.0f / 3.0f);
    const float eXX = gXX - tr3, eYY = gYY - tr3, eZZ = gZZ - tr3;
    const float eXY = 0.5f * (gXY + gYX), eXZ = 0.5f * (gXZ + gZX), eYZ = 0.5f * (gYZ + gZY);
    const float rXY = 0.5f * (gXY - gYX), rXZ = 0.5f * (gXZ - gZX), rYZ = 0.5f * (gYZ - gZY);
    const float rYX = -rXY, rZX = -rXZ, rZY = -rYZ;
    p.dSXX[i] = 2.0f * muEff * eXX + 2.0f * (sXYi * rXY + sXZi * rXZ);
    p.dSYY[i] = 2.0f * muEff * eYY + 2.0f * (sXYi * rYX + sYZi * rYZ);
    p.dSZZ[i] = 2.0f * muEff * eZZ + 2.0f * (sXZi * rZX + sYZi * rZY);
    p.dSXY[i] = 2.0f * muEff * eXY + sXXi * rYX + sXZi * rYZ + sYYi * rXY + sYZi * rXZ;
    p.dSXZ[i] = 2.0f * muEff * eXZ + sXXi * rZX + sXYi * rZY + sZZi * rXZ + sYZi * rXY;
    p.dSYZ[i] = 2.0f * muEff * eYZ + sXYi * rZX + sYYi * rZY + sXZi * rYX + sZZi * rYZ;
    if (tempI < st.tMelt && damI < 1.0f) {
        const float sigmaMax = maxPrincipalStress(pI, sXXi, sYYi, sZZi, sXYi, sXZi, sYZi);
        const float stiff = fmaxf(st.bulkK + (4.0f / 3.0f) * st.muShear, 1.0e-12f);
        const float epsT = fmaxf(0.0f, sigmaMax) / stiff;
        const float epsF = fmaxf(__ldg(&p.epsFail[i]), 1.0e-8f);
        const float cCrack = fmaxf(csI, sqrtf((st.bulkK + (4.0f / 3.0f) * st.muShear) / rhoI));
        p.dDamageCbrtDt[i] = (epsT > epsF) ? (0.4f * cCrack / hi) : 0.0f;
    } else {
        p.dDamageCbrtDt[i] = 0.0f;
    }
}

// ----------------------------------------------------------------- drift ---
// XSPH position update (sph_gravity.cu:1376-1489).  Neighbour positions come
// from the leaf records (the positions before this drift), so no thread reads
// a position another thread is moving.  The position add is done in FP64.
__global__ void __launch_bounds__(128) driftKernel(AstraeaParticles p, Work w, uint32_t n, const float* dtDev,
                                                   float dtHost, bool useList, bool toScratch,
                                                   uint32_t* boundsWords) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float mn[3] = {1.0e30f, 1.0e30f, 1.0e30f}, mx[3] = {-1.0e30f, -1.0e30f, -1.0e30f};
    if (i < n) {
        const float dt = (dtDev != nullptr) ? *dtDev : dtHost;
        const F8 rec = ldg256(&w.drift[i].a);
        const float4 me = rec.a, vr = rec.b;               // {x, y, z, H}, {vx, vy, vz, rho}
        const float Hi = me.w;
        const float normI = __ldg(&w.driftAux[i]).y;
        const float invHi = 1.0f / Hi;
        const float rhoI = fmaxf(vr.w, 1.0e-9f);
        float sx = 0.f, sy = 0.f, sz = 0.f;
        uint32_t nPairs = 0;
        if (useList && n >= 2u) {
            // one 32-byte record per candidate: {x, y, z, H}, {vx, vy, vz, rho}
            forEachCandidatePrefetched(w, i, [&](uint32_t j) { return ldg256(&w.drift[j].a); }, [&](uint32_t j, const F8& rj) {
                const float4 q = rj.a;
                const float dx = __fsub_rn(me.x, q.x), dy = __fsub_rn(me.y, q.y), dz = __fsub_rn(me.z, q.z);
                const float r2 = len2Engine(dx, dy, dz);
                const float Hj = q.w;
                const float Hm = fmaxf(Hi, Hj);
                if (!(r2 < __fmul_rn(Hm, Hm))) return;
                ++nPairs;
                const float4 vj = rj.b;
                const float2 aj = __ldg(&w.driftAux[j]);          // {m, Wendland norm of H_j}
                const float r = sqrtf(r2);
                const float wb = 0.5f * (wendlandC2I(r, Hi, invHi, normI) + wendlandC2N(r, Hj, aj.y));
                const float rb = 0.5f * (rhoI + fmaxf(vj.w, 1.0e-9f));
                const float co = __fdividef(aj.x, rb) * wb;
                sx += co * (vj.x - vr.x);
                sy += co * (vj.y - vr.y);
                sz += co * (vj.z - vr.z);
            });
        }
        addCount(w.status, kCntDriftPairs, nPairs);
        const double d = static_cast<double>(dt);
        const float nx = static_cast<float>(static_cast<double>(me.x) + d * (static_cast<double>(vr.x) + 0.25 * static_cast<double>(sx)));
        const float ny = static_cast<float>(static_cast<double>(me.y) + d * (static_cast<double>(vr.y) + 0.25 * static_cast<double>(sy)));
        const float nz = static_cast<float>(static_cast<double>(me.z) + d * (static_cast<double>(vr.z) + 0.25 * static_cast<double>(sz)));
        if (toScratch) {
            w.driftPos[i] = make_float4(nx, ny, nz, 0.0f);
        } else {
            p.posX[i] = nx; p.posY[i] = ny; p.posZ[i] = nz;
        }
        mn[0] = mx[0] = nx; mn[1] = mx[1] = ny; mn[2] = mx[2] = nz;
    }
    if (boundsWords != nullptr) blockBoundsToWords(mn, mx, boundsWords);
}

inline unsigned gridFor(uint32_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

cudaError_t launchBuildNeighbors(const Work& w, uint32_t n, int sms, cudaStream_t st, int warps) {
    if (n == 0) return cudaSuccess;
    const uint32_t groups = (n + 31u) / 32u;
    uint32_t* counter = w.words + kWNbrCounter;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    using NbFn = void (*)(Work, uint32_t, uint32_t, uint32_t*);
    const int wps = (warps == 2 || warps == 8) ? warps : kNbWarps;
    const NbFn kernel = (wps == 2) ? buildNeighborsKernel<2> : (wps == 8) ? buildNeighborsKernel<8>
                                                                         : buildNeighborsKernel<kNbWarps>;
    int perSm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, wps * 32, 0);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = std::min<uint32_t>(static_cast<uint32_t>(std::max(1, perSm) * sms),
                                               (groups + wps - 1) / wps);
    kernel<<<blocks, wps * 32, 0, st>>>(w, n, groups, counter);
    return cudaGetLastError();
}

cudaError_t launchPass1(const AstraeaParticles& p, const Work& w, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    pass1Kernel<<<gridFor(n, 128), 128, 0, st>>>(p, w, n);
    return cudaGetLastError();
}

cudaError_t launchPass2(const AstraeaParticles& p, const Work& w, uint32_t n, const uint32_t* livingFlags,
                        cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    pass2Kernel<<<gridFor(n, 128), 128, 0, st>>>(p, w, n, livingFlags);
    return cudaGetLastError();
}

cudaError_t launchDrift(const AstraeaParticles& p, const Work& w, uint32_t n, const float* dtDev, float dtHost,
                        bool useList, bool toScratch, uint32_t* boundsWords, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    driftKernel<<<gridFor(n, 128), 128, 0, st>>>(p, w, n, dtDev, dtHost, useList, toScratch, boundsWords);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
