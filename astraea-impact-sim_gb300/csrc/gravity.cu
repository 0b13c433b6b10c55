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
//     once, one per lane, and decided by three tests of increasing cost:
//     (1) a sound lower bound on every member's distance to the node's COM
//     (the larger of the group-box distance and the distance to the group's
//     26-direction bounding polytope) accepts most far nodes; (2) the exact
//     test of the member that lies furthest towards the node (looked up per
//     group for 26 directions) opens most near ones; (3) the few nodes still
//     undecided are tested by all 32 members at once, two nodes per warp
//     iteration (f32x2) from a shared-memory list, so no lane loops over the
//     group;
//   * accepted monopoles and reached leaves are appended to two per-warp
//     interaction lists in shared memory; every 32 entries the warp evaluates
//     them with each lane summing its own particle's force from broadcast
//     shared-memory reads, two entries per instruction on the packed FP32
//     pipes (add/mul/fma.rn.f32x2) plus one rsqrt per pair;
//   * a persistent grid pulls groups from an atomic counter.
#include "kernels.h"

namespace astraea_gb300 {
namespace {

constexpr int kGravWarps = 4;
constexpr int kGravStack = 768;           // entries per warp (peak use: 274 at 1M, 322 at 16M)
constexpr int kGravList = 64;

// Interaction lists are stored pair-interleaved so that one 16-byte shared
// load yields packed (entry 2k, entry 2k+1) operands for the f32x2 pipes:
// mlist[8k..8k+7] = {xA, xB, yA, yB, zA, zB, -GmA, -GmB}; plist likewise,
// with peps[2k..2k+1] = {eps_jA / 2, eps_jB / 2}.  With the quadrupole
// (far-field mode 1) an mlist pair block is 20 floats: the 8 above, then
// G Q_xx, G Q_yy, G Q_zz, G Q_xy, G Q_xz, G Q_yz of both entries, where
// Q = 3 S - tr(S) I is the node's traceless quadrupole.  Both lists are
// rings of 64 entries: a round appends at most 32 behind the pending ones
// (at most 31), and a flush evaluates the 32 oldest, which start at entry 0
// or 32 (the head toggles), so no entry is ever moved and the evaluation
// order is the append order.
// dirPos[k] (k = 9 (sx + 1) + 3 (sy + 1) + (sz + 1), s in {-1, 0, 1}): the
// member with the largest projection on the unit direction s / |s| (first
// member on ties) and, in .w, that projection measured from the group-box
// centre.  und[] holds the compacted undecided nodes of one walk round; the
// same storage holds the member positions while dirPos is computed.
template <bool kInside, bool kQuad, bool kExpand = false>
struct __align__(16) GravWarpSmem {
    int stack[kGravStack];
    float mlist[(kQuad ? 20 : 8) * (kGravList / 2)];
    float plist[8 * (kGravList / 2)];
    float peps[kGravList];
    float4 dirPos[27];
    float4 und[32];                    // {com.x, com.y, com.z, dNode^2}
    float4 undMin[kInside ? 32 : 1];
    float4 undMax[kInside ? 32 : 1];
    // far-field mode 3 only; last, and whole float4s, so the arrays above
    // keep the 16-byte alignment of their vector loads in every variant
    float4 flist4[kExpand ? 5 * (kGravList / 2) : 1];   // far nodes of the group expansion (mlist layout)
    float4 facc4[kExpand ? 5 : 1];                      // the group's expansion coefficients (see farTaylor)
};
// the vector loads of the lists (16 bytes) and of peps (8 bytes)
template <bool kInside, bool kQuad, bool kExpand>
constexpr bool gravSmemAligned() {
    using S = GravWarpSmem<kInside, kQuad, kExpand>;
    return offsetof(S, mlist) % 16 == 0 && offsetof(S, plist) % 16 == 0 && offsetof(S, peps) % 16 == 0 &&
           offsetof(S, dirPos) % 16 == 0 && offsetof(S, und) % 16 == 0 && offsetof(S, undMin) % 16 == 0 &&
           offsetof(S, undMax) % 16 == 0 && offsetof(S, flist4) % 16 == 0 && offsetof(S, facc4) % 16 == 0 &&
           sizeof(S) % 16 == 0;
}
static_assert(gravSmemAligned<false, false, false>() && gravSmemAligned<true, false, false>() &&
              gravSmemAligned<false, true, false>() && gravSmemAligned<true, true, false>() &&
              gravSmemAligned<false, true, true>() && gravSmemAligned<true, true, true>(),
              "gravity shared-memory layout must keep 16-byte alignment");

__device__ __forceinline__ uint32_t laneMaskLt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The engine's per-member acceptance test (sph_gravity.cu:914-929) with the
// engine's rounding (len2Engine): dNode^2 < theta^2 r^2, r^2 > 1e-20 and,
// when checkInside, the member outside the node box.
__device__ __forceinline__ bool acceptsMember(float px, float py, float pz, float4 com, float dd, float theta2,
                                              bool checkInside, float4 bmin, float4 bmax) {
    const float r2 = len2Engine(__fsub_rn(px, com.x), __fsub_rn(py, com.y), __fsub_rn(pz, com.z));
    bool ok = (dd < __fmul_rn(theta2, r2)) && (r2 > 1.0e-20f);
    if (ok && checkInside && px >= bmin.x && px <= bmax.x && py >= bmin.y && py <= bmax.y && pz >= bmin.z &&
        pz <= bmax.z)
        ok = false;
    return ok;
}

__device__ __forceinline__ f2 rsqrt2(f2 v) {
    float a, b;
    unpack2(v, a, b);
    return pack2(rsqrtf(a), rsqrtf(b));
}

struct Accum2 {
    f2 ax, ay, az, phi;   // two partial sums each (even / odd entries)
};

// Monopole terms: f = -G m / (r^2 + eps_i^2 + 1e-20)^(3/2) (sph_gravity.cu:935-942),
// two entries per instruction.  `pairs` pairs starting at list pair `first`.
// E2 = packed eps_i^2 + 1e-20 (eps >= 8e-7, so 1e-20 is below half an ulp of
// eps^2 and the order of the two additions does not matter).
// kQuad adds the quadrupole field of the node, r = x_i - COM, with the same
// softened 1/r:  a += G [Q r / r^5 - 5/2 (r.Q.r) r / r^7],
//                phi -= G (r.Q.r) / (2 r^5).
template <bool kQuad>
__device__ __forceinline__ void evalMonopoles2(const float* list, int first, int pairs, f2 X, f2 Y, f2 Z, f2 E2,
                                               Accum2& a) {
    constexpr int kW = kQuad ? 20 : 8;
    const f2 kHalfNeg = pack2(-0.5f, -0.5f), kFiveHalvesNeg = pack2(-2.5f, -2.5f);
#pragma unroll 2
    for (int k = first; k < first + pairs; ++k) {
        const float* b = list + kW * k;
        const ulonglong2 u = *reinterpret_cast<const ulonglong2*>(b);       // (x), (y)
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(b + 4);   // (z), (-Gm)
        const f2 dx = sub2(X, u.x), dy = sub2(Y, u.y), dz = sub2(Z, v.x);
        const f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const f2 inv = rsqrt2(add2(r2, E2));
        const f2 inv2 = mul2(inv, inv);
        const f2 inv3 = mul2(inv2, inv);
        const f2 f = mul2(v.y, inv3);
        a.ax = fma2(f, dx, a.ax);
        a.ay = fma2(f, dy, a.ay);
        a.az = fma2(f, dz, a.az);
        a.phi = fma2(v.y, inv, a.phi);
        if constexpr (kQuad) {
            const ulonglong2 q0 = *reinterpret_cast<const ulonglong2*>(b + 8);    // Qxx, Qyy
            const ulonglong2 q1 = *reinterpret_cast<const ulonglong2*>(b + 12);   // Qzz, Qxy
            const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(b + 16);   // Qxz, Qyz
            const f2 qr0 = fma2(q2.x, dz, fma2(q1.y, dy, mul2(q0.x, dx)));
            const f2 qr1 = fma2(q2.y, dz, fma2(q0.y, dy, mul2(q1.y, dx)));
            const f2 qr2 = fma2(q1.x, dz, fma2(q2.y, dy, mul2(q2.x, dx)));
            const f2 rqr = fma2(dz, qr2, fma2(dy, qr1, mul2(dx, qr0)));
            const f2 i5 = mul2(inv3, inv2);
            const f2 t = mul2(mul2(rqr, mul2(i5, inv2)), kFiveHalvesNeg);
            a.ax = fma2(t, dx, fma2(qr0, i5, a.ax));
            a.ay = fma2(t, dy, fma2(qr1, i5, a.ay));
            a.az = fma2(t, dz, fma2(qr2, i5, a.az));
            a.phi = fma2(mul2(rqr, i5), kHalfNeg, a.phi);
        }
    }
}

// Particle-particle terms with eps_ij = (eps_i + eps_j)/2 (sph_gravity.cu:875-889).
// The list includes the particle itself; its term adds exactly zero force
// (dx = dy = dz = 0) and a potential the caller subtracts again.
__device__ __forceinline__ void evalParticles2(const float* list, const float* peps, int first, int pairs, f2 X,
                                               f2 Y, f2 Z, f2 HE, Accum2& a) {
#pragma unroll 2
    for (int k = first; k < first + pairs; ++k) {
        const ulonglong2 u = *reinterpret_cast<const ulonglong2*>(list + 8 * k);
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(list + 8 * k + 4);
        const f2 ej = *reinterpret_cast<const f2*>(peps + 2 * k);
        const f2 dx = sub2(X, u.x), dy = sub2(Y, u.y), dz = sub2(Z, v.x);
        const f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const f2 eij = add2(HE, ej);
        const f2 inv = rsqrt2(fma2(eij, eij, r2));
        const f2 f = mul2(v.y, mul2(inv, mul2(inv, inv)));
        a.ax = fma2(f, dx, a.ax);
        a.ay = fma2(f, dy, a.ay);
        a.az = fma2(f, dz, a.az);
        a.phi = fma2(v.y, inv, a.phi);
    }
}

// Store entry `slot` of a pair-interleaved list.
__device__ __forceinline__ void putEntry(float* list, int slot, float x, float y, float z, float w) {
    float* b = list + 8 * (slot >> 1) + (slot & 1);
    b[0] = x; b[2] = y; b[4] = z; b[6] = w;
}

// Monopole entry of the mlist; with kQuad also its six quadrupole terms.
template <bool kQuad>
__device__ __forceinline__ void putMono(float* list, int slot, const float (&e)[10]) {
    float* b = list + (kQuad ? 20 : 8) * (slot >> 1) + (slot & 1);
#pragma unroll
    for (int k = 0; k < (kQuad ? 10 : 4); ++k) b[2 * k] = e[k];
}
template <bool kQuad>
__device__ __forceinline__ void getMono(const float* list, int slot, float (&e)[10]) {
    const float* b = list + (kQuad ? 20 : 8) * (slot >> 1) + (slot & 1);
#pragma unroll
    for (int k = 0; k < (kQuad ? 10 : 4); ++k) e[k] = b[2 * k];
}

// Far-field mode 3: the field of a far node about the group centre c, to
// second order in d = x_i - c.  With r = c - COM, s^2 = r^2 + eps_g^2 (Plummer
// softening with the group's mean eps^2), GM = G m:
//   phi(c) = -GM/s - (r.Q.r)/(2 s^5),   a(c) = -GM r/s^3 + [Q r/s^5 - 5/2 (r.Q.r) r/s^7]
// (monopole + quadrupole, Q = G (3S - tr S I), the expression of the member
// evaluation), and the monopole's derivatives
//   J_ij = da_i/dx_j = -GM (d_ij/s^3 - 3 r_i r_j/s^5)
//   H_ijk = dJ_ij/dx_k = -GM (-3 (d_ij r_k + d_ik r_j + d_jk r_i)/s^5 + 15 r_i r_j r_k/s^7).
// Coefficients (20): phi, a (3), J xx yy zz xy xz yz (6), H xxx yyy zzz xxy
// xxz xyy yyz xzz yzz xyz (10).  A member then takes
//   a_i = a + J d + 1/2 H:dd,   phi_i = phi - a.d - 1/2 d.J.d.
__device__ __forceinline__ void farTaylor(const float (&e)[10], float cx, float cy, float cz, float epsG2,
                                          float (&t)[20]) {
    const float rx = cx - e[0], ry = cy - e[1], rz = cz - e[2];
    const float s2 = rx * rx + ry * ry + rz * rz + epsG2;
    const float is = rsqrtf(s2), is2 = is * is, is3 = is * is2, is5 = is3 * is2, is7 = is5 * is2;
    const float gm = -e[3];                       // e[3] = -G m
    // quadrupole part of phi and a
    const float q0 = e[4] * rx + e[7] * ry + e[8] * rz;
    const float q1 = e[7] * rx + e[5] * ry + e[9] * rz;
    const float q2 = e[8] * rx + e[9] * ry + e[6] * rz;
    const float rqr = rx * q0 + ry * q1 + rz * q2;
    const float tq = -2.5f * rqr * is7;
    t[0] = -gm * is - 0.5f * rqr * is5;
    t[1] = -gm * is3 * rx + q0 * is5 + tq * rx;
    t[2] = -gm * is3 * ry + q1 * is5 + tq * ry;
    t[3] = -gm * is3 * rz + q2 * is5 + tq * rz;
    const float a3 = -gm * is3, b5 = 3.0f * gm * is5;   // J = a3 I + b5 r r^T
    t[4] = a3 + b5 * rx * rx; t[5] = a3 + b5 * ry * ry; t[6] = a3 + b5 * rz * rz;
    t[7] = b5 * rx * ry; t[8] = b5 * rx * rz; t[9] = b5 * ry * rz;
    const float c5 = 3.0f * gm * is5, c7 = -15.0f * gm * is7;   // H = c5 (sym d r) + c7 r r r
    t[10] = 3.0f * c5 * rx + c7 * rx * rx * rx;          // xxx
    t[11] = 3.0f * c5 * ry + c7 * ry * ry * ry;          // yyy
    t[12] = 3.0f * c5 * rz + c7 * rz * rz * rz;          // zzz
    t[13] = c5 * ry + c7 * rx * rx * ry;                  // xxy
    t[14] = c5 * rz + c7 * rx * rx * rz;                  // xxz
    t[15] = c5 * rx + c7 * rx * ry * ry;                  // xyy
    t[16] = c5 * rz + c7 * ry * ry * rz;                  // yyz
    t[17] = c5 * rx + c7 * rx * rz * rz;                  // xzz
    t[18] = c5 * ry + c7 * ry * rz * rz;                  // yzz
    t[19] = c7 * rx * ry * rz;                            // xyz
}

// 1 / |s| for a direction s in {-1, 0, 1}^3 with nz non-zero components.
__device__ __forceinline__ float invDirNorm(int nz) { return nz == 3 ? 0.57735027f : (nz == 2 ? 0.70710678f : 1.0f); }

// kDebug: the variant that serves the debugging calls (per-group interaction
// counts, the trace of one group's accepted nodes and leaves); their checks
// are kept out of the production variants, where they cost 2 % of the walk.
template <int kWarps, bool kInside, bool kQuad, bool kLearned, bool kExpand = false, bool kDebug = false>
__global__ void __launch_bounds__(kWarps * 32) gravityKernel(AstraeaParticles p, Work w, uint32_t n,
                                                                 float theta2, uint32_t numGroups,
                                                                 uint32_t* groupCounter, FarCapture ff) {
    static_assert(!kExpand || kQuad, "the group expansion is a quadrupole mode");
    __shared__ GravWarpSmem<kInside, kQuad, kExpand> smem[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    GravWarpSmem<kInside, kQuad, kExpand>& S = smem[warp];
    unsigned long long nInter = 0, nTests = 0, nUndecided = 0, nRounds = 0, nGroupEvals = 0, nBucketLeaves = 0;
    int spPeak = 0;
    bool overflowed = false;

    if (w.runIf != nullptr && *w.runIf == 0u) return;   // the gate of the learned mode passed
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
        const bool active = i < n;                  // active members are lanes 0 .. act-1
        const int act = static_cast<int>(min(32u, n - g * 32u));
        const unsigned long long interBefore = nInter;
        float4 me = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float epsI = 0.8e-6f;
        if (active) {
            me = __ldg(&w.leaf[i].a);
            const float4 aux = __ldg(&w.leafAux[i]);
            epsI = aux.y;
            me.w = aux.w;                                // the mass
        }
        const float xi = me.x, yi = me.y, zi = me.z;
        const float epsI2 = epsI * epsI + 1.0e-20f;
        const float gminx = warpMinF(active ? xi : 3.0e38f), gmaxx = warpMaxF(active ? xi : -3.0e38f);
        const float gminy = warpMinF(active ? yi : 3.0e38f), gmaxy = warpMaxF(active ? yi : -3.0e38f);
        const float gminz = warpMinF(active ? zi : 3.0e38f), gmaxz = warpMaxF(active ? zi : -3.0e38f);
        const float cxg = 0.5f * (gminx + gmaxx), cyg = 0.5f * (gminy + gmaxy), czg = 0.5f * (gminz + gmaxz);
        const float gExt = (gmaxx - gminx) + (gmaxy - gminy) + (gmaxz - gminz);
        const bool emitFar = kLearned && (g % ff.groupStride) == 0u;
        if (kLearned && lane == 0) ff.groups[g] = make_float4(cxg, cyg, czg, gExt);

        // Per-direction extreme members (dirPos); member positions staged in und[].
        S.und[lane] = make_float4(xi, yi, zi, 0.0f);
        __syncwarp();
        if (lane < 27) {
            const float sx = static_cast<float>(lane / 9 - 1), sy = static_cast<float>((lane / 3) % 3 - 1),
                        sz = static_cast<float>(lane % 3 - 1);
            const float inv = invDirNorm(static_cast<int>(fabsf(sx) + fabsf(sy) + fabsf(sz)));
            float best = -3.0e38f;
            int bi = 0;
            for (int m = 0; m < act; ++m) {
                const float4 q = S.und[m];
                const float pr = (sx * (q.x - cxg) + sy * (q.y - cyg) + sz * (q.z - czg)) * inv;
                if (pr > best) { best = pr; bi = m; }
            }
            const float4 q = S.und[bi];
            S.dirPos[lane] = make_float4(q.x, q.y, q.z, best);
        }
        if (lane == 0) { S.stack[0] = rootL; S.stack[1] = rootR; }
        int sp = 2, mCount = 0, pCount = 0, fCount = 0;
        int mHead = 0, pHead = 0;   // first pending entry of each ring list (0 or 32)
        uint32_t rounds = 0;
        // group expansion: the group's radius about its box centre c (IEEE
        // operations, so the far decision is reproducible) and mean eps^2
        float rg2 = 0.0f, epsG2 = 0.0f;
        if (kExpand) {
            rg2 = warpMaxF(active ? len2Exact(__fsub_rn(xi, cxg), __fsub_rn(yi, cyg), __fsub_rn(zi, czg)) : 0.0f);
            float e2 = active ? epsI * epsI : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            epsG2 = e2 / static_cast<float>(act);
            if (lane < 20) reinterpret_cast<float*>(S.facc4)[lane] = 0.0f;
        }
        const f2 X = pack2(xi, xi), Y = pack2(yi, yi), Z = pack2(zi, zi);
        const f2 E2 = pack2(epsI2, epsI2), HE = pack2(0.5f * epsI, 0.5f * epsI);
        Accum2 acc{0ull, 0ull, 0ull, 0ull};
        const uint32_t base = g * 32u;
        unsigned selfSeen = 0u;   // bit l: member l met its own leaf
        // far list -> the group's expansion coefficients: lane l takes entry l
        // of the first `cnt`, the 20 coefficients are summed over the warp
        auto flushFar = [&](int cnt) {
            if constexpr (!kExpand) return;
            float t[20];
            if (lane < cnt) {
                float e[10];
                getMono<true>(reinterpret_cast<const float*>(S.flist4), lane, e);
                farTaylor(e, cxg, cyg, czg, epsG2, t);
            } else {
#pragma unroll
                for (int k = 0; k < 20; ++k) t[k] = 0.0f;
            }
            float mine = 0.0f;
#pragma unroll
            for (int k = 0; k < 20; ++k) {
                float v = t[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == k) mine = v;
            }
            if (lane < 20) reinterpret_cast<float*>(S.facc4)[lane] += mine;
            __syncwarp();
        };
        auto flushP = [&]() {                 // evaluate the 32 entries from pHead
            if (active) evalParticles2(S.plist, S.peps, pHead >> 1, 16, X, Y, Z, HE, acc);
            nInter += static_cast<unsigned long long>(act) * 32u;
            __syncwarp();
            pCount -= 32;
            pHead ^= 32;
        };
        __syncwarp();

        while (sp > 0) {
            if (++rounds > 2u * n + 64u) {     // only reachable on a corrupted tree
                overflowed = true;
                break;
            }
            spPeak = max(spPeak, sp);
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
            bool farOk = false;
            float dd = 0.0f;
            float4 bmin = make_float4(0.f, 0.f, 0.f, 0.f), bmax = bmin;
            // Without the inside-box rule the tests run on every lane, the
            // results kept only where isNode (a lane without a node reads the
            // root's record): as a branch around them the walk was 2.4 % slower
            // at 1M.  With the rule (theta^2 > 1/3) the branch stays: there the
            // masked form needs more registers and was slower.
            if (kInside ? isNode : true) {
                const int cn = isNode ? c : 0;
                const float4* rec = w.node + 4 * static_cast<size_t>(cn);
                r0 = __ldg(&rec[0]);
                const float4 r1 = __ldg(&rec[1]);
                cl = __float_as_int(r1.y);
                cr = __float_as_int(r1.z);
                dd = r1.x;                       // dNode^2, rounded once by the refit
                bool disjoint = true;   // the inside-box rule of the theta test (kInside)
                bool boxApart = true;   // the same rule for the far test (theta_far^2 > 1/3)
                if (kInside || kLearned) {
                    bmin = __ldg(&rec[2]);
                    bmax = __ldg(&rec[3]);
                    boxApart = bmax.x < gminx || bmin.x > gmaxx || bmax.y < gminy || bmin.y > gmaxy ||
                               bmax.z < gminz || bmin.z > gmaxz;
                    if (kInside) disjoint = boxApart;
                }
                // (1) Sound lower bound on every member's distance to the COM:
                // the group-box distance, or the distance to the supporting
                // plane of the group in the direction s of the COM (all
                // members lie behind it).  Rounding: the box terms are single
                // subtractions (relative error 2^-24), the plane term carries
                // an absolute margin of 1e-6 (|u|_1 + group extent), several
                // times its error bound; 0.99999 covers the final products.
                const float bx = fmaxf(0.0f, fmaxf(gminx - r0.x, r0.x - gmaxx));
                const float by = fmaxf(0.0f, fmaxf(gminy - r0.y, r0.y - gmaxy));
                const float bz = fmaxf(0.0f, fmaxf(gminz - r0.z, r0.z - gmaxz));
                const float D2 = bx * bx + by * by + bz * bz;
                const float ux = r0.x - cxg, uy = r0.y - cyg, uz = r0.z - czg;
                const float ax = fabsf(ux), ay = fabsf(uy), az = fabsf(uz);
                const float t = 0.41421356f * fmaxf(ax, fmaxf(ay, az));
                const int sx = (ux >= t) - (ux <= -t), sy = (uy >= t) - (uy <= -t), sz = (uz >= t) - (uz <= -t);
                const float4 dp = S.dirPos[13 + 9 * sx + 3 * sy + sz];
                const float inv = invDirNorm(abs(sx) + abs(sy) + abs(sz));
                const float L = (static_cast<float>(sx) * ux + static_cast<float>(sy) * uy +
                                 static_cast<float>(sz) * uz) * inv - dp.w - 1.0e-6f * (ax + ay + az + gExt);
                const float Lb2 = fmaxf(D2, L > 0.0f ? L * L : 0.0f);
                // far test of mode 2: every member passes theta_far (by the
                // sound bound) and the node is far against the group's size
                if (kLearned)
                    farOk = isNode && emitFar && boxApart && Lb2 > 2.0e-20f && dd < ff.thetaFar2 * Lb2 * 0.99999f &&
                            gExt * gExt <= ff.gamma2 * (ux * ux + uy * uy + uz * uz);
                // (1) accepts; else (2) the member furthest towards the node
                // opens it; else (3) the whole group decides below
                const bool boundAccepts = disjoint && Lb2 > 2.0e-20f && dd < theta2 * Lb2 * 0.99999f;
                if (kInside) {
                    if (boundAccepts)
                        accept = true;
                    else if (acceptsMember(dp.x, dp.y, dp.z, r0, dd, theta2, kInside, bmin, bmax))
                        undecided = true;
                } else {
                    const bool extremeAccepts = acceptsMember(dp.x, dp.y, dp.z, r0, dd, theta2, kInside, bmin, bmax);
                    accept = isNode && boundAccepts;
                    undecided = isNode && !boundAccepts && extremeAccepts;
                }
            }
            // (3) exact test of each undecided node by all members at once
            const unsigned und = __ballot_sync(0xffffffffu, undecided);
            if (und) {
                const int nu = __popc(und);
                nUndecided += nu;
                const int slot = __popc(und & laneMaskLt());
                // pair-interleaved in und's storage: {comxA, comxB, comyA,
                // comyB, comzA, comzB, ddA, ddB} for undecided nodes 2k, 2k+1
                float* undP = reinterpret_cast<float*>(S.und);
                if (undecided) {
                    float* ub = undP + 8 * (slot >> 1) + (slot & 1);
                    ub[0] = r0.x; ub[2] = r0.y; ub[4] = r0.z; ub[6] = dd;
                    if (kInside) { S.undMin[slot] = bmin; S.undMax[slot] = bmax; }
                }
                __syncwarp();
                unsigned bits = 0u;
                // the engine's member test (acceptsMember) on two nodes per
                // iteration, rounded as the engine rounds it (len2Engine:
                // explicit __fmaf_rn / __fmul_rn, which the compiler neither
                // splits nor re-fuses, so a member on the theta boundary is
                // decided as the engine decides it)
                for (int k = 0; k < nu; k += 2) {
                    const float* ub = undP + 4 * k;
                    const float4 pa = *reinterpret_cast<const float4*>(ub);       // com xA, xB, yA, yB
                    const float4 pb = *reinterpret_cast<const float4*>(ub + 4);   // com zA, zB, ddA, ddB
                    const float r2a = len2Engine(__fsub_rn(xi, pa.x), __fsub_rn(yi, pa.z), __fsub_rn(zi, pb.x));
                    const float r2b = len2Engine(__fsub_rn(xi, pa.y), __fsub_rn(yi, pa.w), __fsub_rn(zi, pb.y));
                    const float ta = __fmul_rn(theta2, r2a), tb = __fmul_rn(theta2, r2b);
                    const float dda = pb.z, ddb = pb.w;
                    bool okA = dda < ta && r2a > 1.0e-20f, okB = ddb < tb && r2b > 1.0e-20f;
                    if (kInside) {
                        const float4 mnA = S.undMin[k], mxA = S.undMax[k];
                        const float4 mnB = S.undMin[k + 1], mxB = S.undMax[k + 1];
                        if (okA && xi >= mnA.x && xi <= mxA.x && yi >= mnA.y && yi <= mxA.y && zi >= mnA.z &&
                            zi <= mxA.z)
                            okA = false;
                        if (okB && xi >= mnB.x && xi <= mxB.x && yi >= mnB.y && yi <= mxB.y && zi >= mnB.z &&
                            zi <= mxB.z)
                            okB = false;
                    }
                    bits |= (__all_sync(0xffffffffu, !active || okA) ? 1u : 0u) << k;
                    if (k + 1 < nu) bits |= (__all_sync(0xffffffffu, !active || okB) ? 1u : 0u) << (k + 1);
                }
                if (undecided) accept = (bits >> slot) & 1u;
                __syncwarp();
            }
            if (kLearned) {
                // a node the theta test opens but the far test takes: a
                // monopole plus the learned correction of this (group, node)
                bool far = isNode && !accept && farOk;
                const unsigned farMask = __ballot_sync(0xffffffffu, far);
                if (farMask) {
                    uint32_t fb = 0;
                    if (lane == 0) fb = atomicAdd(ff.count, static_cast<uint32_t>(__popc(farMask)));
                    fb = __shfl_sync(0xffffffffu, fb, 0);
                    if (far) {
                        const uint32_t slot = fb + static_cast<uint32_t>(__popc(farMask & laneMaskLt()));
                        if (slot < ff.cap) {                     // full buffer: the node is opened
                            ff.pairs[slot] = make_uint2(g, static_cast<uint32_t>(c));
                            accept = true;
                        }
                    }
                }
            }
            bool open = isNode && !accept;
            // mode 3: an opened node of at most leafBucket particles is not
            // descended; its sorted leaf range is evaluated particle-particle
            uint2 brng = make_uint2(1u, 0u);
            if (kExpand && open && w.leafBucket > 0u) {
                const uint2 r = __ldg(&w.nodeRange[c]);
                if (r.x <= r.y && r.y < n && r.y - r.x < w.leafBucket) {
                    brng = r;
                    open = false;
                }
            }
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
            // mode 3: an accepted node far against the group (group radius <=
            // gamma |c - COM|) joins the group's expansion instead of being
            // evaluated by every member
            bool far = false;
            if (kExpand && accept) {
                const float R2 = len2Exact(__fsub_rn(cxg, r0.x), __fsub_rn(cyg, r0.y), __fsub_rn(czg, r0.z));
                far = rg2 <= __fmul_rn(w.expandGamma2, R2);
            }
            const unsigned accMask = __ballot_sync(0xffffffffu, accept && !far);
            const unsigned farMask = kExpand ? __ballot_sync(0xffffffffu, far) : 0u;
            if (kDebug && w.traceList != nullptr && g == w.traceGroup && (accept || isLeaf)) {
                const uint32_t k = atomicAdd(reinterpret_cast<uint32_t*>(w.traceList), 1u);
                if (k < w.traceCap) w.traceList[1 + k] = c;
            }
            if (accept) {
                float e[10] = {r0.x, r0.y, r0.z, -kGPsuF * r0.w, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (kQuad) {
                    const float4 s0 = __ldg(&w.nodeQuad[2 * static_cast<size_t>(c)]);      // Sxx Syy Szz Sxy
                    const float4 s1 = __ldg(&w.nodeQuad[2 * static_cast<size_t>(c) + 1]);  // Sxz Syz
                    const float tr = s0.x + s0.y + s0.z;
                    e[4] = kGPsuF * (3.0f * s0.x - tr);
                    e[5] = kGPsuF * (3.0f * s0.y - tr);
                    e[6] = kGPsuF * (3.0f * s0.z - tr);
                    e[7] = kGPsuF * 3.0f * s0.w;
                    e[8] = kGPsuF * 3.0f * s1.x;
                    e[9] = kGPsuF * 3.0f * s1.y;
                }
                if constexpr (kExpand) {
                    if (far)
                        putMono<true>(reinterpret_cast<float*>(S.flist4), fCount + __popc(farMask & laneMaskLt()), e);
                    else
                        putMono<kQuad>(S.mlist, (mHead + mCount + __popc(accMask & laneMaskLt())) & 63, e);
                } else {
                    putMono<kQuad>(S.mlist, (mHead + mCount + __popc(accMask & laneMaskLt())) & 63, e);
                }
            }
            mCount += __popc(accMask);
            if (kExpand) {
                fCount += __popc(farMask);
                nGroupEvals += __popc(farMask);
                __syncwarp();
                if (fCount >= 32) {
                    flushFar(32);
                    fCount -= 32;
                    if (lane < fCount) {
                        float e2[10];
                        getMono<true>(reinterpret_cast<const float*>(S.flist4), 32 + lane, e2);
                        putMono<true>(reinterpret_cast<float*>(S.flist4), lane, e2);
                    }
                    __syncwarp();
                }
            }
            const unsigned leafMask = __ballot_sync(0xffffffffu, isLeaf);
            unsigned selfBit = 0u;
            if (isLeaf) {
                const int j = ~c;
                const float4 pa = __ldg(&w.leaf[j].a);
                const float4 aux = __ldg(&w.leafAux[j]);
                const float4 pm = make_float4(pa.x, pa.y, pa.z, aux.w);
                const float ej = aux.y;
                const int slot = (pHead + pCount + __popc(leafMask & laneMaskLt())) & 63;
                putEntry(S.plist, slot, pm.x, pm.y, pm.z, -kGPsuF * pm.w);
                S.peps[slot] = 0.5f * ej;
                const uint32_t rel = static_cast<uint32_t>(j) - base;
                if (rel < 32u) selfBit = 1u << rel;
            }
            selfSeen |= __reduce_or_sync(0xffffffffu, selfBit);
            pCount += __popc(leafMask);
            nTests += __popc(__ballot_sync(0xffffffffu, isNode));
            __syncwarp();
            if (mCount >= 32) {                 // evaluate the 32 entries from mHead
                if (active) evalMonopoles2<kQuad>(S.mlist, mHead >> 1, 16, X, Y, Z, E2, acc);
                nInter += static_cast<unsigned long long>(act) * 32u;
                __syncwarp();
                mCount -= 32;
                mHead ^= 32;
            }
            if (pCount >= 32) flushP();
            if (kExpand) {
                // leaf buckets of this round: each range (at most 32 sorted
                // particles) appended to the particle list by the warp at once
                unsigned bucketMask = __ballot_sync(0xffffffffu, brng.x <= brng.y);
                while (bucketMask) {
                    const int src = __ffs(bucketMask) - 1;
                    bucketMask &= bucketMask - 1u;
                    const uint32_t first = __shfl_sync(0xffffffffu, brng.x, src);
                    const uint32_t last = __shfl_sync(0xffffffffu, brng.y, src);
                    const uint32_t j = first + static_cast<uint32_t>(lane);
                    const bool has = j <= last;
                    const unsigned hm = __ballot_sync(0xffffffffu, has);
                    unsigned sb = 0u;
                    if (has) {
                        const float4 pm = __ldg(&w.leaf[j].a);
                        const float4 aux = __ldg(&w.leafAux[j]);
                        const int slot = (pHead + pCount + __popc(hm & laneMaskLt())) & 63;
                        putEntry(S.plist, slot, pm.x, pm.y, pm.z, -kGPsuF * aux.w);
                        S.peps[slot] = 0.5f * aux.y;
                        const uint32_t rel = j - base;
                        if (rel < 32u) sb = 1u << rel;
                    }
                    const unsigned selfHere = __reduce_or_sync(0xffffffffu, sb);
                    selfSeen |= selfHere;
                    pCount += __popc(hm);
                    nBucketLeaves += static_cast<unsigned long long>(act) * __popc(hm) - __popc(selfHere);
                    __syncwarp();
                    if (pCount >= 32) flushP();
                }
            }
        }
        if (kExpand && fCount > 0) flushFar(fCount);
        // odd tails: pad with a massless entry (adds exactly zero)
        if (lane == 0) {
            if (mCount & 1) {
                const float zero[10] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                putMono<kQuad>(S.mlist, mHead + mCount, zero);
            }
            if (pCount & 1) { putEntry(S.plist, pHead + pCount, 0.0f, 0.0f, 0.0f, 0.0f); S.peps[pHead + pCount] = 0.0f; }
        }
        __syncwarp();
        if (active) {
            evalMonopoles2<kQuad>(S.mlist, mHead >> 1, (mCount + 1) >> 1, X, Y, Z, E2, acc);
            evalParticles2(S.plist, S.peps, pHead >> 1, (pCount + 1) >> 1, X, Y, Z, HE, acc);
            float a0, a1, b0, b1, c0, c1, d0, d1;
            unpack2(acc.ax, a0, a1);
            unpack2(acc.ay, b0, b1);
            unpack2(acc.az, c0, c1);
            unpack2(acc.phi, d0, d1);
            float phi = d0 + d1;
            if (selfSeen & (1u << lane)) {
                // the self term added to phi: -G m_i / sqrt(eps_i^2), exactly as evaluated
                phi -= (-kGPsuF * me.w) * rsqrtf(__fmul_rn(epsI, epsI));
            }
            float ax = a0 + a1, ay = b0 + b1, az = c0 + c1;
            if (kExpand) {                     // the group's far field at this member (farTaylor)
                const float* t = reinterpret_cast<const float*>(S.facc4);
                const float dx = xi - cxg, dy = yi - cyg, dz = zi - czg;
                const float jx = t[4] * dx + t[7] * dy + t[8] * dz;      // J d
                const float jy = t[7] * dx + t[5] * dy + t[9] * dz;
                const float jz = t[8] * dx + t[9] * dy + t[6] * dz;
                const float xx = dx * dx, yy = dy * dy, zz = dz * dz, xy = dx * dy, xz = dx * dz, yz = dy * dz;
                const float hx = t[10] * xx + t[15] * yy + t[17] * zz + 2.0f * (t[13] * xy + t[14] * xz + t[19] * yz);
                const float hy = t[13] * xx + t[11] * yy + t[18] * zz + 2.0f * (t[15] * xy + t[19] * xz + t[16] * yz);
                const float hz = t[14] * xx + t[16] * yy + t[12] * zz + 2.0f * (t[19] * xy + t[17] * xz + t[18] * yz);
                ax += t[1] + jx + 0.5f * hx;
                ay += t[2] + jy + 0.5f * hy;
                az += t[3] + jz + 0.5f * hz;
                phi += t[0] - (t[1] * dx + t[2] * dy + t[3] * dz) - 0.5f * (jx * dx + jy * dy + jz * dz);
            }
            p.accX[i] = ax;
            p.accY[i] = ay;
            p.accZ[i] = az;
            p.phiGrav[i] = phi;
        }
        nRounds += rounds;
        nInter += static_cast<unsigned long long>(act) * static_cast<unsigned>(mCount + pCount);
        if (lane == 0) {
            nInter -= static_cast<unsigned long long>(__popc(selfSeen));
            if (kDebug && w.groupCounts != nullptr) w.groupCounts[g] = static_cast<uint32_t>(nInter - interBefore);
        }
        __syncwarp();
    }
    if (lane == 0) {
        DevStatus* st = reinterpret_cast<DevStatus*>(w.status);
        atomicAdd(&st->counters[kCntGravityInteractions], nInter);
        atomicAdd(&st->counters[kCntGravityNodeTests], nTests);
        atomicAdd(&st->counters[kCntGravityUndecided], nUndecided);
        if (kExpand) {
            atomicAdd(&st->counters[kCntGravityGroupEvals], nGroupEvals);
            atomicAdd(&st->counters[kCntGravityBucketLeaves], nBucketLeaves);
        }
        atomicAdd(&st->counters[kCntGravityRounds], nRounds);
        atomicMax(&st->counters[kCntGravityStackPeak], static_cast<unsigned long long>(spPeak));
        if (overflowed) atomicOr(&st->flags, kFlagStackOverflow);
    }
}

}  // namespace

cudaError_t launchGravity(const AstraeaParticles& p, const Work& w, uint32_t n, float theta, bool quadrupole, int sms,
                          cudaStream_t st, const FarCapture* far, int warps, bool expansion) {
    if (n == 0) return cudaSuccess;
    const float th = fmaxf(0.0f, theta);
    const float theta2 = th * th;
    const bool checkInside = theta2 > 0.333333f;
    const uint32_t groups = (n + 31u) / 32u;
    uint32_t* counter = w.words + kWGroupCounter;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    FarCapture ff{};
    using GravFn = void (*)(AstraeaParticles, Work, uint32_t, float, uint32_t, uint32_t*, FarCapture);
    GravFn kernel = nullptr;
    int wps = kGravWarps;
    if (w.traceList != nullptr || w.groupCounts != nullptr) {
        // the debugging calls (monopole walk, 4-warp blocks)
        kernel = checkInside ? gravityKernel<kGravWarps, true, false, false, false, true>
                             : gravityKernel<kGravWarps, false, false, false, false, true>;
    } else if (expansion && quadrupole && far == nullptr) {
        if (warps == 2) {
            kernel = checkInside ? gravityKernel<2, true, true, false, true> : gravityKernel<2, false, true, false, true>;
            wps = 2;
        } else {
            kernel = checkInside ? gravityKernel<kGravWarps, true, true, false, true>
                                 : gravityKernel<kGravWarps, false, true, false, true>;
        }
    } else if (far != nullptr) {
        ff = *far;
        if (ff.groupStride == 0u) ff.groupStride = 1u;
        kernel = checkInside ? gravityKernel<kGravWarps, true, false, true> : gravityKernel<kGravWarps, false, false, true>;
    } else if (quadrupole && warps == 2) {
        kernel = checkInside ? gravityKernel<2, true, true, false> : gravityKernel<2, false, true, false>;
        wps = 2;
    } else if (quadrupole && warps == 8) {
        kernel = checkInside ? gravityKernel<8, true, true, false> : gravityKernel<8, false, true, false>;
        wps = 8;
    } else if (quadrupole) {
        kernel = checkInside ? gravityKernel<kGravWarps, true, true, false> : gravityKernel<kGravWarps, false, true, false>;
    } else if (warps == 2) {
        kernel = checkInside ? gravityKernel<2, true, false, false> : gravityKernel<2, false, false, false>;
        wps = 2;
    } else if (warps == 8) {
        kernel = checkInside ? gravityKernel<8, true, false, false> : gravityKernel<8, false, false, false>;
        wps = 8;
    } else {
        kernel = checkInside ? gravityKernel<kGravWarps, true, false, false> : gravityKernel<kGravWarps, false, false, false>;
    }
    int perSm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, wps * 32, 0);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = std::min<uint32_t>(static_cast<uint32_t>(std::max(1, perSm) * sms),
                                               (groups + wps - 1) / wps);
    kernel<<<blocks, wps * 32, 0, st>>>(p, w, n, theta2, groups, counter, ff);
    return cudaGetLastError();
}

}  // namespace astraea_gb300
