// ff.cu -- far-field mode 2: a learned correction of the Barnes-Hut
// monopole that lets the walk accept far nodes at a larger opening angle.
//
// The gravity walk (gravity.cu, kLearned) takes a node that the theta test
// opens when every member of the group passes theta_far (by the sound
// distance bound) and the node is far against the group's size
// (L1 extent <= gamma r).  It records the (group, node) pair.  For each pair
// a small MLP predicts, from the node's features seen from the group centre
// c, the residual between the node's exact field and its monopole at c and
// the residual's Jacobian there; every member i then adds
// sum_pairs [R + J (x_i - c)] to its acceleration.
//
// Features (16): u = (COM - c)/r (3), dNode/r, S/(M dNode^2) (the node's
// central second moments, 6), L1 group extent / r, and five zeros.
// Outputs (16, 12 used): R r^2/(G M) (3) and J r^3/(G M) (row-major 3x3),
// each divided by a per-output scale fitted to the training labels.
// Network: 16 -> 64 -> 64 -> 16, SiLU, BF16 operands with FP32
// accumulation on the tensor cores (mma.sync m16n8k16), FP32 master weights
// trained with Adam.  Labels are FP64 direct sums over the node's particles
// (Karras nodes cover contiguous sorted ranges), made from the solver's own
// trees.  A gate compares the corrected accelerations of sampled particles
// with an FP32 direct sum.
#include <algorithm>

#include <cuda_bf16.h>

#include "kernels.h"

namespace astraea_gb300 {
namespace ff {

namespace {

using bf16 = __nv_bfloat16;
constexpr float kG = 66.7430f;
constexpr double kGd = 66.7430;

// ------------------------------------------------------------ features --
__device__ __forceinline__ float4 nodeRec(const Work& w, uint32_t c, int k) {
    return __ldg(&w.node[4 * static_cast<size_t>(c) + k]);
}

// Features of node c seen from the group record grp {centre, L1 extent};
// also returns r and the node mass.
__device__ void pairFeatures(const Work& w, uint32_t c, float4 grp, float* f, float* rOut, float* mOut) {
    const float4 r0 = nodeRec(w, c, 0);               // {COM, mass}
    const float dd = nodeRec(w, c, 1).x;              // dNode^2
    const float4 s0 = __ldg(&w.nodeQuad[2 * static_cast<size_t>(c)]);
    const float4 s1 = __ldg(&w.nodeQuad[2 * static_cast<size_t>(c) + 1]);
    const float ux = r0.x - grp.x, uy = r0.y - grp.y, uz = r0.z - grp.z;
    const float r = sqrtf(ux * ux + uy * uy + uz * uz);
    const float inv = (r > 0.0f) ? 1.0f / r : 0.0f;
    const float sN = (r0.w > 0.0f && dd > 0.0f) ? 1.0f / (r0.w * dd) : 0.0f;
    f[0] = ux * inv; f[1] = uy * inv; f[2] = uz * inv;
    f[3] = sqrtf(dd) * inv;
    f[4] = s0.x * sN; f[5] = s0.y * sN; f[6] = s0.z * sN;
    f[7] = s0.w * sN; f[8] = s1.x * sN; f[9] = s1.y * sN;
    f[10] = grp.w * inv;
    f[11] = 0.0f; f[12] = 0.0f; f[13] = 0.0f; f[14] = 0.0f; f[15] = 0.0f;
    *rOut = r;
    *mOut = r0.w;
}

// ------------------------------------------------------- warp-level GEMM --
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum class Store { Set, AtomicAdd };

// C[M x N] (row-major, FP32) = or += opA(A)[M x K] opB(B)[K x N], operands
// BF16 in shared memory; M, K multiples of 16, N a multiple of 8.  Element
// (m, k) of A is A[k lda + m] when kTA, else A[m lda + k]; element (k, n)
// of B is B[n ldb + k] when kTB, else B[k ldb + n].  Fragments follow the
// m16n8k16 layout: lane = 4 g + t holds A(g [+8], 2t [+1] [+8]),
// B(2t [+1] [+8], g) and C(g [+8], 2t [+1]).
template <bool kTA, bool kTB, Store kS>
__device__ void warpGemm(const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc, int M, int N, int K) {
    const int lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
    auto ea = [&](int m, int k) -> uint32_t {
        return __bfloat16_as_ushort(kTA ? A[k * lda + m] : A[m * lda + k]);
    };
    auto eb = [&](int k, int n) -> uint32_t {
        return __bfloat16_as_ushort(kTB ? B[n * ldb + k] : B[k * ldb + n]);
    };
    for (int mt = 0; mt < M; mt += 16) {
        for (int nt = 0; nt < N; nt += 8) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            const int m0 = mt + gq, n0 = nt + gq;
            for (int kt = 0; kt < K; kt += 16) {
                const int k0 = kt + 2 * t4;
                const uint32_t a[4] = {ea(m0, k0) | (ea(m0, k0 + 1) << 16), ea(m0 + 8, k0) | (ea(m0 + 8, k0 + 1) << 16),
                                       ea(m0, k0 + 8) | (ea(m0, k0 + 9) << 16),
                                       ea(m0 + 8, k0 + 8) | (ea(m0 + 8, k0 + 9) << 16)};
                const uint32_t b[2] = {eb(k0, n0) | (eb(k0 + 1, n0) << 16), eb(k0 + 8, n0) | (eb(k0 + 9, n0) << 16)};
                mma16816(c, a, b);
            }
            float* d0 = C + (mt + gq) * ldc + nt + 2 * t4;
            float* d1 = d0 + 8 * ldc;
            if (kS == Store::Set) {
                d0[0] = c[0]; d0[1] = c[1]; d1[0] = c[2]; d1[1] = c[3];
            } else {
                atomicAdd(d0, c[0]); atomicAdd(d0 + 1, c[1]); atomicAdd(d1, c[2]); atomicAdd(d1 + 1, c[3]);
            }
        }
    }
}

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

// ------------------------------------------------------ shared layouts --
constexpr int kWarps = 4;
// weights (BF16) and biases (FP32) of one block
struct WeightsSmem {
    bf16 w1[kIn * kHid];
    bf16 w2[kHid * kHid];
    bf16 w3[kHid * kOut];
    float b1[kHid], b2[kHid], b3[kOut];
    float scale[kOut];
};
// per-warp forward buffers (16 rows)
struct FwdSmem {
    bf16 x[16 * kIn];
    bf16 h1[16 * kHid];
    bf16 h2[16 * kHid];
    float z1[16 * kHid];
    float z2[16 * kHid];
    float y[16 * kOut];
};
// per-warp backward buffers
struct BwdSmem {
    bf16 dy[16 * kOut];
    bf16 dz2[16 * kHid];
    bf16 dz1[16 * kHid];
    float dh[16 * kHid];
};

__device__ void loadWeights(WeightsSmem& W, const float* params, const float* scale) {
    for (int e = threadIdx.x; e < kIn * kHid; e += blockDim.x) W.w1[e] = __float2bfloat16_rn(params[kW1 + e]);
    for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) W.w2[e] = __float2bfloat16_rn(params[kW2 + e]);
    for (int e = threadIdx.x; e < kHid * kOut; e += blockDim.x) W.w3[e] = __float2bfloat16_rn(params[kW3 + e]);
    for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
        W.b1[e] = params[kB1 + e];
        W.b2[e] = params[kB2 + e];
    }
    for (int e = threadIdx.x; e < kOut; e += blockDim.x) {
        W.b3[e] = params[kB3 + e];
        W.scale[e] = (scale != nullptr) ? scale[e] : 1.0f;
    }
}

// Forward pass of the 16 rows staged in F.x; leaves y = network output.
__device__ void forward16(const WeightsSmem& W, FwdSmem& F) {
    const int lane = threadIdx.x & 31;
    warpGemm<false, false, Store::Set>(F.x, kIn, W.w1, kHid, F.z1, kHid, 16, kHid, kIn);
    __syncwarp();
    for (int e = lane; e < 16 * kHid; e += 32) {
        const float z = F.z1[e] + W.b1[e % kHid];
        F.z1[e] = z;
        F.h1[e] = __float2bfloat16_rn(z * sigm(z));
    }
    __syncwarp();
    warpGemm<false, false, Store::Set>(F.h1, kHid, W.w2, kHid, F.z2, kHid, 16, kHid, kHid);
    __syncwarp();
    for (int e = lane; e < 16 * kHid; e += 32) {
        const float z = F.z2[e] + W.b2[e % kHid];
        F.z2[e] = z;
        F.h2[e] = __float2bfloat16_rn(z * sigm(z));
    }
    __syncwarp();
    warpGemm<false, false, Store::Set>(F.h2, kHid, W.w3, kOut, F.y, kOut, 16, kOut, kHid);
    __syncwarp();
    for (int e = lane; e < 16 * kOut; e += 32) F.y[e] += W.b3[e % kOut];
    __syncwarp();
}

// --------------------------------------------------------------- kernels --
// Training: loss = mean over rows and the 12 used outputs of
// (y - label/scale)^2; gradients summed into grads, loss into *loss.
__global__ void __launch_bounds__(kWarps * 32) trainKernel(const float* params, const float* scale, const float* feat,
                                                           const float* label, uint32_t count, float* grads,
                                                           float* loss) {
    extern __shared__ __align__(16) unsigned char smRaw[];
    WeightsSmem& W = *reinterpret_cast<WeightsSmem*>(smRaw);
    float* G = reinterpret_cast<float*>(smRaw + sizeof(WeightsSmem));
    unsigned char* warpBase = smRaw + sizeof(WeightsSmem) + sizeof(float) * kParams;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    FwdSmem& F = *reinterpret_cast<FwdSmem*>(warpBase + warp * (sizeof(FwdSmem) + sizeof(BwdSmem)));
    BwdSmem& B = *reinterpret_cast<BwdSmem*>(warpBase + warp * (sizeof(FwdSmem) + sizeof(BwdSmem)) + sizeof(FwdSmem));
    loadWeights(W, params, scale);
    for (int e = threadIdx.x; e < kParams; e += blockDim.x) G[e] = 0.0f;
    __syncthreads();
    const float norm = 2.0f / (static_cast<float>(count) * static_cast<float>(kUsedOut));
    float lossLocal = 0.0f;
    const uint32_t tiles = (count + 15u) / 16u;
    for (uint32_t t = blockIdx.x * kWarps + warp; t < tiles; t += gridDim.x * kWarps) {
        const uint32_t r0 = t * 16u;
        for (int e = lane; e < 16 * kIn; e += 32) {
            const uint32_t r = r0 + e / kIn;
            F.x[e] = __float2bfloat16_rn(r < count ? feat[static_cast<size_t>(r) * kIn + e % kIn] : 0.0f);
        }
        __syncwarp();
        forward16(W, F);
        for (int e = lane; e < 16 * kOut; e += 32) {
            const uint32_t r = r0 + e / kOut;
            const int o = e % kOut;
            float d = 0.0f;
            if (r < count && o < kUsedOut) d = F.y[e] - label[static_cast<size_t>(r) * kOut + o] / W.scale[o];
            lossLocal += d * d;
            const float g = norm * d;
            B.dy[e] = __float2bfloat16_rn(g);
            atomicAdd(&G[kB3 + o], g);
        }
        __syncwarp();
        warpGemm<true, false, Store::AtomicAdd>(F.h2, kHid, B.dy, kOut, G + kW3, kOut, kHid, kOut, 16);
        warpGemm<false, true, Store::Set>(B.dy, kOut, W.w3, kOut, B.dh, kHid, 16, kHid, kOut);
        __syncwarp();
        for (int e = lane; e < 16 * kHid; e += 32) {
            const float z = F.z2[e], s = sigm(z);
            const float g = B.dh[e] * (s * (1.0f + z * (1.0f - s)));
            B.dz2[e] = __float2bfloat16_rn(g);
            atomicAdd(&G[kB2 + e % kHid], g);
        }
        __syncwarp();
        warpGemm<true, false, Store::AtomicAdd>(F.h1, kHid, B.dz2, kHid, G + kW2, kHid, kHid, kHid, 16);
        warpGemm<false, true, Store::Set>(B.dz2, kHid, W.w2, kHid, B.dh, kHid, 16, kHid, kHid);
        __syncwarp();
        for (int e = lane; e < 16 * kHid; e += 32) {
            const float z = F.z1[e], s = sigm(z);
            const float g = B.dh[e] * (s * (1.0f + z * (1.0f - s)));
            B.dz1[e] = __float2bfloat16_rn(g);
            atomicAdd(&G[kB1 + e % kHid], g);
        }
        __syncwarp();
        warpGemm<true, false, Store::AtomicAdd>(F.x, kIn, B.dz1, kHid, G + kW1, kHid, kIn, kHid, 16);
        __syncwarp();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kParams; e += blockDim.x) atomicAdd(&grads[e], G[e]);
    for (int o = 16; o > 0; o >>= 1) lossLocal += __shfl_xor_sync(0xffffffffu, lossLocal, o);
    if (lane == 0) atomicAdd(loss, lossLocal / (static_cast<float>(count) * static_cast<float>(kUsedOut)));
}

__global__ void adamKernel(float* params, float* grads, float* m, float* v, float lr, float c1, float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kParams) return;
    const float g = grads[e];
    const float mm = 0.9f * m[e] + 0.1f * g;
    const float vv = 0.999f * v[e] + 0.001f * g * g;
    m[e] = mm;
    v[e] = vv;
    params[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1.0e-8f);
    grads[e] = 0.0f;
}

// Network outputs (normalised units) for rows of features.
__global__ void __launch_bounds__(kWarps * 32) predictKernel(const float* params, const float* feat, uint32_t count,
                                                             float* out) {
    extern __shared__ __align__(16) unsigned char smRaw[];
    WeightsSmem& W = *reinterpret_cast<WeightsSmem*>(smRaw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    FwdSmem& F = *reinterpret_cast<FwdSmem*>(smRaw + sizeof(WeightsSmem) + warp * sizeof(FwdSmem));
    loadWeights(W, params, nullptr);
    __syncthreads();
    const uint32_t tiles = (count + 15u) / 16u;
    for (uint32_t t = blockIdx.x * kWarps + warp; t < tiles; t += gridDim.x * kWarps) {
        const uint32_t r0 = t * 16u;
        for (int e = lane; e < 16 * kIn; e += 32) {
            const uint32_t r = r0 + e / kIn;
            F.x[e] = __float2bfloat16_rn(r < count ? feat[static_cast<size_t>(r) * kIn + e % kIn] : 0.0f);
        }
        __syncwarp();
        forward16(W, F);
        for (int e = lane; e < 16 * kOut; e += 32) {
            const uint32_t r = r0 + e / kOut;
            if (r < count) out[static_cast<size_t>(r) * kOut + e % kOut] = F.y[e];
        }
        __syncwarp();
    }
}

// Inference on the walk's pairs: features, network, and the physical
// residual and Jacobian summed into the group's 12 correction words.
__global__ void __launch_bounds__(kWarps * 32) applyKernel(const float* params, const float* scale, Work w,
                                                           const uint2* pairs, const uint32_t* countWord,
                                                           uint32_t cap, const float4* groups, float* groupCorr) {
    extern __shared__ __align__(16) unsigned char smRaw[];
    WeightsSmem& W = *reinterpret_cast<WeightsSmem*>(smRaw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wb = smRaw + sizeof(WeightsSmem) + warp * (sizeof(FwdSmem) + 16 * 4 * sizeof(float));
    FwdSmem& F = *reinterpret_cast<FwdSmem*>(wb);
    float* meta = reinterpret_cast<float*>(wb + sizeof(FwdSmem));   // per row: group, GM/r^2, GM/r^3, valid
    loadWeights(W, params, scale);
    __syncthreads();
    const uint32_t count = min(*countWord, cap);
    const uint32_t tiles = (count + 15u) / 16u;
    for (uint32_t t = blockIdx.x * kWarps + warp; t < tiles; t += gridDim.x * kWarps) {
        const uint32_t r = t * 16u + static_cast<uint32_t>(lane);
        if (lane < 16) {
            float f[16];
            float rr = 0.0f, mm = 0.0f;
            uint32_t g = 0;
            const bool valid = r < count;
            if (valid) {
                const uint2 pr = pairs[r];
                g = pr.x;
                pairFeatures(w, pr.y, groups[pr.x], f, &rr, &mm);
            } else {
                for (int k = 0; k < 16; ++k) f[k] = 0.0f;
            }
            for (int k = 0; k < kIn; ++k) F.x[lane * kIn + k] = __float2bfloat16_rn(f[k]);
            const float s2 = (valid && rr > 0.0f) ? kG * mm / (rr * rr) : 0.0f;
            meta[4 * lane + 0] = __uint_as_float(g);
            meta[4 * lane + 1] = s2;
            meta[4 * lane + 2] = (rr > 0.0f) ? s2 / rr : 0.0f;
            meta[4 * lane + 3] = valid ? 1.0f : 0.0f;
        }
        __syncwarp();
        forward16(W, F);
        if (lane < 16 && meta[4 * lane + 3] != 0.0f) {
            const uint32_t g = __float_as_uint(meta[4 * lane + 0]);
            const float s2 = meta[4 * lane + 1], s3 = meta[4 * lane + 2];
            float* dst = groupCorr + 12 * static_cast<size_t>(g);
            for (int o = 0; o < kUsedOut; ++o) atomicAdd(&dst[o], F.y[lane * kOut + o] * W.scale[o] * (o < 3 ? s2 : s3));
        }
        __syncwarp();
    }
}

// a_i += R + J (x_i - c) of the particle's group (groups of 32 sorted
// particles, as the walk forms them).
__global__ void correctKernel(AstraeaParticles p, const float4* groups, const float* groupCorr, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t g = i >> 5;
    const float4 c = groups[g];
    const float* q = groupCorr + 12 * static_cast<size_t>(g);
    const float dx = p.posX[i] - c.x, dy = p.posY[i] - c.y, dz = p.posZ[i] - c.z;
    p.accX[i] += q[0] + q[3] * dx + q[4] * dy + q[5] * dz;
    p.accY[i] += q[1] + q[6] * dx + q[7] * dy + q[8] * dz;
    p.accZ[i] += q[2] + q[9] * dx + q[10] * dy + q[11] * dz;
}

// Training rows: features and FP64 labels of each pair, one warp per pair.
// The node's particles are the sorted range between its leftmost and
// rightmost leaves; the label is the exact field of that range at the group
// centre minus the node's monopole, and the Jacobian of that difference.
constexpr int kLabelWarps = 8;
__global__ void __launch_bounds__(kLabelWarps * 32) labelKernel(Work w, uint32_t n, const uint2* pairs,
                                                                uint32_t count, const float4* groups, float* feat,
                                                                float* label) {
    const uint32_t pIdx = blockIdx.x * kLabelWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (pIdx >= count) return;
    const uint2 pr = pairs[pIdx];
    const uint32_t c = pr.y;
    const float4 grp = groups[pr.x];
    // leftmost / rightmost leaf (bounded descent)
    int lo = static_cast<int>(c), hi = static_cast<int>(c);
    for (int s = 0; s < 4096 && lo >= 0; ++s) lo = __float_as_int(nodeRec(w, static_cast<uint32_t>(lo), 1).y);
    for (int s = 0; s < 4096 && hi >= 0; ++s) hi = __float_as_int(nodeRec(w, static_cast<uint32_t>(hi), 1).z);
    const bool ok = lo < 0 && hi < 0;
    const uint32_t first = ok ? static_cast<uint32_t>(~lo) : 1u, last = ok ? static_cast<uint32_t>(~hi) : 0u;
    const double cx = grp.x, cy = grp.y, cz = grp.z;
    double a[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t j = first + static_cast<uint32_t>(lane); j <= last && j < n; j += 32u) {
        const float4 pa = __ldg(&w.leaf[j].a);
        const float4 pm = make_float4(pa.x, pa.y, pa.z, __ldg(&w.leafAux[j]).w);
        const double dx = cx - pm.x, dy = cy - pm.y, dz = cz - pm.z;
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 > 0.0)) continue;
        const double ir = 1.0 / sqrt(r2), ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
        const double gm = kGd * pm.w;
        const double d[3] = {dx, dy, dz};
        for (int k = 0; k < 3; ++k) a[k] -= gm * d[k] * ir3;
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) a[3 + 3 * r + k] -= gm * (((r == k) ? ir3 : 0.0) - 3.0 * d[r] * d[k] * ir5);
    }
    for (int k = 0; k < 12; ++k)
        for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
    if (lane != 0) return;
    float f[16], rr = 0.0f, mm = 0.0f;
    pairFeatures(w, c, grp, f, &rr, &mm);
    const float4 r0 = nodeRec(w, c, 0);
    const double dx = cx - r0.x, dy = cy - r0.y, dz = cz - r0.z;
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double ir = 1.0 / sqrt(r2), ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
    const double gm = kGd * r0.w;
    const double d[3] = {dx, dy, dz};
    double res[12];
    for (int k = 0; k < 3; ++k) res[k] = a[k] + gm * d[k] * ir3;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) res[3 + 3 * r + k] = a[3 + 3 * r + k] + gm * (((r == k) ? ir3 : 0.0) - 3.0 * d[r] * d[k] * ir5);
    const double rad = sqrt(r2), s2 = (gm > 0.0) ? r2 / gm : 0.0, s3 = s2 * rad;
    float* fo = feat + static_cast<size_t>(pIdx) * kIn;
    float* lo2 = label + static_cast<size_t>(pIdx) * kOut;
    for (int k = 0; k < kIn; ++k) fo[k] = ok ? f[k] : 0.0f;
    for (int k = 0; k < kOut; ++k) lo2[k] = (ok && k < kUsedOut) ? static_cast<float>(res[k] * (k < 3 ? s2 : s3)) : 0.0f;
}

// The gate's spot check: target k is the k-th of K evenly spaced sorted
// particles.  Block (s, k) sums the softened pull (eps_ij softening, as the
// walk's leaves) of sorted particles [s kGateSlice, (s+1) kGateSlice) on
// target k and adds it to gate->acc[3k..3k+2]; K n pair terms spread over
// every SM.  kF64: pair terms in FP64 (positions widened before the
// subtraction), the spot check against an FP64 direct sum.  Otherwise FP32
// pair terms, each thread's run of kGateRun terms in FP32 and everything
// above in FP64: within ~1e-6 relative of the FP64 sum, three orders below any
// useful tolerance, at a fraction of the cost (FP64 issues at a small
// fraction of the FP32 rate on this part).
constexpr int kGateThreads = 256;
constexpr int kGateRun = 16;
constexpr uint32_t kGateSlice = kGateThreads * kGateRun;

__device__ __forceinline__ uint32_t gateTarget(uint32_t k, uint32_t n, uint32_t K) {
    return (K > 1u) ? static_cast<uint32_t>((static_cast<uint64_t>(k) * (n - 1u)) / (K - 1u)) : 0u;
}

template <bool kF64>
__global__ void __launch_bounds__(kGateThreads) gateSumKernel(Work w, uint32_t n, uint32_t K, GateDev* gate) {
    __shared__ double red[3][kGateThreads / 32];
    const uint32_t k = blockIdx.y;
    const uint32_t t = gateTarget(k, n, K);
    const float4 me = __ldg(&w.leaf[t].a);
    const float ei = __ldg(&w.leafAux[t]).y;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    const uint32_t j0 = blockIdx.x * kGateSlice + threadIdx.x;
    if constexpr (kF64) {
        const double xi = me.x, yi = me.y, zi = me.z, hei = 0.5 * static_cast<double>(ei);
#pragma unroll 4
        for (int r = 0; r < kGateRun; ++r) {
            const uint32_t j = j0 + static_cast<uint32_t>(r) * kGateThreads;
            if (j >= n || j == t) continue;
            const float4 pa = __ldg(&w.leaf[j].a);
            const float4 aux = __ldg(&w.leafAux[j]);
            const float4 pm = make_float4(pa.x, pa.y, pa.z, aux.w);
            const double e = hei + 0.5 * static_cast<double>(aux.y);
            const double dx = xi - pm.x, dy = yi - pm.y, dz = zi - pm.z;
            const double ir = rsqrt(dx * dx + dy * dy + dz * dz + e * e);
            const double f = -static_cast<double>(kG) * pm.w * ir * ir * ir;
            sx += f * dx; sy += f * dy; sz += f * dz;
        }
    } else {
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
#pragma unroll 4
        for (int r = 0; r < kGateRun; ++r) {
            const uint32_t j = j0 + static_cast<uint32_t>(r) * kGateThreads;
            if (j >= n || j == t) continue;
            const float4 pa = __ldg(&w.leaf[j].a);
            const float4 aux = __ldg(&w.leafAux[j]);
            const float4 pm = make_float4(pa.x, pa.y, pa.z, aux.w);
            const float e = 0.5f * (ei + aux.y);
            const float dx = me.x - pm.x, dy = me.y - pm.y, dz = me.z - pm.z;
            const float ir = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e * e))));
            const float f = -kG * pm.w * ir * ir * ir;
            ax = fmaf(f, dx, ax); ay = fmaf(f, dy, ay); az = fmaf(f, dz, az);
        }
        sx = ax; sy = ay; sz = az;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][warp] = sx; red[1][warp] = sy; red[2][warp] = sz; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int q = 0; q < kGateThreads / 32; ++q) v += red[threadIdx.x][q];
        atomicAdd(&gate->acc[3u * k + threadIdx.x], v);
    }
}

// The gate's decision, on the device: RMS over the K targets of
// |a - a_ref| / |a_ref| against the tolerance; runFallback = 1 makes the
// following plain walk run, 0 makes it return at once.  Also the statistics
// ff_stats reads, and the sums cleared for the next gate.
__global__ void __launch_bounds__(kGateMaxTargets) gateDecideKernel(AstraeaParticles p, uint32_t n, GateDev* gate,
                                                                    uint32_t K, float tolerance,
                                                                    const uint32_t* pairCount, uint32_t pairCap) {
    __shared__ double red[kGateMaxTargets / 32];
    double err = 0.0;
    if (threadIdx.x < K) {
        const uint32_t t = gateTarget(threadIdx.x, n, K);
        double* a = gate->acc + 3u * threadIdx.x;
        const double rx = a[0], ry = a[1], rz = a[2];
        const double ex = p.accX[t] - rx, ey = p.accY[t] - ry, ez = p.accZ[t] - rz;
        const double ref = rx * rx + ry * ry + rz * rz;
        if (ref > 0.0) err = (ex * ex + ey * ey + ez * ez) / ref;
        a[0] = a[1] = a[2] = 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) err += __shfl_xor_sync(0xffffffffu, err, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = err;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (uint32_t q = 0; q < blockDim.x / 32; ++q) sum += red[q];
        const double rms = sqrt(sum / static_cast<double>(K));
        const bool pass = rms <= static_cast<double>(tolerance);
        gate->runFallback = pass ? 0u : 1u;
        gate->lastRms = static_cast<float>(rms);
        gate->lastPairs = min(*pairCount, pairCap);
        if (!pass) gate->fallbacks += 1ull;
    }
}

inline unsigned blocks(size_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

size_t trainSmem() { return sizeof(WeightsSmem) + sizeof(float) * kParams + kWarps * (sizeof(FwdSmem) + sizeof(BwdSmem)); }
size_t predictSmem() { return sizeof(WeightsSmem) + kWarps * sizeof(FwdSmem); }
size_t applySmem() { return sizeof(WeightsSmem) + kWarps * (sizeof(FwdSmem) + 16 * 4 * sizeof(float)); }

cudaError_t allowSmem(const void* fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

}  // namespace

cudaError_t prepareKernels() {
    cudaError_t e = allowSmem(reinterpret_cast<const void*>(trainKernel), trainSmem());
    if (e == cudaSuccess) e = allowSmem(reinterpret_cast<const void*>(predictKernel), predictSmem());
    if (e == cudaSuccess) e = allowSmem(reinterpret_cast<const void*>(applyKernel), applySmem());
    return e;
}

cudaError_t launchLabels(const Work& w, uint32_t n, const uint2* pairs, uint32_t count, const float4* groups,
                         float* feat, float* label, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    labelKernel<<<blocks(count, kLabelWarps), kLabelWarps * 32, 0, st>>>(w, n, pairs, count, groups, feat, label);
    return cudaGetLastError();
}

cudaError_t launchTrain(const Net& net, const float* feat, const float* label, uint32_t count, int sms,
                        cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const unsigned tiles = blocks(count, 16);
    const unsigned grid = std::min<unsigned>(blocks(tiles, kWarps), static_cast<unsigned>(2 * sms));
    trainKernel<<<grid, kWarps * 32, trainSmem(), st>>>(net.params, net.outScale, feat, label, count, net.grads,
                                                        net.loss);
    return cudaGetLastError();
}

cudaError_t launchAdam(const Net& net, float lr, int step, cudaStream_t st) {
    const float c1 = 1.0f - powf(0.9f, static_cast<float>(step));
    const float c2 = 1.0f - powf(0.999f, static_cast<float>(step));
    adamKernel<<<blocks(kParams, 256), 256, 0, st>>>(net.params, net.grads, net.adamM, net.adamV, lr, c1, c2);
    return cudaGetLastError();
}

cudaError_t launchPredict(const Net& net, const float* feat, uint32_t count, float* out, int sms, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const unsigned grid = std::min<unsigned>(blocks(blocks(count, 16), kWarps), static_cast<unsigned>(2 * sms));
    predictKernel<<<grid, kWarps * 32, predictSmem(), st>>>(net.params, feat, count, out);
    return cudaGetLastError();
}

cudaError_t launchApply(const Net& net, const Work& w, const uint2* pairs, const uint32_t* countWord, uint32_t cap,
                        const float4* groups, float* groupCorr, int sms, cudaStream_t st) {
    applyKernel<<<static_cast<unsigned>(4 * sms), kWarps * 32, applySmem(), st>>>(net.params, net.outScale, w, pairs,
                                                                                   countWord, cap, groups, groupCorr);
    return cudaGetLastError();
}

cudaError_t launchCorrect(const AstraeaParticles& p, const float4* groups, const float* groupCorr, uint32_t n,
                          cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    correctKernel<<<blocks(n, 256), 256, 0, st>>>(p, groups, groupCorr, n);
    return cudaGetLastError();
}

cudaError_t launchGate(const AstraeaParticles& p, const Work& w, uint32_t n, uint32_t K, float tolerance,
                       const uint32_t* pairCount, uint32_t pairCap, GateDev* gate, bool fp32Pairs, cudaStream_t st) {
    if (n == 0u || K == 0u || K > kGateMaxTargets) return cudaErrorInvalidValue;
    const dim3 grid(blocks(n, kGateSlice), K);
    if (fp32Pairs)
        gateSumKernel<false><<<grid, kGateThreads, 0, st>>>(w, n, K, gate);
    else
        gateSumKernel<true><<<grid, kGateThreads, 0, st>>>(w, n, K, gate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const unsigned threads = ((K + 31u) / 32u) * 32u;
    gateDecideKernel<<<1, threads, 0, st>>>(p, n, gate, K, tolerance, pairCount, pairCap);
    return cudaGetLastError();
}

}  // namespace ff
}  // namespace astraea_gb300
