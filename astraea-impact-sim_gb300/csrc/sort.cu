// sort.cu -- onesweep LSD radix sort of (u64 key, u32 value) pairs for sm_103a.
//
// Replaces the cub::DeviceRadixSort::SortPairs call of
// engine/sph_gravity.cu:2028-2046 (stable, bits [0, 63), value = original
// index).  Design (Adinets & Merrill's single-pass "onesweep"):
//   * one up-front kernel builds the histograms of all 8-bit digits in one
//     read of the keys (and, for the Morton path, computes the 63-bit codes
//     from positions on the fly, engine/sph_gravity.cu:151-171 + 335-361);
//   * one kernel per digit: a tile of 4096 keys is ranked stably in shared
//     memory (warp match-any ranking in input order), the tile's bin counts
//     are published, the exclusive prefix over earlier tiles comes from a
//     decoupled look-back, and keys/values are scattered through a
//     shared-memory staging buffer so global writes stay coalesced per bin.
// Every look-back spin is bounded; a timeout sets a device status flag and
// the tile proceeds with the prefix gathered so far (an underestimate, so the
// tile's destinations stay inside its bin).  The result is then not sorted,
// and later passes see keys that no longer match the digit histograms, so
// every store is also checked against n.
#include <algorithm>
#include <atomic>

#include "internal.h"

namespace astraea_gb300 {
namespace {

constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

// Scratch layout: internal.h (sortScratchWordsFor).
constexpr size_t kHistWords = kSortHistWords;
constexpr size_t kCounterWords = kSortCounterWords;

__device__ __forceinline__ uint32_t lanemaskLt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t loadVolatile(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void storeRelaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// 63-bit Morton code of one position (engine/sph_gravity.cu:161-171, 347-359);
// the products and sums are separate IEEE operations, as in the reference.
__device__ __forceinline__ uint64_t mortonCode(float x, float y, float z, const float* b6, const float* inv3) {
    const float fx = fminf(fmaxf(__fmul_rn(__fsub_rn(x, b6[0]), inv3[0]), 0.0f), 2097151.0f);
    const float fy = fminf(fmaxf(__fmul_rn(__fsub_rn(y, b6[1]), inv3[1]), 0.0f), 2097151.0f);
    const float fz = fminf(fmaxf(__fmul_rn(__fsub_rn(z, b6[2]), inv3[2]), 0.0f), 2097151.0f);
    const uint64_t ix = static_cast<uint64_t>(static_cast<uint32_t>(fx));
    const uint64_t iy = static_cast<uint64_t>(static_cast<uint32_t>(fy));
    const uint64_t iz = static_cast<uint64_t>(static_cast<uint32_t>(fz));
    return (spreadBits21(ix) << 2) | (spreadBits21(iy) << 1) | spreadBits21(iz);
}

template <bool kMorton>
__global__ void __launch_bounds__(256) histogramKernel(const uint64_t* __restrict__ keysIn, MortonSource ms,
                                                       uint64_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                       uint32_t n, int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][kSortBins];
    __shared__ float sB[6];
    __shared__ float sInv[3];
    for (int t = threadIdx.x; t < kSortMaxPasses * kSortBins; t += blockDim.x) (&sh[0][0])[t] = 0u;
    if (kMorton && threadIdx.x == 0) {
        for (int k = 0; k < 6; ++k) sB[k] = floatFromOrdered(ms.boundsOrdered[k]);
        for (int k = 0; k < 3; ++k) {
            const float span = sB[3 + k] - sB[k];
            sInv[k] = (span > 1.0e-6f) ? (2097151.0f / span) : 0.0f;   // sph_gravity.cu:350-355
        }
        if (blockIdx.x == 0 && ms.boundsFloatOut != nullptr)
            for (int k = 0; k < 6; ++k) ms.boundsFloatOut[k] = sB[k];
    }
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t key;
        if (kMorton) {
            float x, y, z;
            if (ms.xyz != nullptr) {
                const float4 q = ms.xyz[i];
                x = q.x; y = q.y; z = q.z;
            } else {
                x = __ldg(&ms.x[i]); y = __ldg(&ms.y[i]); z = __ldg(&ms.z[i]);
            }
            key = mortonCode(x, y, z, sB, sInv);
            keysOut[i] = key;
            valsOut[i] = i;
        } else {
            key = keysIn[i];
        }
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(key >> (8 * p)) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < passes * kSortBins; t += blockDim.x) {
        const uint32_t c = (&sh[0][0])[t];
        if (c) atomicAdd(&hist[t], c);
    }
}

// Sum, for bin `bin`, the counts of tiles [0, tile) by walking back over the
// published status words until a tile that carries an inclusive prefix.  The
// walk reads four status words per step (independent loads, so one L2 round
// trip per four tiles instead of one per tile) and takes them in order: it
// stops at the first inclusive prefix, and at the first unpublished word it
// polls that word again.  Every poll of an unpublished word counts against
// spinLimit; on running out the walk stops (returns false) with the partial
// sum in *excl, which keeps the caller's destinations inside its bin.
constexpr int kLookbackWindow = 4;

__device__ __forceinline__ bool lookbackExclusive(const uint32_t* lookback, uint32_t tile, int bin,
                                                  uint32_t spinLimit, uint32_t* excl) {
    int64_t j = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0, sum = 0;
    while (j >= 0) {
        uint32_t v[kLookbackWindow];
#pragma unroll
        for (int q = 0; q < kLookbackWindow; ++q)   // before tile 0: an empty inclusive prefix
            v[q] = (j - q >= 0) ? loadVolatile(lookback + static_cast<size_t>(j - q) * kSortBins + bin) : kFlagPrefix;
        int used = 0;
        bool unpublished = false, prefix = false;
#pragma unroll
        for (int q = 0; q < kLookbackWindow; ++q) {
            if (unpublished || prefix) continue;
            const uint32_t flag = v[q] & ~kValueMask;
            if (flag == 0u) {
                unpublished = true;
            } else {
                sum += v[q] & kValueMask;
                ++used;
                prefix = (flag == kFlagPrefix);
            }
        }
        if (prefix) break;
        j -= used;
        if (unpublished) {
            if (spins >= spinLimit) { *excl = sum; return false; }
            ++spins;
            __nanosleep(32);
        }
    }
    *excl = sum;
    return true;
}

// Failure-detection probe: one thread runs the look-back wait on a status
// word that nothing publishes, so the wait must give up after spinLimit polls
// and report it through the status flags.
__global__ void lookbackProbeKernel(const uint32_t* neverSet, DevStatus* status, uint32_t spinLimit,
                                    uint32_t* result) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t excl = 0;
    const bool ok = lookbackExclusive(neverSet, 1u, 0, spinLimit, &excl);
    if (!ok) atomicOr(&status->flags, kFlagLookbackTimeout);
    *result = ok ? 1u : 2u;
}

struct SortSmem {
    uint64_t keys[kSortTile];
    uint32_t vals[kSortTile];
    uint32_t warpHist[kSortThreads / 32][kSortBins];
    uint32_t binStart[kSortBins];     // global exclusive offset of each bin (this pass)
    uint32_t tileExcl[kSortBins];     // exclusive offset of each bin inside this tile
    uint32_t globalBase[kSortBins];   // destination = globalBase[bin] + tile-local slot
    uint32_t scanTmp[kSortBins];
    uint32_t tile;
    uint32_t count;
};

// Block-wide exclusive scan of 256 values (one per thread, blockDim == 256).
__device__ __forceinline__ uint32_t blockExclusiveScan256(uint32_t v, uint32_t* tmp) {
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) tmp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < 8) ? tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < 8) tmp[lane] = w;   // inclusive warp totals
    }
    __syncthreads();
    const uint32_t warpOff = (warp > 0) ? tmp[warp - 1] : 0u;
    __syncthreads();
    return warpOff + incl - v;
}

__global__ void __launch_bounds__(kSortThreads) onesweepKernel(const uint64_t* __restrict__ keysIn,
                                                               const uint32_t* __restrict__ valsIn,
                                                               uint64_t* __restrict__ keysOut,
                                                               uint32_t* __restrict__ valsOut, uint32_t n, int pass,
                                                               const uint32_t* __restrict__ hist,
                                                               uint32_t* __restrict__ tileCounter,
                                                               uint32_t* __restrict__ lookback, DevStatus* status,
                                                               uint32_t spinLimit) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    SortSmem& s = *reinterpret_cast<SortSmem*>(smemRaw);
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int shift = 8 * pass;

    // Global start of every bin for this pass (exclusive scan of the histogram).
    const uint32_t binCount = hist[pass * kSortBins + t];
    const uint32_t binStart = blockExclusiveScan256(binCount, s.scanTmp);
    s.binStart[t] = binStart;
    for (int w = 0; w < kSortThreads / 32; ++w) s.warpHist[w][t] = 0u;
    if (t == 0) s.tile = atomicAdd(tileCounter, 1u);
    __syncthreads();
    const uint32_t tile = s.tile;
    const uint32_t tileBase = tile * static_cast<uint32_t>(kSortTile);
    const uint32_t warpBase = tileBase + static_cast<uint32_t>(warp) * (kSortItems * 32);

    // Load (warp-striped: item k of lane l is element warpBase + 32k + l) and
    // rank stably inside the warp: items are visited in (k, lane) order, which
    // is input order.
    uint64_t key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
    uint32_t digit[kSortItems];
    uint32_t* wh = s.warpHist[warp];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t idx = warpBase + static_cast<uint32_t>(k * 32 + lane);
        const bool ok = idx < n;
        key[k] = ok ? keysIn[idx] : 0ull;
        val[k] = ok ? valsIn[idx] : 0u;
        digit[k] = ok ? static_cast<uint32_t>((key[k] >> shift) & 0xFFu) : 0x100u;
    }
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t d = digit[k];
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const bool ok = d < 0x100u;
        const uint32_t before = ok ? wh[d] : 0u;
        __syncwarp();
        rank[k] = before + __popc(peers & lanemaskLt());
        const int leader = __ffs(peers) - 1;
        if (ok && lane == leader) wh[d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // Per-bin tile totals and per-warp exclusive offsets (thread t owns bin t).
    uint32_t total = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) {
        const uint32_t c = s.warpHist[w][t];
        s.warpHist[w][t] = total;
        total += c;
    }
    // Publish this tile's aggregate as early as possible.
    uint32_t* myStatus = lookback + static_cast<size_t>(tile) * kSortBins + t;
    storeRelaxed(myStatus, (tile == 0 ? kFlagPrefix : kFlagAggregate) | total);
    const uint32_t tileExcl = blockExclusiveScan256(total, s.scanTmp);
    s.tileExcl[t] = tileExcl;

    // Decoupled look-back over earlier tiles for bin t.
    uint32_t excl = 0;
    if (tile > 0) {
        if (!lookbackExclusive(lookback, tile, t, spinLimit, &excl)) atomicOr(&status->flags, kFlagLookbackTimeout);
        storeRelaxed(myStatus, kFlagPrefix | ((excl + total) & kValueMask));
    }
    s.globalBase[t] = s.binStart[t] + excl - tileExcl;
    __syncthreads();

    // Stage into shared memory in bin order, then write out coalesced.
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t d = digit[k];
        if (d < 0x100u) {
            const uint32_t slot = s.tileExcl[d] + s.warpHist[warp][d] + rank[k];
            s.keys[slot] = key[k];
            s.vals[slot] = val[k];
        }
    }
    __syncthreads();
    const uint32_t tileCount = (tileBase < n) ? min(static_cast<uint32_t>(kSortTile), n - tileBase) : 0u;
    for (uint32_t slot = t; slot < tileCount; slot += kSortThreads) {
        const uint64_t kk = s.keys[slot];
        const uint32_t d = static_cast<uint32_t>((kk >> shift) & 0xFFu);
        const uint32_t dst = s.globalBase[d] + slot;
        // Always true for a consistent input.  After a look-back timeout in an
        // earlier pass the keys are no longer a permutation of the histogram's,
        // and a bin can overflow its range: the check keeps the writes in [0, n).
        if (dst < n) {
            keysOut[dst] = kk;
            valsOut[dst] = s.vals[slot];
        }
    }
}

}  // namespace

cudaError_t launchLookbackProbe(const uint32_t* neverSet, DevStatus* status, uint32_t spinLimit, uint32_t* result,
                                cudaStream_t stream) {
    lookbackProbeKernel<<<1, 32, 0, stream>>>(neverSet, status, spinLimit, result);
    return cudaGetLastError();
}

size_t sortScratchWords(uint32_t n, uint32_t* maxTilesOut) {
    if (maxTilesOut) *maxTilesOut = sortTiles(n);
    return sortScratchWordsFor(n);
}

cudaError_t radixSortPairs(uint64_t* keysA, uint32_t* valsA, uint64_t* keysB, uint32_t* valsB, uint32_t n,
                           int endBit, uint32_t* scratch, size_t scratchWords, uint32_t maxTiles, DevStatus* status,
                           uint32_t spinLimit, KeySource src, const MortonSource* morton, bool* resultInA,
                           cudaStream_t stream) {
    *resultInA = true;
    if (n == 0) return cudaSuccess;
    const int passes = std::max(1, std::min(kSortMaxPasses, (endBit + 7) / 8));
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    if (tiles > maxTiles || n > kValueMask) return cudaErrorInvalidValue;
    const size_t need = kHistWords + kCounterWords + static_cast<size_t>(passes) * tiles * kSortBins;
    if (need > scratchWords) return cudaErrorInvalidValue;
    uint32_t* hist = scratch;
    uint32_t* counters = scratch + kHistWords;
    uint32_t* look = counters + kCounterWords;
    cudaError_t e = cudaMemsetAsync(scratch, 0, need * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;

    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int hBlocks = static_cast<int>(std::min<uint32_t>((n + 255) / 256, static_cast<uint32_t>(sms) * 4u));
    if (src == KeySource::MortonFromPositions) {
        histogramKernel<true><<<hBlocks, 256, 0, stream>>>(nullptr, *morton, keysA, valsA, n, passes, hist);
    } else {
        MortonSource none{};
        histogramKernel<false><<<hBlocks, 256, 0, stream>>>(keysA, none, nullptr, nullptr, n, passes, hist);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;

    const size_t smem = sizeof(SortSmem);
    // The shared-memory attribute is set once per device; host threads that
    // sort on the same device at once may both set it (the same value), and
    // the flag is atomic, so neither reads it torn.
    static std::atomic<bool> attrSet[64] = {};
    if (dev < 0 || dev >= 64 || !attrSet[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(onesweepKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attrSet[dev].store(true, std::memory_order_release);
    }
    uint64_t* kin = keysA;
    uint32_t* vin = valsA;
    uint64_t* kout = keysB;
    uint32_t* vout = valsB;
    for (int p = 0; p < passes; ++p) {
        onesweepKernel<<<tiles, kSortThreads, smem, stream>>>(kin, vin, kout, vout, n, p, hist, counters + p,
                                                              look + static_cast<size_t>(p) * tiles * kSortBins,
                                                              status, spinLimit);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    *resultInA = (kin == keysA);
    return cudaSuccess;
}

}  // namespace astraea_gb300
