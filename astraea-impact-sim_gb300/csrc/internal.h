// internal.h -- host-side launchers shared between the library's translation
// units.  Not part of the public C-ABI (include/astraea_gb300.h).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "astraea_gb300.h"
#include "common.cuh"

namespace astraea_gb300 {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per tile
constexpr int kSortBins = 256;
constexpr int kSortMaxPasses = 8;

// Onesweep scratch layout (32-bit words):
//   [0, kSortHistWords)                              digit histograms, one per pass
//   [kSortHistWords, + kSortCounterWords)            tile counters, one per pass
//   then kSortMaxPasses * tiles * kSortBins          look-back status words
constexpr size_t kSortHistWords = static_cast<size_t>(kSortMaxPasses) * kSortBins;
constexpr size_t kSortCounterWords = 8;
constexpr uint32_t sortTiles(uint32_t n) { return n == 0u ? 1u : (n + kSortTile - 1u) / kSortTile; }
constexpr size_t sortScratchWordsFor(uint32_t n) {
    return kSortHistWords + kSortCounterWords + static_cast<size_t>(kSortMaxPasses) * sortTiles(n) * kSortBins;
}

// Number of 32-bit words of onesweep scratch for n keys.
size_t sortScratchWords(uint32_t n, uint32_t* maxTilesOut);

// Where the keys of the sort come from.
enum class KeySource { Array, MortonFromPositions };

struct MortonSource {
    const float* x;        // either SoA x/y/z ...
    const float* y;
    const float* z;
    const float4* xyz;     // ... or float4 {x, y, z, _} (used when non-null)
    const uint32_t* boundsOrdered;  // 6 ordered-uint words of the scene AABB
    float* boundsFloatOut;          // optional: decoded bounds written by block 0
};

// Stable LSD radix sort of (u64 key, u32 value) over bits [0, endBit).
// Data starts in (keysA, valsA); (keysB, valsB) is the ping-pong partner.
// Returns (through *resultInA) which pair holds the sorted output.
// With src == MortonFromPositions the keys and values (iota) are generated
// from positions in the histogram kernel and written into (keysA, valsA).
cudaError_t radixSortPairs(uint64_t* keysA, uint32_t* valsA, uint64_t* keysB, uint32_t* valsB, uint32_t n,
                           int endBit, uint32_t* scratch, size_t scratchWords, uint32_t maxTiles, DevStatus* status,
                           uint32_t spinLimit, KeySource src, const MortonSource* morton, bool* resultInA,
                           cudaStream_t stream);

// Failure-detection probe of the bounded look-back wait (see sort.cu).
cudaError_t launchLookbackProbe(const uint32_t* neverSet, DevStatus* status, uint32_t spinLimit, uint32_t* result,
                                cudaStream_t stream);

}  // namespace astraea_gb300
