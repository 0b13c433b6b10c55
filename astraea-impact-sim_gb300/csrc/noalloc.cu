// noalloc.cu -- a radix sort entry point that never allocates device memory.
//
// astraea_gb300_radix_sort_pairs allocates its scratch (digit histograms,
// look-back words, tile counters) with cudaMalloc on first use.  Some callers
// cannot allow that: code running inside a memory pool or arena that owns all
// device memory of the process, plug-ins whose host forbids allocation after
// start-up, and callers that must not hit an allocator's implicit device
// synchronisation on a latency-critical path.  For them this file provides
// astraea_gb300_radix_sort_pairs_noalloc: the same onesweep sort, with its
// scratch in a fixed array of device memory that is part of the library image
// itself.  The caller still provides the key/value buffers (in and out).
//
// Limits and behaviour:
//   * at most kNoAllocMaxKeys keys per call; larger calls return
//     ASTRAEA_ERR_CAPACITY without touching the GPU;
//   * every GPU that loads the library holds the array (about 2.1 MB) until
//     the process exits;
//   * the array is shared by all calls: each call clears the sort's parts that
//     must start at zero before its kernels run, but two calls whose work
//     overlaps on the GPU (different streams, or different host threads) race
//     on it;
//   * a look-back wait that gives up sets a flag in a status block kept in the
//     same array; the flag stays set until astraea_gb300_reset_device_status,
//     and astraea_gb300_read_device_status and astraea_gb300_reduce_dt_psu
//     report it like the allocating sort's (the result of such a call is not
//     sorted);
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (set-up, once per device); make that first call
//     before any stream capture.  The address is kept for the life of the
//     process, so cudaDeviceReset between calls is not supported.
#include <cstring>
#include <mutex>
#include <string>

#include "kernels.h"

namespace astraea_gb300 {

// Internal accessors of capi.cu (stream of the C-ABI, last-error message,
// look-back spin limit).
cudaStream_t capiStream();
void capiSetLastError(const std::string& msg);
uint32_t capiSpinLimit();

namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
constexpr size_t kStatusWords = (sizeof(DevStatus) + 255) / 256 * 64;   // 256-byte aligned status block
constexpr size_t kSortWordsMax = sortScratchWordsFor(kNoAllocMaxKeys);   // the sort's own layout

// [0, kStatusWords): a DevStatus for the look-back flag (zero at load, cleared
// only by astraea_gb300_reset_device_status); then the sort scratch.
static __device__ __align__(256) uint32_t g_noallocScratch[kStatusWords + kSortWordsMax];
static_assert(sizeof(g_noallocScratch) / sizeof(uint32_t) >= kStatusWords + sortScratchWordsFor(kNoAllocMaxKeys),
              "the fixed array must hold the sort's scratch for the largest call");

std::mutex g_setupMutex;
uint32_t* g_scratchAddr[64] = {};

uint32_t* scratchAddressIfSetUp() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_setupMutex);
    return g_scratchAddr[dev];
}

}  // namespace

// Device address of the flags word of the no-allocation sort's status block on
// the current device, or null while no call has set the device up (its flags
// are then zero).  Used by the status entry points of capi.cu.
uint32_t* noallocStatusFlagsAddress() {
    uint32_t* base = scratchAddressIfSetUp();
    return base == nullptr ? nullptr : &reinterpret_cast<DevStatus*>(base)->flags;
}

}  // namespace astraea_gb300

using namespace astraea_gb300;

extern "C" AstraeaStatus astraea_gb300_radix_sort_pairs_noalloc(uint64_t* keysIn, uint64_t* keysOut,
                                                                uint32_t* valsIn, uint32_t* valsOut, uint32_t n,
                                                                int endBit) {
    if (n > kNoAllocMaxKeys) {
        capiSetLastError("radix_sort_pairs_noalloc: " + std::to_string(n) + " keys exceed the fixed scratch limit of " +
                         std::to_string(kNoAllocMaxKeys) + " keys");
        return ASTRAEA_ERR_CAPACITY;
    }
    if (n == 0u) return ASTRAEA_OK;
    if (!keysIn || !keysOut || !valsIn || !valsOut || endBit < 1 || endBit > 64) {
        capiSetLastError("radix_sort_pairs_noalloc: bad argument");
        return ASTRAEA_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        capiSetLastError(std::string("radix_sort_pairs_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return ASTRAEA_ERR_CUDA;
    }
    uint32_t* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        if (g_scratchAddr[dev] == nullptr) {   // set-up, once per device, with that device current
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noallocScratch);
            if (e != cudaSuccess) {
                capiSetLastError(std::string("radix_sort_pairs_noalloc: cudaGetSymbolAddress: ") +
                                 cudaGetErrorString(e));
                return ASTRAEA_ERR_CUDA;
            }
            g_scratchAddr[dev] = static_cast<uint32_t*>(ptr);
        }
        base = g_scratchAddr[dev];
    }
    cudaStream_t st = capiStream();
    DevStatus* status = reinterpret_cast<DevStatus*>(base);
    uint32_t* sortScratch = base + kStatusWords;
    const uint32_t maxTiles = sortTiles(kNoAllocMaxKeys);
    bool inA = true;
    e = radixSortPairs(keysIn, valsIn, keysOut, valsOut, n, endBit, sortScratch, kSortWordsMax, maxTiles, status,
                       capiSpinLimit(), KeySource::Array, nullptr, &inA, st);
    if (e == cudaSuccess && inA) {
        e = cudaMemcpyAsync(keysOut, keysIn, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(valsOut, valsIn, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    }
    if (e != cudaSuccess) {
        capiSetLastError(std::string("radix_sort_pairs_noalloc: ") + cudaGetErrorString(e));
        return ASTRAEA_ERR_CUDA;
    }
    return ASTRAEA_OK;
}
