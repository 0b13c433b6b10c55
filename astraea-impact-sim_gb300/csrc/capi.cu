// capi.cu -- the C-ABI of include/astraea_gb300.h: allocation, the stage
// entry points that replace astraea::cuda::launch* (engine/sph_gravity.cu:
// 1796-2161), the fused step, and library-owned scratch.
//
// Scratch ("workspace") lives with the BVH it serves: it is keyed by the
// BVH's leftChild device pointer and created on the first build.  It holds
// the packed leaf / node records the tree walks read, the neighbour lists,
// the onesweep scratch and a few device words (bounds, living flags, dt).
// Nothing is allocated per step; astraea_gb300_reserve allocates everything
// ahead of time for callers that capture steps in a CUDA graph.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <string>
#include <utility>

#include "kernels.h"

using namespace astraea_gb300;

namespace {

thread_local std::string g_lastError;
std::atomic<cudaStream_t> g_stream{nullptr};
std::atomic<uint32_t> g_spinLimit{1u << 22};
std::atomic<int> g_nodeRounding{0};   // 0: exact moment sums, 1: the engine's FP32 bottom-up rounding
std::atomic<int> g_farField{0};   // 0: monopole (the engine's), 1: + quadrupole, 2: + learned correction,
                                  // 3: quadrupole + leaf buckets + group expansion of far nodes
std::atomic<uint32_t> g_leafBucket{16};      // mode 3: leaf bucket (particles)
std::atomic<float> g_expandGamma{0.3f};      // mode 3: group radius <= gamma |c - COM| takes the expansion
std::atomic<bool> g_stageTiming{false};   // events between the fused step's stages
constexpr int kStageCount = ASTRAEA_STAGE_COUNT;
std::mutex g_mutex;

AstraeaStatus fail(AstraeaStatus s, const std::string& msg) {
    g_lastError = msg;
    return s;
}

#define AG_CUDA(expr)                                                                                     \
    do {                                                                                                  \
        const cudaError_t agErr = (expr);                                                                 \
        if (agErr != cudaSuccess)                                                                         \
            return fail(ASTRAEA_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(agErr));        \
    } while (0)

cudaStream_t stream() { return g_stream.load(); }

int currentDevice() {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int smCount() {
    static int cache[64] = {};
    const int d = currentDevice();
    if (d >= 0 && d < 64 && cache[d] > 0) return cache[d];
    int s = 0;
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, d);
    if (s <= 0) s = 1;
    if (d >= 0 && d < 64) cache[d] = s;
    return s;
}

// ------------------------------------------------------- per-device state
struct DeviceState {
    DevStatus* status = nullptr;   // device (flags, dt word, counters)
    uint32_t* hostWord = nullptr;  // pinned, 4 words
    uint32_t* zeroWords = nullptr; // device, 8 zero words (absent living flags)
};
std::map<int, DeviceState> g_devices;

AstraeaStatus deviceState(DeviceState** out) {
    const int d = currentDevice();
    auto it = g_devices.find(d);
    if (it == g_devices.end()) {
        DeviceState s;
        AG_CUDA(cudaMalloc(&s.status, sizeof(DevStatus)));
        AG_CUDA(cudaMemset(s.status, 0, sizeof(DevStatus)));
        AG_CUDA(cudaMallocHost(&s.hostWord, 4 * sizeof(uint32_t)));
        AG_CUDA(cudaMalloc(&s.zeroWords, 8 * sizeof(uint32_t)));
        AG_CUDA(cudaMemset(s.zeroWords, 0, 8 * sizeof(uint32_t)));
        it = g_devices.emplace(d, s).first;
    }
    *out = &it->second;
    return ASTRAEA_OK;
}

// ------------------------------------------------------------- workspace
// The per-tree buffers of far-field mode 2: pair records, group centres and
// corrections, the pair-count word and the gate's device state.  One set
// per workspace (per BVH), so instances of an ensemble stepping in mode 2
// on their own streams neither share nor race on them; allocated at a
// workspace's first mode-2 call (an eager call: before any stream capture).
struct FfBuffers {
    uint2* pairs = nullptr;
    uint32_t pairCap = 0;
    float4* groups = nullptr;
    float* groupCorr = nullptr;
    uint32_t groupCap = 0;
    uint32_t* word = nullptr;      // [0]: pair count
    ff::GateDev* gate = nullptr;   // spot-check sums, decision, statistics
    bool lastCallGated = false;
    void release() {
        if (pairs) cudaFree(pairs);
        if (groups) cudaFree(groups);
        if (groupCorr) cudaFree(groupCorr);
        if (word) cudaFree(word);
        if (gate) cudaFree(gate);
        *this = FfBuffers{};
    }
};

struct Workspace {
    int device = 0;
    Work w{};
    uint32_t capacity = 0;
    void* block = nullptr;         // one allocation for all arrays
    float* dtSlots = nullptr;      // 2 floats (inside block)
    uint32_t* rawMin = nullptr;    // 2 words (inside block)
    bool treeBuilt = false;        // node records hold a tree built here
    uint32_t builtN = 0;           // particle count of that tree
    bool momentsBuilt = false;     // ... with second moments (far-field modes 1 and 2)
    bool stepCacheValid = false;   // neighbour lists + device dt valid for the next fused step
    const void* stepToken = nullptr;
    uint32_t stepCount = 0;
    int parity = 0;
    // stage timing: event k is recorded where stage k of the fused step
    // starts, event kStageCount where the step ends (created on first use)
    cudaEvent_t stageEv[kStageCount + 1] = {};
    bool stageRecorded = false;
    FfBuffers ff;                  // far-field mode 2 (created on first use)
};
std::map<std::pair<int, const void*>, Workspace*> g_work;

uint32_t maxNeighbors() {
    static uint32_t v = [] {
        const char* e = std::getenv("ASTRAEA_GB300_MAX_NEIGHBORS");
        long x = e ? std::strtol(e, nullptr, 10) : 192;
        if (x < 32) x = 32;
        if (x > 4096) x = 4096;
        return static_cast<uint32_t>((x + 3) & ~3L);
    }();
    return v;
}

size_t alignUp(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

AstraeaStatus allocWorkspace(Workspace* ws, uint32_t capacity) {
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    const size_t C = std::max<uint32_t>(capacity, 2u);
    const uint32_t maxNbr = maxNeighbors();
    uint32_t maxTiles = 0;
    const size_t sortWords = sortScratchWords(static_cast<uint32_t>(C), &maxTiles);
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += alignUp(bytes); return o; };
    const size_t oLeaf = take(C * 32), oAux = take(C * 16), oRec = take(C * 16 * kRec2Width);
    const size_t nbMax = refitBlocks(static_cast<uint32_t>(C)), levMax = refitLevels(static_cast<uint32_t>(nbMax));
    const size_t oNode = take(C * 64), oRange = take(C * 8), oLScan = take(C * 64), oMScan = take(C * 80);
    const size_t oTable = take(levMax * nbMax * 32), oBMom = take(nbMax * 80), oQuad = take(C * 32);
    const size_t oDrift = take(C * 16);
    const size_t oDRec = take(C * 32), oDAux = take(C * 8);
    const size_t oCnt = take(C * 4), oList = take((C + 31) / 32 * 32 * maxNbr * 4), oWords = take(kWCount * 4);
    const size_t oSort = take(sortWords * 4), oDt = take(64);
    void* block = nullptr;
    AG_CUDA(cudaMalloc(&block, off));
    char* b = static_cast<char*>(block);
    if (ws->block) cudaFree(ws->block);
    ws->block = block;
    ws->capacity = static_cast<uint32_t>(C);
    ws->device = currentDevice();
    Work& w = ws->w;
    w.capacity = static_cast<uint32_t>(C);
    w.maxNbr = maxNbr;
    w.leaf = reinterpret_cast<Rec32*>(b + oLeaf);
    w.leafAux = reinterpret_cast<float4*>(b + oAux);
    w.rec2 = reinterpret_cast<float4*>(b + oRec);
    w.node = reinterpret_cast<float4*>(b + oNode);
    w.nodeRange = reinterpret_cast<uint2*>(b + oRange);
    w.leafScan = reinterpret_cast<float4*>(b + oLScan);
    w.momScan = reinterpret_cast<long long*>(b + oMScan);
    w.blockTable = reinterpret_cast<float4*>(b + oTable);
    w.blockMom = reinterpret_cast<long long*>(b + oBMom);
    w.nodeQuad = reinterpret_cast<float4*>(b + oQuad);
    w.driftPos = reinterpret_cast<float4*>(b + oDrift);
    w.drift = reinterpret_cast<Rec32*>(b + oDRec);
    w.driftAux = reinterpret_cast<float2*>(b + oDAux);
    w.nbrCount = reinterpret_cast<uint32_t*>(b + oCnt);
    w.nbrList = reinterpret_cast<uint32_t*>(b + oList);
    w.words = reinterpret_cast<uint32_t*>(b + oWords);
    w.sortScratch = reinterpret_cast<uint32_t*>(b + oSort);
    w.sortScratchWords = sortWords;
    w.sortMaxTiles = maxTiles;
    w.status = ds->status;
    ws->dtSlots = reinterpret_cast<float*>(b + oDt);
    ws->rawMin = reinterpret_cast<uint32_t*>(b + oDt + 16);
    AG_CUDA(cudaMemset(w.words, 0, kWCount * 4));
    AG_CUDA(cudaMemset(b + oDt, 0, 64));
    ws->treeBuilt = false;
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

// Workspace of a BVH; created (or grown) when `create`.
AstraeaStatus workspaceFor(const AstraeaRadixBvh* bvh, uint32_t need, bool create, Workspace** out) {
    if (bvh == nullptr || bvh->leftChild == nullptr) return fail(ASTRAEA_ERR_INVALID, "BVH descriptor has no leftChild array");
    std::lock_guard<std::mutex> lock(g_mutex);
    const auto key = std::make_pair(currentDevice(), static_cast<const void*>(bvh->leftChild));
    auto it = g_work.find(key);
    if (it == g_work.end()) {
        if (!create) return fail(ASTRAEA_ERR_INVALID, "BVH was not built by astraea_gb300_sort_and_build_bvh");
        Workspace* ws = new Workspace();
        const AstraeaStatus s = allocWorkspace(ws, need);
        if (s != ASTRAEA_OK) { delete ws; return s; }
        it = g_work.emplace(key, ws).first;
    } else if (it->second->capacity < need) {
        if (!create) return fail(ASTRAEA_ERR_CAPACITY, "workspace smaller than particle count");
        const AstraeaStatus s = allocWorkspace(it->second, need);
        if (s != ASTRAEA_OK) return s;
    }
    *out = it->second;
    return ASTRAEA_OK;
}

void dropWorkspace(const void* leftChild) {
    std::lock_guard<std::mutex> lock(g_mutex);
    for (auto it = g_work.begin(); it != g_work.end(); ++it) {
        if (it->first.second == leftChild) {
            cudaFree(it->second->block);
            for (cudaEvent_t e : it->second->stageEv)
                if (e) cudaEventDestroy(e);
            it->second->ff.release();
            delete it->second;
            g_work.erase(it);
            return;
        }
    }
}

template <typename T>
cudaError_t allocArr(T*& p, size_t count) {
    p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
}
template <typename T>
void freeArr(T*& p) {
    if (p) { cudaFree(p); p = nullptr; }
}

#define AG_ALL_PARTICLE_ARRAYS(X)                                                                          \
    X(posX) X(posY) X(posZ) X(velX) X(velY) X(velZ) X(velHalfX) X(velHalfY) X(velHalfZ) X(accX) X(accY)     \
        X(accZ) X(mass) X(h) X(h0) X(rho) X(drhoDt) X(pressure) X(soundSpeed) X(u) X(duDt) X(tempK)         \
            X(radPowerW) X(sXX) X(sYY) X(sZZ) X(sXY) X(sXZ) X(sYZ) X(dSXX) X(dSYY) X(dSZZ) X(dSXY) X(dSXZ)   \
                X(dSYZ) X(damage) X(damageCbrt) X(dDamageCbrtDt) X(epsFail) X(divV) X(curlVX) X(curlVY)     \
                    X(curlVZ) X(shepardC) X(surfFactor) X(phiGrav) X(materialId) X(phaseId) X(bodyId)      \
                        X(originalId) X(tracerIndex) X(tracerRestRadiusPsu) X(tracerRestNormalX)           \
                            X(tracerRestNormalY) X(tracerRestNormalZ) X(tracerIsOcean)

void swapParticlePointers(AstraeaParticles& a, AstraeaParticles& b) {   // sph_gravity.cu:1745-1784
#define AG_SWAP(f) std::swap(a.f, b.f);
    AG_ALL_PARTICLE_ARRAYS(AG_SWAP)
#undef AG_SWAP
}

AstraeaStatus checkLaunch(cudaError_t e, const char* what) {
    if (e != cudaSuccess) return fail(ASTRAEA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return ASTRAEA_OK;
}
#define AG_LAUNCH(expr)                                              \
    do {                                                             \
        const AstraeaStatus agS = checkLaunch((expr), #expr);        \
        if (agS != ASTRAEA_OK) return agS;                           \
    } while (0)

// ------------------------------------------------------------ autotuning
// Warps per block of the two tree walks, per device and power-of-two
// particle count (bucket floor(log2 n)); {4, 4} until tuned.  The gravity
// walk is tuned per variant (gravityVariant): its variants differ in
// registers and work per node, so the best shape of one is not the best of
// another (1M impact: 8 warps for the monopole walk at theta 0.5, 4 for the
// quadrupole walk at theta 0.7, 10 % apart).
std::mutex g_tuneMutex;
std::map<std::pair<int, int>, AstraeaTuning> g_tuning;
std::map<std::tuple<int, int, int>, uint32_t> g_gravTuning;
constexpr int kGravityVariants = 6;

int tuneBucket(uint32_t n) {
    int b = 0;
    while (b < 31 && (2u << b) <= n) ++b;
    return b;
}

AstraeaTuning tuningFor(uint32_t n) {
    std::lock_guard<std::mutex> lock(g_tuneMutex);
    const auto it = g_tuning.find(std::make_pair(currentDevice(), tuneBucket(n)));
    return (it == g_tuning.end()) ? AstraeaTuning{4u, 4u, 0.0f, 0.0f} : it->second;
}

// The gravity walk a call runs: 2 kind + inside, kind 0 the monopole walk
// (mode 0, the learned mode's fallback, or no moments built), 1 the
// quadrupole walk (mode 1), 2 the expansion walk (mode 3); inside = the
// inside-box rule of theta^2 > 1/3 (the same test as launchGravity).
int gravityVariant(int mode, bool moments, float theta) {
    const int kind = (!moments || mode == 0 || mode == 2) ? 0 : (mode == 1 ? 1 : 2);
    const float th = std::max(0.0f, theta);
    return 2 * kind + ((th * th > 0.333333f) ? 1 : 0);
}

uint32_t gravityWarpsFor(uint32_t n, int variant) {
    std::lock_guard<std::mutex> lock(g_tuneMutex);
    const auto it = g_gravTuning.find(std::make_tuple(currentDevice(), tuneBucket(n), variant));
    return (it == g_gravTuning.end()) ? 4u : it->second;
}

// ------------------------------------------- far-field mode 2 (learned)
struct FfState {
    ff::Net net{};
    bool ready = false;            // parameters initialised or loaded
    int adamStep = 0;
    AstraeaFarFieldConfig cfg{0.8f, 0.3f, 0.0f, 64u, 64u, 0u};
    const FfBuffers* last = nullptr;   // buffers of the last mode-2 gravity call (for ff_stats)
    float* pinned = nullptr;       // 4 floats / words for read-backs
    AstraeaFarFieldStats stats{0ull, 0ull, 0u, 0u, -1.0f, 0.0f};
};
std::map<int, FfState> g_ff;

AstraeaStatus ffState(FfState** out) {
    FfState& f = g_ff[currentDevice()];
    if (f.net.params == nullptr) {
        AG_CUDA(cudaMalloc(&f.net.params, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMalloc(&f.net.grads, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMalloc(&f.net.adamM, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMalloc(&f.net.adamV, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMalloc(&f.net.outScale, ff::kOut * sizeof(float)));
        AG_CUDA(cudaMalloc(&f.net.loss, sizeof(float)));
        AG_CUDA(cudaMallocHost(&f.pinned, 4 * sizeof(float)));
        AG_CUDA(cudaMemset(f.net.params, 0, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMemset(f.net.grads, 0, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMemset(f.net.adamM, 0, ff::kParams * sizeof(float)));
        AG_CUDA(cudaMemset(f.net.adamV, 0, ff::kParams * sizeof(float)));
        const float ones[ff::kOut] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
        AG_CUDA(cudaMemcpy(f.net.outScale, ones, sizeof(ones), cudaMemcpyHostToDevice));
        AG_CUDA(ff::prepareKernels());
    }
    *out = &f;
    return ASTRAEA_OK;
}

AstraeaStatus ffCapacity(FfBuffers* b, const FfState* f, uint32_t groups) {
    if (b->word == nullptr) {
        AG_CUDA(cudaMalloc(&b->word, 4 * sizeof(uint32_t)));
        AG_CUDA(cudaMalloc(&b->gate, sizeof(ff::GateDev)));
        AG_CUDA(cudaMemset(b->gate, 0, sizeof(ff::GateDev)));
    }
    const uint64_t want = static_cast<uint64_t>(groups) * std::max<uint32_t>(1u, f->cfg.pairsPerGroup);
    if (want > 0xFFFFFFFFull) return fail(ASTRAEA_ERR_CAPACITY, "far-field pair buffer above 2^32 entries");
    if (b->pairCap < want) {
        if (b->pairs) cudaFree(b->pairs);
        b->pairs = nullptr;
        b->pairCap = 0;
        AG_CUDA(cudaMalloc(&b->pairs, want * sizeof(uint2)));
        b->pairCap = static_cast<uint32_t>(want);
    }
    if (b->groupCap < groups) {
        if (b->groups) cudaFree(b->groups);
        if (b->groupCorr) cudaFree(b->groupCorr);
        b->groups = nullptr;
        b->groupCorr = nullptr;
        b->groupCap = 0;
        AG_CUDA(cudaMalloc(&b->groups, groups * sizeof(float4)));
        AG_CUDA(cudaMalloc(&b->groupCorr, 12ull * groups * sizeof(float)));
        b->groupCap = groups;
    }
    return ASTRAEA_OK;
}

// The mode-2 walk: the theta walk plus the far test; records pairs into the
// workspace's own buffers.
AstraeaStatus ffWalk(AstraeaParticles* p, Workspace* ws, uint32_t n, float theta, FfState* f, uint32_t stride) {
    const uint32_t groups = (n + 31u) / 32u;
    FfBuffers* b = &ws->ff;
    AstraeaStatus s = ffCapacity(b, f, groups);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_CUDA(cudaMemsetAsync(b->word, 0, sizeof(uint32_t), st));
    FarCapture cap{b->pairs, b->pairCap, b->word, b->groups, f->cfg.thetaFar * f->cfg.thetaFar,
                   f->cfg.gamma * f->cfg.gamma, std::max<uint32_t>(1u, stride)};
    AG_LAUNCH(launchGravity(*p, ws->w, n, theta, false, smCount(), st, &cap));
    return ASTRAEA_OK;
}

// Gravity of far-field mode 2: walk, network on the recorded pairs,
// per-member correction, and (gateTolerance > 0) the gate: a direct-sum spot
// check of gateTargets particles (FP32 pair terms with FP64 sums, or FP64)
// decides on the device whether the plain walk at theta that follows runs or
// returns at once.  No host round trip, so a gated step can be captured in a
// CUDA graph.
// ev (optional, 6 events): recorded before the walk, the network, the
// correction, the spot check, the fallback walk and at the end.
AstraeaStatus learnedGravity(AstraeaParticles* p, Workspace* ws, uint32_t n, float theta, bool gate,
                             cudaEvent_t* ev = nullptr) {
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    if (!f->ready) return fail(ASTRAEA_ERR_INVALID, "far-field mode 2 needs network parameters (ff_init / ff_set_params)");
    cudaStream_t st = stream();
    auto mark = [&](int k) { if (ev != nullptr) cudaEventRecord(ev[k], st); };
    mark(0);
    s = ffWalk(p, ws, n, theta, f, 1u);
    if (s != ASTRAEA_OK) return s;
    const uint32_t groups = (n + 31u) / 32u;
    mark(1);
    FfBuffers* b = &ws->ff;
    AG_CUDA(cudaMemsetAsync(b->groupCorr, 0, 12ull * groups * sizeof(float), st));
    AG_LAUNCH(ff::launchApply(f->net, ws->w, b->pairs, b->word, b->pairCap, b->groups, b->groupCorr, smCount(), st));
    mark(2);
    AG_LAUNCH(ff::launchCorrect(*p, b->groups, b->groupCorr, n, st));
    mark(3);
    f->stats.calls++;
    b->lastCallGated = false;
    f->last = b;
    if (gate && f->cfg.gateTolerance > 0.0f && n >= 2u) {
        const uint32_t K = std::max<uint32_t>(1u, std::min(f->cfg.gateTargets, n));
        AG_LAUNCH(ff::launchGate(*p, ws->w, n, K, f->cfg.gateTolerance, b->word, b->pairCap, b->gate,
                                 f->cfg.gateFp64Pairs == 0u, st));
        mark(4);
        Work w = ws->w;
        w.runIf = &b->gate->runFallback;       // the plain walk at theta, run only when the gate failed
        AG_LAUNCH(launchGravity(*p, w, n, theta, false, smCount(), st, nullptr,
                                static_cast<int>(gravityWarpsFor(n, gravityVariant(0, false, theta)))));
        b->lastCallGated = true;
    } else {
        mark(4);
    }
    mark(5);
    return ASTRAEA_OK;
}

// The gravity walk of far-field modes 0, 1 and 3 on a built workspace.
cudaError_t modeGravity(const AstraeaParticles& p, const Work& w0, uint32_t n, float theta, int mode, bool moments,
                        int sms, cudaStream_t st, int warps) {
    if (mode == 3 && moments) {
        Work w = w0;
        w.leafBucket = g_leafBucket.load();
        const float gm = g_expandGamma.load();
        w.expandGamma2 = gm * gm;
        return launchGravity(p, w, n, theta, true, sms, st, nullptr, warps, true);
    }
    return launchGravity(p, w0, n, theta, moments && mode == 1, sms, st, nullptr, warps);
}

uint32_t* livingPtr(const AstraeaRadixBvh* bvh, Workspace* ws) {
    return (bvh->livingFlags != nullptr) ? bvh->livingFlags : ws->w.words + kWLiving;
}

// Sort + permutation + Karras + refit shared by the stage call and the step.
// Events between the stages of one fused step (null events: timing off).
struct StageMarks {
    cudaEvent_t* ev = nullptr;
    cudaStream_t st = nullptr;
    void mark(int k) const {
        if (ev != nullptr) cudaEventRecord(ev[k], st);
    }
};

AstraeaStatus buildTree(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh, Workspace* ws,
                        const float4* driftPos, bool allFields, const StageMarks& marks = StageMarks{}) {
    const uint32_t n = p->count;
    cudaStream_t st = stream();
    Work& w = ws->w;
    uint32_t* living = livingPtr(bvh, ws);
    if (living != w.words + kWLiving) AG_CUDA(cudaMemsetAsync(living, 0, 2 * sizeof(uint32_t), st));
    MortonSource ms{};
    if (driftPos != nullptr) {
        ms.xyz = driftPos;
    } else {
        ms.x = p->posX; ms.y = p->posY; ms.z = p->posZ;
    }
    ms.boundsOrdered = w.words + kWBounds;
    ms.boundsFloatOut = bvh->sceneBoundsFloat;
    bool inA = true;
    // keys/values start in the *Sorted arrays; after an even number of passes
    // the sorted pairs are back there.
    AG_LAUNCH(radixSortPairs(bvh->mortonCodesSorted, bvh->indicesSorted, bvh->mortonCodes, bvh->indicesIn, n, 63,
                             w.sortScratch, w.sortScratchWords, w.sortMaxTiles, w.status, g_spinLimit.load(),
                             KeySource::MortonFromPositions, &ms, &inA, st));
    if (!inA) {
        AG_CUDA(cudaMemcpyAsync(bvh->mortonCodesSorted, bvh->mortonCodes, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        AG_CUDA(cudaMemcpyAsync(bvh->indicesSorted, bvh->indicesIn, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    }
    if (bvh->sceneBoundsOrdered != nullptr)
        AG_CUDA(cudaMemcpyAsync(bvh->sceneBoundsOrdered, w.words + kWBounds, 6 * sizeof(uint32_t),
                                cudaMemcpyDeviceToDevice, st));
    marks.mark(ASTRAEA_STAGE_PERMUTE);
    // The fused step (allFields == false) keeps its tree in the library's node
    // records only; the descriptor's node arrays (SoA and packed) are written
    // by the stage call, whose callers may read them.
    AstraeaRadixBvh kb = *bvh;
    if (!allFields) {
        kb.aabbMinX = nullptr;
        kb.nodeComMass = nullptr;
    }
    AG_LAUNCH(launchPermuteLeavesKarras(*p, *alt, kb, driftPos, w, n, living, allFields, st));
    swapParticlePointers(*p, *alt);
    alt->count = p->count;
    marks.mark(ASTRAEA_STAGE_REFIT);
    const bool moments = g_farField.load() != 0;
    AG_LAUNCH(launchRefit(kb, w, n, moments, st));
    if (g_nodeRounding.load() != 0) AG_LAUNCH(launchEngineNodeMoments(*p, kb, w, n, st));
    ws->treeBuilt = true;
    ws->builtN = n;
    ws->momentsBuilt = moments;
    return ASTRAEA_OK;
}

// Workspace holding a tree built here for exactly n particles.
AstraeaStatus builtWorkspace(const AstraeaRadixBvh* bvh, uint32_t n, Workspace** out) {
    AstraeaStatus s = workspaceFor(bvh, n, false, out);
    if (s != ASTRAEA_OK) return s;
    if (!(*out)->treeBuilt || (*out)->builtN != n)
        return fail(ASTRAEA_ERR_INVALID, "BVH holds no tree built by astraea_gb300_sort_and_build_bvh for this count");
    return ASTRAEA_OK;
}

float hostClampDt(uint32_t bits, float prevDt, float maxDt) {   // sph_gravity.cu:2137-2160
    const float floorDt = fminf(1.0e-5f, maxDt);
    const float upper = (prevDt > 0.0f) ? fminf(prevDt * 1.15f, maxDt) : maxDt;
    float raw = 0.0f;
    std::memcpy(&raw, &bits, sizeof(float));
    if (bits == 0x7f7f7f7fu || !std::isfinite(raw) || raw <= 0.0f) raw = upper;
    return fminf(upper, fmaxf(floorDt, raw));
}

}  // namespace

// Accessors for the other translation units of the library (noalloc.cu).
namespace astraea_gb300 {
cudaStream_t capiStream() { return stream(); }
void capiSetLastError(const std::string& msg) { g_lastError = msg; }
uint32_t capiSpinLimit() { return g_spinLimit.load(); }
uint32_t* noallocStatusFlagsAddress();   // noalloc.cu
}  // namespace astraea_gb300

extern "C" {

const char* astraea_gb300_last_error(void) { return g_lastError.c_str(); }
int astraea_gb300_abi_version(void) { return ASTRAEA_GB300_ABI_VERSION; }

AstraeaStatus astraea_gb300_set_stream(void* s) {
    g_stream.store(static_cast<cudaStream_t>(s));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_far_field(int mode) {
    if (mode < 0 || mode > 3) return fail(ASTRAEA_ERR_INVALID, "far-field mode must be 0, 1, 2 or 3");
    g_farField.store(mode);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_node_rounding(int mode) {
    if (mode < 0 || mode > 1) return fail(ASTRAEA_ERR_INVALID, "node rounding must be 0 or 1");
    g_nodeRounding.store(mode);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_far_field_expansion(uint32_t leafBucket, float gamma) {
    if (leafBucket > 32u) return fail(ASTRAEA_ERR_INVALID, "leaf bucket must be at most 32 particles");
    if (!(gamma >= 0.0f && gamma < 1.0f)) return fail(ASTRAEA_ERR_INVALID, "gamma must be in [0, 1)");
    g_leafBucket.store(leafBucket);
    g_expandGamma.store(gamma);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_lookback_spin_limit(uint32_t limit) {
    g_spinLimit.store(limit == 0u ? (1u << 22) : limit);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_read_device_status(uint32_t* flags, uint64_t* counters8) {
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    DevStatus h{};
    AG_CUDA(cudaStreamSynchronize(stream()));
    AG_CUDA(cudaMemcpy(&h, ds->status, sizeof(DevStatus), cudaMemcpyDeviceToHost));
    if (uint32_t* na = noallocStatusFlagsAddress()) {   // the no-allocation sort's own status block
        uint32_t f = 0;
        AG_CUDA(cudaMemcpy(&f, na, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        h.flags |= f;
    }
    if (flags) *flags = h.flags;
    if (counters8)
        for (int k = 0; k < 8; ++k) counters8[k] = h.counters[k];
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_reset_device_status(void) {
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    AG_CUDA(cudaMemsetAsync(ds->status, 0, sizeof(DevStatus), stream()));
    if (uint32_t* na = noallocStatusFlagsAddress()) AG_CUDA(cudaMemsetAsync(na, 0, sizeof(uint32_t), stream()));
    return ASTRAEA_OK;
}

// ------------------------------------------------------------ allocation
AstraeaStatus astraea_gb300_allocate_radix_bvh(AstraeaRadixBvh* bvh, uint32_t capacity) {
    if (bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null BVH");
    AstraeaStatus s = astraea_gb300_free_radix_bvh(bvh);
    if (s != ASTRAEA_OK) return s;
    if (capacity == 0u) return ASTRAEA_OK;
    const size_t nodes = 2u * static_cast<size_t>(capacity) - 1u;       // sph_gravity.cu:1812-1842
    const size_t internal = (capacity > 1u) ? static_cast<size_t>(capacity - 1u) : 1u;
    AG_CUDA(allocArr(bvh->mortonCodes, capacity));
    AG_CUDA(allocArr(bvh->mortonCodesSorted, capacity));
    AG_CUDA(allocArr(bvh->indicesIn, capacity));
    AG_CUDA(allocArr(bvh->indicesSorted, capacity));
    AG_CUDA(allocArr(bvh->leftChild, internal));
    AG_CUDA(allocArr(bvh->rightChild, internal));
    AG_CUDA(allocArr(bvh->parent, nodes));
    AG_CUDA(allocArr(bvh->atomicVisited, internal));
    AG_CUDA(allocArr(bvh->aabbMinX, nodes)); AG_CUDA(allocArr(bvh->aabbMinY, nodes)); AG_CUDA(allocArr(bvh->aabbMinZ, nodes));
    AG_CUDA(allocArr(bvh->aabbMaxX, nodes)); AG_CUDA(allocArr(bvh->aabbMaxY, nodes)); AG_CUDA(allocArr(bvh->aabbMaxZ, nodes));
    AG_CUDA(allocArr(bvh->nodeMass, nodes));
    AG_CUDA(allocArr(bvh->comX, nodes)); AG_CUDA(allocArr(bvh->comY, nodes)); AG_CUDA(allocArr(bvh->comZ, nodes));
    AG_CUDA(allocArr(bvh->nodeMaxH, nodes));
    AG_CUDA(allocArr(bvh->sceneBoundsOrdered, 6));
    AG_CUDA(allocArr(bvh->sceneBoundsFloat, 6));
    AG_CUDA(allocArr(bvh->livingFlags, 2));
    AG_CUDA(allocArr(bvh->nodeComMass, nodes));
    AG_CUDA(allocArr(bvh->nodeMinExtent, nodes));
    AG_CUDA(allocArr(bvh->nodeMaxHPacked, nodes));
    AG_CUDA(cudaMemset(bvh->livingFlags, 0, 2 * sizeof(uint32_t)));
    bvh->cubTempStorage = nullptr;
    bvh->cubTempBytes = 0;
    bvh->capacity = capacity;
    Workspace* ws = nullptr;
    return workspaceFor(bvh, capacity, true, &ws);
}

AstraeaStatus astraea_gb300_free_radix_bvh(AstraeaRadixBvh* bvh) {
    if (bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null BVH");
    if (bvh->leftChild != nullptr) dropWorkspace(bvh->leftChild);
    freeArr(bvh->mortonCodes); freeArr(bvh->mortonCodesSorted); freeArr(bvh->indicesIn); freeArr(bvh->indicesSorted);
    freeArr(bvh->leftChild); freeArr(bvh->rightChild); freeArr(bvh->parent); freeArr(bvh->atomicVisited);
    freeArr(bvh->aabbMinX); freeArr(bvh->aabbMinY); freeArr(bvh->aabbMinZ);
    freeArr(bvh->aabbMaxX); freeArr(bvh->aabbMaxY); freeArr(bvh->aabbMaxZ);
    freeArr(bvh->nodeMass); freeArr(bvh->comX); freeArr(bvh->comY); freeArr(bvh->comZ); freeArr(bvh->nodeMaxH);
    freeArr(bvh->sceneBoundsOrdered); freeArr(bvh->sceneBoundsFloat); freeArr(bvh->livingFlags);
    freeArr(bvh->nodeComMass); freeArr(bvh->nodeMinExtent); freeArr(bvh->nodeMaxHPacked);
    if (bvh->cubTempStorage) { cudaFree(bvh->cubTempStorage); bvh->cubTempStorage = nullptr; }
    bvh->cubTempBytes = 0;
    bvh->capacity = 0;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_allocate_particle_buffers(AstraeaParticles* p, uint32_t capacity) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    astraea_gb300_free_particle_buffers(p);
    if (capacity == 0u) return ASTRAEA_OK;
#define AG_ALLOC(f) AG_CUDA(allocArr(p->f, capacity));
    AG_ALL_PARTICLE_ARRAYS(AG_ALLOC)
#undef AG_ALLOC
    p->capacity = capacity;
    p->count = 0;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_free_particle_buffers(AstraeaParticles* p) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
#define AG_FREE(f) freeArr(p->f);
    AG_ALL_PARTICLE_ARRAYS(AG_FREE)
#undef AG_FREE
    p->capacity = 0;
    p->count = 0;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_reserve(const AstraeaRadixBvh* bvh, uint32_t capacity) {
    Workspace* ws = nullptr;
    AstraeaStatus s = workspaceFor(bvh, capacity, true, &ws);
    if (s != ASTRAEA_OK) return s;
    DeviceState* ds = nullptr;
    return deviceState(&ds);
}

AstraeaStatus astraea_gb300_release_scratch(const AstraeaRadixBvh* bvh) {
    if (bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null BVH");
    if (bvh->leftChild != nullptr) dropWorkspace(bvh->leftChild);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_invalidate_step_cache(const AstraeaRadixBvh* bvh) {
    Workspace* ws = nullptr;
    AstraeaStatus s = workspaceFor(bvh, 0, false, &ws);
    if (s != ASTRAEA_OK) return ASTRAEA_OK;   // nothing cached
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

// ---------------------------------------------------------------- stages
AstraeaStatus astraea_gb300_clear_stats(AstraeaParticles* p) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    if (p->count == 0u) return ASTRAEA_OK;
    AG_LAUNCH(launchClearStats(*p, p->count, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_sort_and_build_bvh(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh) {
    if (p == nullptr || alt == nullptr || bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    if (bvh->capacity < n || alt->capacity < n)                            // sph_gravity.cu:2001-2003
        return fail(ASTRAEA_ERR_CAPACITY, "launchSortAndBuildBvh: device buffers capacity < particle count");
    Workspace* ws = nullptr;
    AstraeaStatus s = workspaceFor(bvh, std::max(bvh->capacity, n), true, &ws);
    if (s != ASTRAEA_OK) return s;
    if (bvh->livingFlags == nullptr) bvh->livingFlags = ws->w.words + kWLiving;   // sph_gravity.cu:2008-2011
    AG_LAUNCH(launchInitBounds(ws->w.words, stream()));
    AG_LAUNCH(launchBounds(*p, n, ws->w.words, smCount(), stream()));
    s = buildTree(p, alt, bvh, ws, nullptr, true);
    if (s != ASTRAEA_OK) return s;
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_sph_pass1_neighbors(AstraeaParticles* p, const AstraeaRadixBvh* bvh) {
    if (p == nullptr || bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, true, st));
    AG_LAUNCH(launchBuildNeighbors(ws->w, n, smCount(), st, static_cast<int>(tuningFor(n).neighborWarps)));
    AG_LAUNCH(launchPass1(*p, ws->w, n, st));
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_evaluate_eos(AstraeaParticles* p) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    if (p->count == 0u) return ASTRAEA_OK;
    AG_LAUNCH(launchEos(*p, nullptr, p->count, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_gravity_barnes_hut(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta) {
    if (p == nullptr || bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, stream()));
    const int mode = g_farField.load();
    if (mode != 0 && !ws->momentsBuilt)
        return fail(ASTRAEA_ERR_INVALID, "far-field modes 1, 2 and 3 need a tree built in that mode");
    if (mode == 2) {
        s = learnedGravity(p, ws, n, theta, true);
        if (s != ASTRAEA_OK) return s;
    } else {
        AG_LAUNCH(modeGravity(*p, ws->w, n, theta, mode, true, smCount(), stream(),
                              static_cast<int>(gravityWarpsFor(n, gravityVariant(mode, true, theta)))));
    }
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_debug_gravity_group_trace(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                                     uint32_t group, int32_t* trace, uint32_t capacity) {
    if (p == nullptr || bvh == nullptr || trace == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    if (g_farField.load() != 0) return fail(ASTRAEA_ERR_INVALID, "the trace is taken in far-field mode 0");
    AG_CUDA(cudaMemsetAsync(trace, 0, sizeof(int32_t), stream()));
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, stream()));
    Work w = ws->w;
    w.traceList = trace;
    w.traceGroup = group;
    w.traceCap = capacity;
    AG_LAUNCH(launchGravity(*p, w, n, theta, false, smCount(), stream(), nullptr,
                            static_cast<int>(gravityWarpsFor(n, gravityVariant(0, false, theta)))));
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_debug_gravity_group_counts(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                                      uint32_t* groupCounts) {
    if (p == nullptr || bvh == nullptr || groupCounts == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    if (g_farField.load() != 0) return fail(ASTRAEA_ERR_INVALID, "group counts are taken in far-field mode 0");
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, stream()));
    Work w = ws->w;
    w.groupCounts = groupCounts;
    AG_LAUNCH(launchGravity(*p, w, n, theta, false, smCount(), stream(), nullptr,
                            static_cast<int>(gravityWarpsFor(n, gravityVariant(0, false, theta)))));
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_sph_pass2_forces(AstraeaParticles* p, const AstraeaRadixBvh* bvh) {
    if (p == nullptr || bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    DeviceState* ds = nullptr;
    s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, true, st));
    AG_LAUNCH(launchBuildNeighbors(ws->w, n, smCount(), st, static_cast<int>(tuningFor(n).neighborWarps)));
    AG_LAUNCH(launchPackPass2Records(*p, ws->w, n, st));
    const uint32_t* living = (bvh->livingFlags != nullptr) ? bvh->livingFlags : ds->zeroWords;   // :2104
    AG_LAUNCH(launchPass2(*p, ws->w, n, living, st));
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_leapfrog_kick_half(AstraeaParticles* p, float halfDtPsu, int includeXsph,
                                               int clampThermal) {
    (void)includeXsph;   // unused by the engine kernel too (sph_gravity.cu:1297)
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    if (p->count == 0u) return ASTRAEA_OK;
    KickArgs a{};
    a.halfDtHost = halfDtPsu;
    a.dtMode = 0;
    a.clampThermal = clampThermal != 0;
    AG_LAUNCH(launchKick(*p, p->count, a, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_leapfrog_drift(AstraeaParticles* p, float dtPsu, const AstraeaRadixBvh* bvh) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    cudaStream_t st = stream();
    const bool useBvh = bvh != nullptr && bvh->capacity >= n && bvh->leftChild != nullptr &&   // :2127
                        bvh->rightChild != nullptr && n >= 2u;
    if (!useBvh) {
        AG_LAUNCH(launchDriftPlain(*p, n, dtPsu, st));
        return ASTRAEA_OK;
    }
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, true, st));
    AG_LAUNCH(launchBuildNeighbors(ws->w, n, smCount(), st, static_cast<int>(tuningFor(n).neighborWarps)));
    AG_LAUNCH(launchDrift(*p, ws->w, n, nullptr, dtPsu, true, false, nullptr, st));
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_reduce_dt_psu(const AstraeaParticles* p, float prevDtPsu, float maxDtPsu, float* outDt) {
    if (p == nullptr || outDt == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const float upper = (prevDtPsu > 0.0f) ? fminf(prevDtPsu * 1.15f, maxDtPsu) : maxDtPsu;
    if (p->count == 0u) { *outDt = upper; return ASTRAEA_OK; }
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    uint32_t* dtWord = &ds->status->dtBits;
    AG_CUDA(cudaMemsetAsync(dtWord, 0x7f, sizeof(uint32_t), st));       // sph_gravity.cu:2146
    AG_LAUNCH(launchReduceDt(*p, p->count, dtWord, smCount(), st));
    // flags + dt bits in one copy: the blocking read the engine does anyway
    AG_CUDA(cudaMemcpyAsync(ds->hostWord, ds->status, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ds->hostWord[2] = 0u;
    if (uint32_t* na = noallocStatusFlagsAddress())
        AG_CUDA(cudaMemcpyAsync(ds->hostWord + 2, na, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AG_CUDA(cudaStreamSynchronize(st));
    if ((ds->hostWord[0] | ds->hostWord[2]) & kFlagLookbackTimeout)
        return fail(ASTRAEA_ERR_DEVICE_TIMEOUT, "a radix-sort look-back wait timed out; results since the last status "
                                                "reset are invalid (astraea_gb300_reset_device_status clears it)");
    *outDt = hostClampDt(ds->hostWord[1], prevDtPsu, maxDtPsu);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_pack_render_records(const AstraeaParticles* p, uint8_t* records20, uint8_t* speedBytes,
                                                float sysComX, float sysComY, float sysComZ) {
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    if (p->count == 0u || records20 == nullptr) return ASTRAEA_OK;            // sph_gravity.cu:2195-2197
    AG_LAUNCH(launchPackRender(*p, p->count, records20, speedBytes, sysComX, sysComY, sysComZ, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_extract_tracers(const AstraeaParticles* p, uint8_t* records40, uint32_t tracerCount,
                                            uint32_t tracerGridRes, float livingComX, float livingComY,
                                            float livingComZ, float sysComX, float sysComY, float sysComZ) {
    (void)tracerGridRes;                                                     // unused, as in the engine
    if (p == nullptr) return fail(ASTRAEA_ERR_INVALID, "null particle descriptor");
    AG_LAUNCH(launchExtractTracers(*p, p->count, records40, tracerCount, livingComX, livingComY, livingComZ, sysComX,
                                   sysComY, sysComZ, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_pcls_frame_bytes(uint32_t particleCount, uint32_t tracerCount, int withSpeed,
                                              size_t* outBytes) {
    if (outBytes == nullptr) return fail(ASTRAEA_ERR_INVALID, "null output");
    const size_t n = particleCount, t = tracerCount;
    *outBytes = 40u + 20u * n + 40u * t + ((withSpeed && n > 0u) ? n : 0u);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_pack_pcls_frame(const AstraeaParticles* p, const AstraeaPclsFrameInfo* info,
                                            uint8_t* frame, size_t frameCapacity, size_t* outFrameBytes) {
    if (p == nullptr || info == nullptr || frame == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count, t = info->tracerCount;
    const bool hasSpeed = info->withSpeed != 0 && n > 0u;                    // binary_protocol.cpp:163
    const size_t payload = 20u * static_cast<size_t>(n) + 40u * static_cast<size_t>(t) + (hasSpeed ? n : 0u);
    if (payload > 0xffffffffull) return fail(ASTRAEA_ERR_CAPACITY, "PCLS payload exceeds 4 GiB");
    if (frameCapacity < 40u + payload) return fail(ASTRAEA_ERR_CAPACITY, "frame buffer too small");
    PclsHeaderWords h{};                                                     // binary_protocol.cpp:76-87, 168-187
    uint32_t flags = 0u;
    if (t > 0u) flags |= 2u;                       // kFlagHasTracers
    if (info->livingBodyPresent) flags |= 4u;      // kFlagHasLivingCom
    if (hasSpeed) flags |= 8u;                     // kFlagHasSpeedArray (never kFlagZlib: no device deflate)
    uint64_t simBits;
    std::memcpy(&simBits, &info->simTimeSec, 8);
    uint32_t dtBits;
    std::memcpy(&dtBits, &info->dtSec, 4);
    h.w[0] = 0x50434C53u;                          // "PCLS"
    h.w[1] = 1u | (flags << 16);                   // version 1
    h.w[2] = static_cast<uint32_t>(simBits);
    h.w[3] = static_cast<uint32_t>(simBits >> 32);
    h.w[4] = static_cast<uint32_t>(info->frameSeq & 0xffffffffull);
    h.w[5] = dtBits;
    h.w[6] = n;
    h.w[7] = t;
    h.w[8] = t > 0u ? info->tracerGridRes : 0u;
    h.w[9] = static_cast<uint32_t>(payload);
    AG_LAUNCH(launchWriteHeader(frame, h, stream()));
    uint8_t* particles = frame + 40;
    uint8_t* tracers = particles + 20u * static_cast<size_t>(n);
    uint8_t* speed = hasSpeed ? tracers + 40u * static_cast<size_t>(t) : nullptr;
    AG_LAUNCH(launchPackRender(*p, n, particles, speed, info->sysCom[0], info->sysCom[1], info->sysCom[2], stream()));
    AG_LAUNCH(launchExtractTracers(*p, n, tracers, t, info->livingCom[0], info->livingCom[1], info->livingCom[2],
                                   info->sysCom[0], info->sysCom[1], info->sysCom[2], stream()));
    if (outFrameBytes != nullptr) *outFrameBytes = 40u + payload;
    return ASTRAEA_OK;
}

static_assert(sizeof(AstraeaTelemetry) == 392, "AstraeaTelemetry layout");

AstraeaStatus astraea_gb300_reduce_telemetry(const AstraeaParticles* p, const AstraeaTelemetryParams* params,
                                             AstraeaTelemetry* out) {
    if (p == nullptr || params == nullptr || out == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof(*out));
    if (p->count == 0u) return ASTRAEA_OK;                                   // simulation.cpp:962-965
    AG_LAUNCH(launchTelemetry(*p, p->count, params->targetRadiusPsu, params->livingBodyPresent, smCount(), out,
                              stream()));
    return ASTRAEA_OK;
}

// Simulation::Impl::relaxLoadedSingleBody (engine/simulation.cpp:585-781)
// with the per-iteration host round trip replaced by device passes.
AstraeaStatus astraea_gb300_relax_single_body(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh,
                                              const double* anchorTempByOrigId, uint32_t anchorCount,
                                              double nominalRadiusPsu, uint32_t steps, double* outFinalVrmsOverVesc) {
    if (p == nullptr || alt == nullptr || bvh == nullptr || outFinalVrmsOverVesc == nullptr)
        return fail(ASTRAEA_ERR_INVALID, "null argument");
    *outFinalVrmsOverVesc = 0.0;
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;                                          // :590-593
    AstraeaStatus s;
#define AG_STAGE(call) do { s = (call); if (s != ASTRAEA_OK) return s; } while (0)
    auto forces = [&]() -> AstraeaStatus {                                   // :616 / :709-711
        AstraeaStatus r = astraea_gb300_evaluate_eos(p);
        if (r == ASTRAEA_OK) r = astraea_gb300_gravity_barnes_hut(p, bvh, 0.5f);
        if (r == ASTRAEA_OK) r = astraea_gb300_sph_pass2_forces(p, bvh);
        return r;
    };
    auto build = [&]() -> AstraeaStatus {
        AstraeaStatus r = astraea_gb300_sort_and_build_bvh(p, alt, bvh);
        if (r == ASTRAEA_OK) r = astraea_gb300_sph_pass1_neighbors(p, bvh);
        return r;
    };
    float prevDt = 0.0f;
    auto step = [&]() -> AstraeaStatus {                                     // :604-616
        float dt = 0.0f;
        AstraeaStatus r = astraea_gb300_reduce_dt_psu(p, prevDt, 0.02f, &dt);
        if (r != ASTRAEA_OK) return r;
        prevDt = dt;
        if ((r = astraea_gb300_leapfrog_kick_half(p, 0.5f * dt, 1, 1)) != ASTRAEA_OK) return r;
        if ((r = astraea_gb300_leapfrog_drift(p, dt, bvh)) != ASTRAEA_OK) return r;
        if ((r = build()) != ASTRAEA_OK) return r;
        if ((r = forces()) != ASTRAEA_OK) return r;
        return astraea_gb300_leapfrog_kick_half(p, 0.5f * dt, 0, 1);
    };
    AG_STAGE(astraea_gb300_clear_stats(p));                                  // evaluateInitialForcesOnDevice
    AG_STAGE(build());
    AG_STAGE(forces());
    for (uint32_t it = 0; it < steps; ++it) {
        AG_STAGE(step());
        AG_LAUNCH(launchRelaxRecentre(*p, p->count, anchorTempByOrigId, anchorCount, smCount(), stream()));
        if (it + 1u < steps) AG_STAGE(forces());                             // :708-712
    }
    if (steps > 0u) {                                                        // :715-737
        AG_STAGE(build());
        AG_STAGE(forces());
        for (int c = 0; c < 4; ++c) AG_STAGE(step());
        AG_STAGE(astraea_gb300_evaluate_eos(p));
    }
    AG_LAUNCH(launchRelaxDiagnostic(*p, p->count, nominalRadiusPsu, smCount(), outFinalVrmsOverVesc, stream()));
    if (steps > 0u) {                                                        // :769-780
        AG_LAUNCH(launchRelaxAnchor(*p, p->count, anchorTempByOrigId, anchorCount, stream()));
        AG_STAGE(astraea_gb300_evaluate_eos(p));
        AG_CUDA(cudaStreamSynchronize(stream()));
    }
#undef AG_STAGE
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_direct_gravity_f64(const AstraeaParticles* p, const uint32_t* targets, uint32_t count,
                                              double* acc3, double* phi) {
    if (p == nullptr || (count > 0u && (targets == nullptr || acc3 == nullptr || phi == nullptr)))
        return fail(ASTRAEA_ERR_INVALID, "null argument");
    AG_LAUNCH(launchDirectGravityF64(*p, p->count, targets, count, acc3, phi, stream()));
    return ASTRAEA_OK;
}

// ------------------------------------------- learned far field (mode 2)
AstraeaStatus astraea_gb300_ff_configure(const AstraeaFarFieldConfig* cfg) {
    if (cfg == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    if (!(cfg->thetaFar > 0.0f) || !(cfg->gamma > 0.0f) || !(cfg->gateTolerance >= 0.0f) || cfg->pairsPerGroup == 0u)
        return fail(ASTRAEA_ERR_INVALID, "ff_configure: thetaFar, gamma, pairsPerGroup must be > 0");
    if (cfg->gateTargets > ff::kGateMaxTargets)
        return fail(ASTRAEA_ERR_INVALID, "ff_configure: gateTargets must be <= 1024");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    f->cfg = *cfg;
    if (f->cfg.gateTargets == 0u) f->cfg.gateTargets = 64u;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_collect(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                       uint32_t groupStride, float* features, float* labels, uint32_t capacity,
                                       uint32_t* outCount) {
    if (p == nullptr || bvh == nullptr || outCount == nullptr || (capacity > 0u && (features == nullptr || labels == nullptr)))
        return fail(ASTRAEA_ERR_INVALID, "null argument");
    *outCount = 0;
    const uint32_t n = p->count;
    if (n < 2u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    if (!ws->momentsBuilt) return fail(ASTRAEA_ERR_INVALID, "ff_collect needs a tree built in far-field mode 2");
    FfState* f = nullptr;
    s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, st));
    s = ffWalk(p, ws, n, theta, f, groupStride);
    if (s != ASTRAEA_OK) return s;
    uint32_t recorded = 0;
    AG_CUDA(cudaMemcpyAsync(f->pinned, ws->ff.word, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AG_CUDA(cudaStreamSynchronize(st));
    std::memcpy(&recorded, f->pinned, sizeof(uint32_t));
    const uint32_t rows = std::min(std::min(recorded, ws->ff.pairCap), capacity);
    AG_LAUNCH(ff::launchLabels(ws->w, n, ws->ff.pairs, rows, ws->ff.groups, features, labels, st));
    AG_CUDA(cudaStreamSynchronize(st));
    ws->stepCacheValid = false;
    *outCount = rows;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_init(uint64_t seed) {
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    std::vector<float> h(ff::kParams, 0.0f);
    uint64_t x = seed ^ 0x2545F4914F6CDD1Dull;
    auto uni = [&]() {                             // xorshift64*, uniform in [-1, 1)
        x ^= x >> 12; x ^= x << 25; x ^= x >> 27;
        return static_cast<float>(static_cast<double>((x * 0x2545F4914F6CDD1Dull) >> 11) * 0x1.0p-52 - 1.0);
    };
    auto fill = [&](int off, int fanIn, int fanOut) {
        const float a = std::sqrt(6.0f / static_cast<float>(fanIn + fanOut));
        for (int k = 0; k < fanIn * fanOut; ++k) h[off + k] = a * uni();
    };
    fill(ff::kW1, ff::kIn, ff::kHid);
    fill(ff::kW2, ff::kHid, ff::kHid);
    fill(ff::kW3, ff::kHid, ff::kOut);
    AG_CUDA(cudaMemcpy(f->net.params, h.data(), ff::kParams * sizeof(float), cudaMemcpyHostToDevice));
    AG_CUDA(cudaMemset(f->net.grads, 0, ff::kParams * sizeof(float)));
    AG_CUDA(cudaMemset(f->net.adamM, 0, ff::kParams * sizeof(float)));
    AG_CUDA(cudaMemset(f->net.adamV, 0, ff::kParams * sizeof(float)));
    f->adamStep = 0;
    f->ready = true;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_fit_output_scale(const float* labels, uint32_t count) {
    if (labels == nullptr || count == 0u) return fail(ASTRAEA_ERR_INVALID, "ff_fit_output_scale: no labels");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    std::vector<float> h(static_cast<size_t>(count) * ff::kOut);
    AG_CUDA(cudaMemcpy(h.data(), labels, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
    float scale[ff::kOut];
    for (int o = 0; o < ff::kOut; ++o) {
        double acc = 0.0;
        for (uint32_t r = 0; r < count; ++r) acc += static_cast<double>(h[static_cast<size_t>(r) * ff::kOut + o]) *
                                                   h[static_cast<size_t>(r) * ff::kOut + o];
        const double rms = std::sqrt(acc / count);
        scale[o] = (o < ff::kUsedOut && rms > 1.0e-12) ? static_cast<float>(rms) : 1.0f;
    }
    AG_CUDA(cudaMemcpy(f->net.outScale, scale, sizeof(scale), cudaMemcpyHostToDevice));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_gradients(const float* features, const float* labels, uint32_t count,
                                         float* outGrads, float* outLoss) {
    if (features == nullptr || labels == nullptr || count == 0u) return fail(ASTRAEA_ERR_INVALID, "ff_gradients: no rows");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_CUDA(cudaMemsetAsync(f->net.grads, 0, ff::kParams * sizeof(float), st));
    AG_CUDA(cudaMemsetAsync(f->net.loss, 0, sizeof(float), st));
    AG_LAUNCH(ff::launchTrain(f->net, features, labels, count, smCount(), st));
    if (outGrads) AG_CUDA(cudaMemcpyAsync(outGrads, f->net.grads, ff::kParams * sizeof(float), cudaMemcpyDeviceToHost, st));
    AG_CUDA(cudaMemcpyAsync(f->pinned, f->net.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    AG_CUDA(cudaMemsetAsync(f->net.grads, 0, ff::kParams * sizeof(float), st));
    AG_CUDA(cudaStreamSynchronize(st));
    f->stats.lastLoss = f->pinned[0];
    if (outLoss) *outLoss = f->pinned[0];
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_train_step(const float* features, const float* labels, uint32_t count,
                                          float learningRate, float* outLoss) {
    if (features == nullptr || labels == nullptr || count == 0u) return fail(ASTRAEA_ERR_INVALID, "ff_train_step: no rows");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    if (!f->ready) return fail(ASTRAEA_ERR_INVALID, "ff_train_step: call ff_init or ff_set_params first");
    cudaStream_t st = stream();
    AG_CUDA(cudaMemsetAsync(f->net.loss, 0, sizeof(float), st));
    AG_LAUNCH(ff::launchTrain(f->net, features, labels, count, smCount(), st));
    AG_LAUNCH(ff::launchAdam(f->net, learningRate, ++f->adamStep, st));
    if (outLoss) {
        AG_CUDA(cudaMemcpyAsync(f->pinned, f->net.loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        AG_CUDA(cudaStreamSynchronize(st));
        f->stats.lastLoss = f->pinned[0];
        *outLoss = f->pinned[0];
    }
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_predict(const float* features, uint32_t count, float* out) {
    if (count == 0u) return ASTRAEA_OK;
    if (features == nullptr || out == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    AG_LAUNCH(ff::launchPredict(f->net, features, count, out, smCount(), stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_get_params(float* params, uint32_t capacity, float* outScale16) {
    if (params == nullptr || capacity < static_cast<uint32_t>(ff::kParams))
        return fail(ASTRAEA_ERR_CAPACITY, "ff_get_params: needs 6288 floats");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    AG_CUDA(cudaStreamSynchronize(stream()));
    AG_CUDA(cudaMemcpy(params, f->net.params, ff::kParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (outScale16) AG_CUDA(cudaMemcpy(outScale16, f->net.outScale, ff::kOut * sizeof(float), cudaMemcpyDeviceToHost));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_set_params(const float* params, uint32_t count, const float* outScale16) {
    if (params == nullptr || count != static_cast<uint32_t>(ff::kParams))
        return fail(ASTRAEA_ERR_INVALID, "ff_set_params: needs exactly 6288 floats");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    AG_CUDA(cudaStreamSynchronize(stream()));
    AG_CUDA(cudaMemcpy(f->net.params, params, ff::kParams * sizeof(float), cudaMemcpyHostToDevice));
    if (outScale16) AG_CUDA(cudaMemcpy(f->net.outScale, outScale16, ff::kOut * sizeof(float), cudaMemcpyHostToDevice));
    AG_CUDA(cudaMemset(f->net.adamM, 0, ff::kParams * sizeof(float)));
    AG_CUDA(cudaMemset(f->net.adamV, 0, ff::kParams * sizeof(float)));
    f->adamStep = 0;
    f->ready = true;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_profile(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta, float* outMs5) {
    if (p == nullptr || bvh == nullptr || outMs5 == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count;
    if (n == 0u) return ASTRAEA_OK;
    if (g_farField.load() != 2) return fail(ASTRAEA_ERR_INVALID, "ff_profile runs far-field mode 2");
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    if (!ws->momentsBuilt) return fail(ASTRAEA_ERR_INVALID, "far-field mode 2 needs a tree built in that mode");
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, stream()));
    cudaEvent_t ev[6] = {};
    for (auto& e : ev) AG_CUDA(cudaEventCreate(&e));
    s = learnedGravity(p, ws, n, theta, true, ev);
    cudaError_t e = cudaEventSynchronize(ev[5]);
    for (int k = 0; k < 5 && e == cudaSuccess && s == ASTRAEA_OK; ++k) e = cudaEventElapsedTime(&outMs5[k], ev[k], ev[k + 1]);
    for (auto& x : ev) cudaEventDestroy(x);
    ws->stepCacheValid = false;
    if (s != ASTRAEA_OK) return s;
    AG_CUDA(e);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_ff_stats(AstraeaFarFieldStats* out) {
    if (out == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    FfState* f = nullptr;
    AstraeaStatus s = ffState(&f);
    if (s != ASTRAEA_OK) return s;
    // fallbacks over every workspace of this device; the last gate's values
    // from the workspace of the last mode-2 call (only compared, never
    // dereferenced: that workspace may have been released since)
    AG_CUDA(cudaDeviceSynchronize());
    uint64_t fallbacks = 0;
    ff::GateDev lastGate{};
    bool lastFound = false, lastGated = false;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        for (const auto& kv : g_work) {
            const FfBuffers& b = kv.second->ff;
            if (kv.first.first != currentDevice() || b.gate == nullptr) continue;
            ff::GateDev g{};
            AG_CUDA(cudaMemcpy(&g, b.gate, sizeof(g), cudaMemcpyDeviceToHost));
            fallbacks += g.fallbacks;
            if (&b == f->last) { lastGate = g; lastFound = true; lastGated = b.lastCallGated; }
        }
    }
    f->stats.fallbacks = fallbacks;
    f->stats.lastPairs = lastFound ? lastGate.lastPairs : 0u;
    f->stats.lastGateRms = (lastFound && lastGated) ? lastGate.lastRms : -1.0f;
    *out = f->stats;
    return ASTRAEA_OK;
}

// ------------------------------------------------------------- autotune
AstraeaStatus astraea_gb300_autotune(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                     AstraeaTuning* out) {
    if (p == nullptr || bvh == nullptr || out == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count;
    *out = tuningFor(n);
    if (n < 2u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    AG_CUDA(cudaEventCreate(&e0));
    AG_CUDA(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } guard{e0, e1};
    const int sms = smCount();
    auto best3 = [&](auto launch, float* ms) -> cudaError_t {
        cudaError_t e = launch();                  // warm-up
        if (e != cudaSuccess) return e;
        float best = 3.0e38f;
        for (int r = 0; r < 3; ++r) {
            if ((e = cudaEventRecord(e0, st)) != cudaSuccess) return e;
            if ((e = launch()) != cudaSuccess) return e;
            if ((e = cudaEventRecord(e1, st)) != cudaSuccess) return e;
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
            float t = 0.0f;
            if ((e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess) return e;
            best = std::min(best, t);
        }
        *ms = best;
        return cudaSuccess;
    };
    // the gravity walk the current far-field mode runs at theta (the learned
    // mode: its plain fallback walk; its own walk has one shape)
    const int mode = g_farField.load();
    const bool moments = ws->momentsBuilt;
    const int variant = gravityVariant(mode, moments, theta);
    const int walkMode = (mode == 2) ? 0 : mode;
    AstraeaTuning t{4u, 4u, 3.0e38f, 3.0e38f};
    for (int wv : {2, 4, 8}) {
        float ms = 0.0f;
        AG_CUDA(best3([&] { return modeGravity(*p, ws->w, n, theta, walkMode, moments, sms, st, wv); }, &ms));
        if (ms < t.gravityMs) { t.gravityMs = ms; t.gravityWarps = static_cast<uint32_t>(wv); }
    }
    for (int wv : {2, 4, 8}) {
        float ms = 0.0f;
        AG_CUDA(best3([&] { return launchBuildNeighbors(ws->w, n, sms, st, wv); }, &ms));
        if (ms < t.neighborMs) { t.neighborMs = ms; t.neighborWarps = static_cast<uint32_t>(wv); }
    }
    ws->stepCacheValid = false;
    {
        std::lock_guard<std::mutex> lock(g_tuneMutex);
        const int dev = currentDevice(), bucket = tuneBucket(n);
        g_gravTuning[std::make_tuple(dev, bucket, variant)] = t.gravityWarps;
        const auto it = g_tuning.find(std::make_pair(dev, bucket));
        AstraeaTuning kept = (it == g_tuning.end()) ? AstraeaTuning{4u, 4u, 0.0f, 0.0f} : it->second;
        kept.neighborWarps = t.neighborWarps;
        kept.neighborMs = t.neighborMs;
        if (variant == 0) {                         // the engine's walk: what get_tuning reports
            kept.gravityWarps = t.gravityWarps;
            kept.gravityMs = t.gravityMs;
        }
        g_tuning[std::make_pair(dev, bucket)] = kept;
    }
    *out = t;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_autotune_expansion(AstraeaParticles* p, const AstraeaRadixBvh* bvh, float theta,
                                               const uint32_t* candidates, uint32_t count, uint32_t* outBucket,
                                               float* outMs) {
    if (p == nullptr || bvh == nullptr || candidates == nullptr || count == 0u || outBucket == nullptr)
        return fail(ASTRAEA_ERR_INVALID, "null argument");
    const uint32_t n = p->count;
    if (n < 2u) return ASTRAEA_OK;
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK) return s;
    if (!ws->momentsBuilt) return fail(ASTRAEA_ERR_INVALID, "far-field mode 3 needs a tree built in that mode");
    for (uint32_t k = 0; k < count; ++k)
        if (candidates[k] > 32u) return fail(ASTRAEA_ERR_INVALID, "leaf bucket must be at most 32 particles");
    cudaStream_t st = stream();
    AG_LAUNCH(launchRefreshLeaves(*p, ws->w, n, false, st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    AG_CUDA(cudaEventCreate(&e0));
    AG_CUDA(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } guard{e0, e1};
    const int sms = smCount(), warps = static_cast<int>(gravityWarpsFor(n, gravityVariant(3, true, theta)));
    const uint32_t keep = g_leafBucket.load();
    float best = 3.0e38f;
    uint32_t bestBucket = keep;
    for (uint32_t k = 0; k < count; ++k) {
        g_leafBucket.store(candidates[k]);
        auto launch = [&] { return modeGravity(*p, ws->w, n, theta, 3, true, sms, st, warps); };
        AG_LAUNCH(launch());                         // warm-up
        float ms = 3.0e38f;
        for (int r = 0; r < 3; ++r) {
            AG_CUDA(cudaEventRecord(e0, st));
            AG_LAUNCH(launch());
            AG_CUDA(cudaEventRecord(e1, st));
            AG_CUDA(cudaEventSynchronize(e1));
            float t = 0.0f;
            AG_CUDA(cudaEventElapsedTime(&t, e0, e1));
            ms = std::min(ms, t);
        }
        if (outMs != nullptr) outMs[k] = ms;
        if (ms < best) { best = ms; bestBucket = candidates[k]; }
    }
    g_leafBucket.store(bestBucket);
    *outBucket = bestBucket;
    ws->stepCacheValid = false;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_get_tuning(uint32_t count, AstraeaTuning* out) {
    if (out == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    *out = tuningFor(count);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_tuning(uint32_t count, const AstraeaTuning* tuning) {
    if (tuning == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    auto ok = [](uint32_t v) { return v == 2u || v == 4u || v == 8u; };
    if (!ok(tuning->gravityWarps) || !ok(tuning->neighborWarps))
        return fail(ASTRAEA_ERR_INVALID, "set_tuning: warps per block must be 2, 4 or 8");
    std::lock_guard<std::mutex> lock(g_tuneMutex);
    const int dev = currentDevice(), bucket = tuneBucket(count);
    g_tuning[std::make_pair(dev, bucket)] = *tuning;
    for (int v = 0; v < kGravityVariants; ++v) g_gravTuning[std::make_tuple(dev, bucket, v)] = tuning->gravityWarps;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_get_gravity_warps(uint32_t count, int farFieldMode, float theta, uint32_t* outWarps) {
    if (outWarps == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    if (farFieldMode < 0 || farFieldMode > 3) return fail(ASTRAEA_ERR_INVALID, "far-field mode must be 0, 1, 2 or 3");
    *outWarps = gravityWarpsFor(count, gravityVariant(farFieldMode, true, theta));
    return ASTRAEA_OK;
}

// ------------------------------------------------------ planet building
static planet::BodySpec toBodySpec(const AstraeaBodySpec& s) {
    return planet::BodySpec{static_cast<int>(s.archetype > 5u ? 99u : s.archetype), s.massKg, s.surfaceTempK,
                            s.coreTempK, s.spinOmegaRadS};
}

AstraeaStatus astraea_gb300_solve_hydrostatic(const AstraeaBodySpec* spec, AstraeaRadialSample* profile,
                                              uint32_t capacity, uint32_t* outCount, double* outRadiusM,
                                              double* outCentralPressurePa) {
    if (spec == nullptr || outCount == nullptr || outRadiusM == nullptr || outCentralPressurePa == nullptr)
        return fail(ASTRAEA_ERR_INVALID, "null argument");
    std::vector<planet::Sample> prof;
    double radius = 0.0, pc = 0.0;
    std::string err;
    if (!planet::solveHydrostatic(toBodySpec(*spec), prof, radius, pc, &err))
        return fail(ASTRAEA_ERR_INVALID, "solve_hydrostatic: " + err);
    *outCount = static_cast<uint32_t>(prof.size());
    *outRadiusM = radius;
    *outCentralPressurePa = pc;
    if (profile == nullptr || capacity < prof.size())
        return fail(ASTRAEA_ERR_CAPACITY, "solve_hydrostatic: profile capacity below the sample count");
    for (size_t i = 0; i < prof.size(); ++i) {
        const planet::Sample& s = prof[i];
        profile[i] = AstraeaRadialSample{s.r, s.rho, s.P, s.M, s.T, static_cast<uint32_t>(s.mat), 0u};
    }
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_build_planet(const AstraeaBodySpec* spec, uint32_t particleCount, uint32_t bodyId,
                                         uint32_t tracerGridRes, uint64_t seed, AstraeaParticles* p, uint32_t offset,
                                         AstraeaPlanetInfo* info) {
    if (spec == nullptr || p == nullptr || info == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    if (particleCount == 0u) return fail(ASTRAEA_ERR_INVALID, "build_planet: particleCount must be > 0");
    if (bodyId > 255u) return fail(ASTRAEA_ERR_INVALID, "build_planet: bodyId must fit in 8 bits");
    if (tracerGridRes > 1024u) return fail(ASTRAEA_ERR_INVALID, "build_planet: tracerGridRes above 1024");
    if (static_cast<uint64_t>(offset) + particleCount > p->capacity)
        return fail(ASTRAEA_ERR_CAPACITY, "build_planet: offset + particleCount exceeds the buffer capacity");
#define AG_NONNULL(f) if (p->f == nullptr) return fail(ASTRAEA_ERR_INVALID, "build_planet: null array " #f);
    AG_ALL_PARTICLE_ARRAYS(AG_NONNULL)
#undef AG_NONNULL
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    planet::BuildResult r{};
    std::string err;
    const cudaError_t e = planet::buildOnDevice(toBodySpec(*spec), particleCount, static_cast<uint8_t>(bodyId),
                                                tracerGridRes, seed, *p, offset, ds->status, g_spinLimit.load(),
                                                stream(), &r, &err);
    if (!err.empty()) return fail(ASTRAEA_ERR_INVALID, "build_planet: " + err);
    AG_CUDA(e);
    *info = AstraeaPlanetInfo{r.radiusM, r.massKg, r.pcPa, r.tracerCount, r.profileCount, r.shellCount, 0u};
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_debug_lookback_probe(uint32_t spinLimit, uint32_t* outResult) {
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    cudaStream_t st = stream();
    uint32_t* words = ds->zeroWords;   // words[0]: never written by anyone; words[4]: result
    AG_LAUNCH(launchLookbackProbe(words, ds->status, spinLimit, words + 4, st));
    AG_CUDA(cudaMemcpyAsync(ds->hostWord, words + 4, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AG_CUDA(cudaStreamSynchronize(st));
    if (outResult) *outResult = ds->hostWord[0];
    return (ds->hostWord[0] == 2u) ? ASTRAEA_ERR_DEVICE_TIMEOUT : ASTRAEA_OK;
}

// -------------------------------------------------------------- fused step
AstraeaStatus astraea_gb300_step(AstraeaParticles* p, AstraeaParticles* alt, AstraeaRadixBvh* bvh, float prevDtPsu,
                                 float maxDtPsu, float theta, float* outDtPsu) {
    if (p == nullptr || alt == nullptr || bvh == nullptr) return fail(ASTRAEA_ERR_INVALID, "null descriptor");
    const uint32_t n = p->count;
    if (n == 0u) return fail(ASTRAEA_ERR_INVALID, "step called with no particles");
    if (bvh->capacity < n || alt->capacity < n)
        return fail(ASTRAEA_ERR_CAPACITY, "step: device buffers capacity < particle count");
    Workspace* ws = nullptr;
    AstraeaStatus s = builtWorkspace(bvh, n, &ws);
    if (s != ASTRAEA_OK)
        return fail(ASTRAEA_ERR_INVALID, "step: build the tree once with astraea_gb300_sort_and_build_bvh first");
    cudaStream_t st = stream();
    Work& w = ws->w;
    const AstraeaTuning tune = tuningFor(n);
    const int sms = smCount();
    int q = ws->parity;
    const bool useBvh = bvh->leftChild != nullptr && bvh->rightChild != nullptr && n >= 2u;
    const bool cacheOk = ws->stepCacheValid && ws->stepToken == static_cast<const void*>(p->posX);
    StageMarks marks;
    if (g_stageTiming.load()) {
        for (cudaEvent_t& e : ws->stageEv)
            if (e == nullptr) AG_CUDA(cudaEventCreate(&e));
        marks.ev = ws->stageEv;
        marks.st = st;
        ws->stageRecorded = true;
    }
    marks.mark(ASTRAEA_STAGE_REFRESH);
    if (!cacheOk) {
        // Device dt state from the caller's previous dt and the current state.
        AG_LAUNCH(launchSetDtSlots(ws->dtSlots, q, prevDtPsu, ws->rawMin, st));
        AG_LAUNCH(launchReduceDt(*p, n, ws->rawMin + q, sms, st));
        AG_LAUNCH(launchRefreshLeaves(*p, w, n, false, st));
        if (useBvh) AG_LAUNCH(launchBuildNeighbors(w, n, sms, st, static_cast<int>(tune.neighborWarps)));
    }
    // 1. opening half kick; dt resolved on the device
    marks.mark(ASTRAEA_STAGE_KICK);
    KickArgs k1{};
    k1.dtMode = 1;
    k1.rawMinIn = ws->rawMin + q;
    k1.dtSlots = ws->dtSlots;
    k1.parity = q;
    k1.maxDt = maxDtPsu;
    k1.resetWord = ws->rawMin + (q ^ 1);
    k1.boundsWordsInit = w.words;
    k1.driftOut = w.drift;
    AG_LAUNCH(launchKick(*p, n, k1, st));
    // 2. XSPH drift on the previous step's neighbour lists -> scratch positions + bounds
    marks.mark(ASTRAEA_STAGE_DRIFT);
    AG_LAUNCH(launchDrift(*p, w, n, ws->dtSlots + (q ^ 1), 0.0f, useBvh, true, w.words, st));
    // 3. sort + permutation (live fields) + Karras + refit
    marks.mark(ASTRAEA_STAGE_SORT);
    s = buildTree(p, alt, bvh, ws, w.driftPos, false, marks);
    if (s != ASTRAEA_OK) return s;
    // 4. neighbour lists for pass 1, pass 2 and the next drift
    marks.mark(ASTRAEA_STAGE_NEIGHBOURS);
    AG_LAUNCH(launchBuildNeighbors(w, n, sms, st, static_cast<int>(tune.neighborWarps)));
    marks.mark(ASTRAEA_STAGE_PASS1);
    AG_LAUNCH(launchPass1(*p, w, n, st));
    marks.mark(ASTRAEA_STAGE_EOS);
    AG_LAUNCH(launchEos(*p, &w, n, st));
    marks.mark(ASTRAEA_STAGE_GRAVITY);
    if (ws->momentsBuilt && g_farField.load() == 2) {
        s = learnedGravity(p, ws, n, theta, true);
        if (s != ASTRAEA_OK) return s;
    } else {
        const int mode = g_farField.load();
        AG_LAUNCH(modeGravity(*p, w, n, theta, mode, ws->momentsBuilt, sms, st,
                              static_cast<int>(gravityWarpsFor(n, gravityVariant(mode, ws->momentsBuilt, theta)))));
    }
    marks.mark(ASTRAEA_STAGE_PASS2);
    AG_LAUNCH(launchPass2(*p, w, n, livingPtr(bvh, ws), st));
    // 5. closing half kick + EOS + next dt minimum
    marks.mark(ASTRAEA_STAGE_KICK_EOS);
    KickArgs k2{};
    k2.dtMode = 2;
    k2.dtSlots = ws->dtSlots;
    k2.parity = q;
    k2.withEos = true;
    k2.rawMinOut = ws->rawMin + (q ^ 1);
    AG_LAUNCH(launchKick(*p, n, k2, st));
    marks.mark(kStageCount);
    if (outDtPsu != nullptr)
        AG_CUDA(cudaMemcpyAsync(outDtPsu, ws->dtSlots + (q ^ 1), sizeof(float), cudaMemcpyDeviceToHost, st));
    ws->parity = q ^ 1;
    ws->stepCacheValid = true;
    ws->stepToken = static_cast<const void*>(p->posX);
    ws->stepCount += 1;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_set_stage_timing(int enable) {
    g_stageTiming.store(enable != 0);
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_read_stage_times(const AstraeaRadixBvh* bvh, float* outMs, uint32_t capacity,
                                             uint32_t* outCount) {
    if (bvh == nullptr || outMs == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    Workspace* ws = nullptr;
    AstraeaStatus s = workspaceFor(bvh, 0u, false, &ws);
    if (s != ASTRAEA_OK) return s;
    if (!ws->stageRecorded) return fail(ASTRAEA_ERR_INVALID, "read_stage_times: no timed fused step on this BVH");
    AG_CUDA(cudaEventSynchronize(ws->stageEv[kStageCount]));
    const uint32_t m = std::min<uint32_t>(capacity, static_cast<uint32_t>(kStageCount));
    for (uint32_t k = 0; k < m; ++k) {
        float t = 0.0f;
        AG_CUDA(cudaEventElapsedTime(&t, ws->stageEv[k], ws->stageEv[k + 1]));
        outMs[k] = t;
    }
    if (outCount != nullptr) *outCount = m;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_read_device_counters(uint64_t* outCounters, uint32_t capacity, uint32_t* outCount) {
    if (outCounters == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    DevStatus h{};
    AG_CUDA(cudaStreamSynchronize(stream()));
    AG_CUDA(cudaMemcpy(&h, ds->status, sizeof(DevStatus), cudaMemcpyDeviceToHost));
    const uint32_t m = std::min<uint32_t>(capacity, static_cast<uint32_t>(kCntCount));
    for (uint32_t k = 0; k < m; ++k) outCounters[k] = h.counters[k];
    if (outCount != nullptr) *outCount = m;
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_measure_fp32_tflops(float* outTflops) {
    if (outTflops == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    AG_LAUNCH(measureFp32Tflops(smCount(), outTflops, stream()));
    return ASTRAEA_OK;
}

AstraeaStatus astraea_gb300_measure_fp32_peaks(float* outScalarTflops, float* outPackedTflops) {
    if (outScalarTflops == nullptr || outPackedTflops == nullptr) return fail(ASTRAEA_ERR_INVALID, "null argument");
    float peak = 0.f;
    AG_LAUNCH(measureFp32TflopsBoth(smCount(), outScalarTflops, outPackedTflops, &peak, stream()));
    return ASTRAEA_OK;
}

// ------------------------------------------------------------ radix sort
AstraeaStatus astraea_gb300_radix_sort_pairs(uint64_t* keysIn, uint64_t* keysOut, uint32_t* valsIn,
                                             uint32_t* valsOut, uint32_t n, int endBit) {
    if (n == 0u) return ASTRAEA_OK;
    if (!keysIn || !keysOut || !valsIn || !valsOut || endBit < 1 || endBit > 64)
        return fail(ASTRAEA_ERR_INVALID, "radix_sort_pairs: bad argument");
    static std::map<int, std::pair<uint32_t*, size_t>> scratch;
    DeviceState* ds = nullptr;
    AstraeaStatus s = deviceState(&ds);
    if (s != ASTRAEA_OK) return s;
    uint32_t maxTiles = 0;
    const size_t words = sortScratchWords(n, &maxTiles);
    uint32_t* buf = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        auto& e = scratch[currentDevice()];
        if (e.second < words) {
            if (e.first) cudaFree(e.first);
            e.first = nullptr;
            e.second = 0;
            AG_CUDA(cudaMalloc(&e.first, words * sizeof(uint32_t)));
            e.second = words;
        }
        buf = e.first;
    }
    cudaStream_t st = stream();
    bool inA = true;
    AG_LAUNCH(radixSortPairs(keysIn, valsIn, keysOut, valsOut, n, endBit, buf, words, maxTiles, ds->status,
                             g_spinLimit.load(), KeySource::Array, nullptr, &inA, st));
    if (inA) {
        AG_CUDA(cudaMemcpyAsync(keysOut, keysIn, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        AG_CUDA(cudaMemcpyAsync(valsOut, valsIn, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    }
    return ASTRAEA_OK;
}

}  // extern "C"
