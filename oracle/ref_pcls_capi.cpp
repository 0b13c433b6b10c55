// ref_pcls_capi.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C entry point over the reference's own PCLS frame builder
// (server/binary_protocol.cpp:155-217), so the oracle's frame encoding can be
// checked against it and golden frames can be generated.  Built only by
// oracle/build_oracle.py, together with server/binary_protocol.cpp compiled
// straight from the reference checkout; the result goes to oracle/_ref/,
// which is never committed.
#include <cstdint>
#include <cstring>
#include <vector>

#include "binary_protocol.hpp"

extern "C" {

// Returns the frame size, or 0 when `cap` is too small.
size_t ref_build_frame(const uint8_t* particles, size_t particleBytes, const uint8_t* tracers, size_t tracerBytes,
                       const uint8_t* speed, size_t speedLen, double simTimeSec, uint64_t frameSeq, float dtSec,
                       int livingBodyPresent, uint32_t tracerGridRes, int compress, uint8_t* out, size_t cap) {
    astraea::TelemetrySnapshot snap;
    snap.simTimeSec = simTimeSec;
    snap.frameSeq = frameSeq;
    snap.dtSec = dtSec;
    snap.livingBodyPresent = livingBodyPresent != 0;
    snap.tracerGridRes = tracerGridRes;
    std::vector<uint8_t> pb(particles, particles + particleBytes);
    std::vector<uint8_t> tb(tracers, tracers + tracerBytes);
    std::vector<uint8_t> sb;
    if (speed != nullptr) sb.assign(speed, speed + speedLen);
    const std::vector<uint8_t> f =
        astraea::server::buildBinaryFrame(snap, pb, tb, speed != nullptr ? &sb : nullptr, compress != 0);
    if (f.size() > cap) return 0;
    std::memcpy(out, f.data(), f.size());
    return f.size();
}

}  // extern "C"
