"""ctypes view of the C-ABI in include/astraea_gb300.h.

The two descriptor structs mirror the engine's ParticleBuffersDevice
(engine/types.hpp:114-161) and RadixBvhDevice (engine/sph_gravity.cuh:26-59)
member for member; FIELDS lists the 56 particle arrays in struct order with
their element types.
"""
import ctypes
import os

import numpy as np

PACKAGE_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PACKAGE_DIR, "libastraea_gb300.so")

# (name, numpy dtype) in ParticleBuffersDevice order.
_F32 = np.float32
FIELDS = [
    ("posX", _F32), ("posY", _F32), ("posZ", _F32),
    ("velX", _F32), ("velY", _F32), ("velZ", _F32),
    ("velHalfX", _F32), ("velHalfY", _F32), ("velHalfZ", _F32),
    ("accX", _F32), ("accY", _F32), ("accZ", _F32),
    ("mass", _F32), ("h", _F32), ("h0", _F32), ("rho", _F32), ("drhoDt", _F32),
    ("pressure", _F32), ("soundSpeed", _F32), ("u", _F32), ("duDt", _F32), ("tempK", _F32),
    ("radPowerW", _F32),
    ("sXX", _F32), ("sYY", _F32), ("sZZ", _F32), ("sXY", _F32), ("sXZ", _F32), ("sYZ", _F32),
    ("dSXX", _F32), ("dSYY", _F32), ("dSZZ", _F32), ("dSXY", _F32), ("dSXZ", _F32), ("dSYZ", _F32),
    ("damage", _F32), ("damageCbrt", _F32), ("dDamageCbrtDt", _F32), ("epsFail", _F32),
    ("divV", _F32), ("curlVX", _F32), ("curlVY", _F32), ("curlVZ", _F32),
    ("shepardC", _F32), ("surfFactor", _F32), ("phiGrav", _F32),
    ("materialId", np.uint8), ("phaseId", np.uint8), ("bodyId", np.uint8),
    ("originalId", np.uint32), ("tracerIndex", np.int32),
    ("tracerRestRadiusPsu", _F32), ("tracerRestNormalX", _F32), ("tracerRestNormalY", _F32),
    ("tracerRestNormalZ", _F32), ("tracerIsOcean", np.uint8),
]
FIELD_NAMES = [f for f, _ in FIELDS]
FIELD_DTYPES = dict(FIELDS)
assert len(FIELDS) == 56


class Particles(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_uint32), ("count", ctypes.c_uint32)] + [
        (name, ctypes.c_void_p) for name, _ in FIELDS
    ]


BVH_POINTERS = [
    "mortonCodes", "mortonCodesSorted", "indicesIn", "indicesSorted",
    "leftChild", "rightChild", "parent", "atomicVisited",
    "aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ",
    "nodeMass", "comX", "comY", "comZ", "nodeMaxH",
]


class RadixBvh(ctypes.Structure):
    _fields_ = (
        [("capacity", ctypes.c_uint32)]
        + [(name, ctypes.c_void_p) for name in BVH_POINTERS]
        + [("cubTempStorage", ctypes.c_void_p), ("cubTempBytes", ctypes.c_size_t),
           ("sceneBoundsOrdered", ctypes.c_void_p), ("sceneBoundsFloat", ctypes.c_void_p),
           ("livingFlags", ctypes.c_void_p), ("nodeComMass", ctypes.c_void_p),
           ("nodeMinExtent", ctypes.c_void_p), ("nodeMaxHPacked", ctypes.c_void_p)]
    )


assert ctypes.sizeof(Particles) == 8 + 56 * 8
assert ctypes.sizeof(RadixBvh) == 8 + 19 * 8 + 8 + 8 + 6 * 8

STATUS_NAMES = {0: "OK", 1: "CUDA", 2: "CAPACITY", 3: "INVALID", 4: "DEVICE_TIMEOUT", 5: "DEVICE_STATE"}
ASTRAEA_ERR_CAPACITY = 2
ASTRAEA_ERR_INVALID = 3

DEVFLAG_LOOKBACK_TIMEOUT = 0x1
DEVFLAG_NEIGHBOR_OVERFLOW = 0x2
DEVFLAG_STACK_OVERFLOW = 0x4

COUNTERS = ["gravity_interactions", "gravity_node_tests", "neighbor_entries", "gravity_rounds",
            "gravity_stack_peak", "fallback_walks", "neighbor_candidates", "gravity_undecided"]
# astraea_gb300_read_device_counters: the eight above, then the SPH pair counts
ALL_COUNTERS = COUNTERS + ["pass1_pairs", "pass2_pairs", "drift_pairs", "gravity_group_evals",
                           "gravity_bucket_leaves"]
# astraea_gb300_read_stage_times order (ASTRAEA_STAGE_*)
STAGES = ["refresh", "kick", "drift", "sort", "permute", "refit", "neighbours", "pass1", "eos", "gravity",
          "pass2", "kick_eos"]

# (symbol, argtypes) of every exported entry point, in header order.
class PclsFrameInfo(ctypes.Structure):
    """AstraeaPclsFrameInfo of include/astraea_gb300.h."""
    _fields_ = [("simTimeSec", ctypes.c_double), ("frameSeq", ctypes.c_uint64), ("dtSec", ctypes.c_float),
                ("tracerCount", ctypes.c_uint32), ("tracerGridRes", ctypes.c_uint32),
                ("livingBodyPresent", ctypes.c_int32), ("withSpeed", ctypes.c_int32),
                ("livingCom", ctypes.c_float * 3), ("sysCom", ctypes.c_float * 3)]


class TelemetryParams(ctypes.Structure):
    """AstraeaTelemetryParams of include/astraea_gb300.h."""
    _fields_ = [("targetRadiusPsu", ctypes.c_double), ("livingBodyPresent", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


_D3 = ctypes.c_double * 3


class Telemetry(ctypes.Structure):
    """AstraeaTelemetry of include/astraea_gb300.h (392 bytes)."""
    _fields_ = [("totalMassPsu", ctypes.c_double), ("sysComPsu", _D3),
                ("massBody0Psu", ctypes.c_double), ("comBody0Psu", _D3), ("velBody0Psu", _D3),
                ("massOtherPsu", ctypes.c_double), ("comOtherPsu", _D3), ("velOtherPsu", _D3),
                ("livingComPsu", _D3),
                ("kineticPsu", ctypes.c_double), ("potentialPsu", ctypes.c_double), ("internalPsu", ctypes.c_double),
                ("momentumPsu", _D3), ("angularMomentumPsu", _D3),
                ("maxTempK", ctypes.c_double), ("maxPressureGPa", ctypes.c_double), ("maxDamage", ctypes.c_double),
                ("radiatedPowerW", ctypes.c_double), ("spinLPsu", ctypes.c_double), ("spinIPsu", ctypes.c_double),
                ("remnantPsu", _D3), ("remnantVelPsu", _D3), ("remnantMassPsu", ctypes.c_double),
                ("remnantRadiusPsu", ctypes.c_double),
                ("boundPlanetMassPsu", ctypes.c_double), ("diskMassPsu", ctypes.c_double),
                ("ejectaMassPsu", ctypes.c_double), ("impactorBoundMassPsu", ctypes.c_double),
                ("remnantSeedIndex", ctypes.c_uint32), ("remnantIterations", ctypes.c_int32)]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out


_P = ctypes.POINTER(Particles)
_B = ctypes.POINTER(RadixBvh)
_U32 = ctypes.c_uint32
_F = ctypes.c_float
_VP = ctypes.c_void_p
class BodySpec(ctypes.Structure):
    """AstraeaBodySpec = BodyInitSpec (engine/types.hpp:60-67)."""
    _fields_ = [("archetype", _U32), ("relaxSteps", _U32), ("massKg", ctypes.c_double),
                ("surfaceTempK", ctypes.c_double), ("coreTempK", ctypes.c_double),
                ("spinOmegaRadS", ctypes.c_double)]


class RadialSample(ctypes.Structure):
    """AstraeaRadialSample = RadialProfileSample (engine/planet_builder.hpp:10-17)."""
    _fields_ = [("rM", ctypes.c_double), ("rhoKgM3", ctypes.c_double), ("pressurePa", ctypes.c_double),
                ("enclosedMassKg", ctypes.c_double), ("tempK", ctypes.c_double), ("material", _U32),
                ("reserved", _U32)]


class PlanetInfo(ctypes.Structure):
    _fields_ = [("equatorialRadiusM", ctypes.c_double), ("actualMassKg", ctypes.c_double),
                ("centralPressurePa", ctypes.c_double), ("tracerCount", _U32), ("profileSamples", _U32),
                ("shells", _U32), ("reserved", _U32)]


class FarFieldConfig(ctypes.Structure):
    _fields_ = [("thetaFar", ctypes.c_float), ("gamma", ctypes.c_float), ("gateTolerance", ctypes.c_float),
                ("gateTargets", _U32), ("pairsPerGroup", _U32), ("gateFp64Pairs", _U32)]


class FarFieldStats(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_uint64), ("fallbacks", ctypes.c_uint64), ("lastPairs", _U32), ("reserved", _U32),
                ("lastGateRms", ctypes.c_float), ("lastLoss", ctypes.c_float)]


FF_PARAMS = 6288


class Tuning(ctypes.Structure):
    _fields_ = [("gravityWarps", _U32), ("neighborWarps", _U32), ("gravityMs", ctypes.c_float),
                ("neighborMs", ctypes.c_float)]


SIGNATURES = [
    ("astraea_gb300_last_error", [], ctypes.c_char_p),
    ("astraea_gb300_abi_version", [], ctypes.c_int),
    ("astraea_gb300_set_stream", [_VP], ctypes.c_int),
    ("astraea_gb300_allocate_radix_bvh", [_B, _U32], ctypes.c_int),
    ("astraea_gb300_free_radix_bvh", [_B], ctypes.c_int),
    ("astraea_gb300_allocate_particle_buffers", [_P, _U32], ctypes.c_int),
    ("astraea_gb300_free_particle_buffers", [_P], ctypes.c_int),
    ("astraea_gb300_clear_stats", [_P], ctypes.c_int),
    ("astraea_gb300_sort_and_build_bvh", [_P, _P, _B], ctypes.c_int),
    ("astraea_gb300_sph_pass1_neighbors", [_P, _B], ctypes.c_int),
    ("astraea_gb300_evaluate_eos", [_P], ctypes.c_int),
    ("astraea_gb300_gravity_barnes_hut", [_P, _B, _F], ctypes.c_int),
    ("astraea_gb300_sph_pass2_forces", [_P, _B], ctypes.c_int),
    ("astraea_gb300_leapfrog_kick_half", [_P, _F, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_leapfrog_drift", [_P, _F, _B], ctypes.c_int),
    ("astraea_gb300_reduce_dt_psu", [_P, _F, _F, ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_pack_render_records", [_P, _VP, _VP, _F, _F, _F], ctypes.c_int),
    ("astraea_gb300_extract_tracers", [_P, _VP, _U32, _U32, _F, _F, _F, _F, _F, _F], ctypes.c_int),
    ("astraea_gb300_pcls_frame_bytes", [_U32, _U32, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    ("astraea_gb300_pack_pcls_frame", [_P, ctypes.POINTER(PclsFrameInfo), _VP, ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    ("astraea_gb300_reduce_telemetry", [_P, ctypes.POINTER(TelemetryParams), ctypes.POINTER(Telemetry)],
     ctypes.c_int),
    ("astraea_gb300_relax_single_body", [_P, _P, _B, _VP, _U32, ctypes.c_double, _U32,
                                         ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    ("astraea_gb300_solve_hydrostatic", [ctypes.POINTER(BodySpec), ctypes.POINTER(RadialSample), _U32,
                                         ctypes.POINTER(_U32), ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    ("astraea_gb300_build_planet", [ctypes.POINTER(BodySpec), _U32, _U32, _U32, ctypes.c_uint64, _P, _U32,
                                    ctypes.POINTER(PlanetInfo)], ctypes.c_int),
    ("astraea_gb300_ff_configure", [ctypes.POINTER(FarFieldConfig)], ctypes.c_int),
    ("astraea_gb300_ff_collect", [_P, _B, _F, _U32, _VP, _VP, _U32, ctypes.POINTER(_U32)], ctypes.c_int),
    ("astraea_gb300_ff_init", [ctypes.c_uint64], ctypes.c_int),
    ("astraea_gb300_ff_fit_output_scale", [_VP, _U32], ctypes.c_int),
    ("astraea_gb300_ff_gradients", [_VP, _VP, _U32, _VP, ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_ff_train_step", [_VP, _VP, _U32, _F, ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_ff_predict", [_VP, _U32, _VP], ctypes.c_int),
    ("astraea_gb300_ff_get_params", [_VP, _U32, _VP], ctypes.c_int),
    ("astraea_gb300_ff_set_params", [_VP, _U32, _VP], ctypes.c_int),
    ("astraea_gb300_ff_stats", [ctypes.POINTER(FarFieldStats)], ctypes.c_int),
    ("astraea_gb300_ff_profile", [_P, _B, _F, ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_autotune", [_P, _B, _F, ctypes.POINTER(Tuning)], ctypes.c_int),
    ("astraea_gb300_get_tuning", [_U32, ctypes.POINTER(Tuning)], ctypes.c_int),
    ("astraea_gb300_set_tuning", [_U32, ctypes.POINTER(Tuning)], ctypes.c_int),
    ("astraea_gb300_get_gravity_warps", [_U32, ctypes.c_int, ctypes.c_float, ctypes.POINTER(_U32)], ctypes.c_int),
    ("astraea_gb300_step", [_P, _P, _B, _F, _F, _F, _VP], ctypes.c_int),
    ("astraea_gb300_invalidate_step_cache", [_B], ctypes.c_int),
    ("astraea_gb300_reserve", [_B, _U32], ctypes.c_int),
    ("astraea_gb300_release_scratch", [_B], ctypes.c_int),
    ("astraea_gb300_radix_sort_pairs", [_VP, _VP, _VP, _VP, _U32, ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_radix_sort_pairs_noalloc", [_VP, _VP, _VP, _VP, _U32, ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_read_device_status", [ctypes.POINTER(_U32), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    ("astraea_gb300_read_device_counters", [ctypes.POINTER(ctypes.c_uint64), _U32, ctypes.POINTER(_U32)], ctypes.c_int),
    ("astraea_gb300_set_stage_timing", [ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_read_stage_times", [_B, ctypes.POINTER(_F), _U32, ctypes.POINTER(_U32)], ctypes.c_int),
    ("astraea_gb300_reset_device_status", [], ctypes.c_int),
    ("astraea_gb300_direct_gravity_f64", [_P, _VP, _U32, _VP, _VP], ctypes.c_int),
    ("astraea_gb300_measure_fp32_tflops", [ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_measure_fp32_peaks", [ctypes.POINTER(_F), ctypes.POINTER(_F)], ctypes.c_int),
    ("astraea_gb300_debug_gravity_group_counts", [_P, _B, _F, _VP], ctypes.c_int),
    ("astraea_gb300_debug_gravity_group_trace", [_P, _B, _F, _U32, _VP, _U32], ctypes.c_int),
    ("astraea_gb300_set_lookback_spin_limit", [_U32], ctypes.c_int),
    ("astraea_gb300_set_far_field", [ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_set_far_field_expansion", [_U32, _F], ctypes.c_int),
    ("astraea_gb300_set_node_rounding", [ctypes.c_int], ctypes.c_int),
    ("astraea_gb300_autotune_expansion", [_P, _B, _F, _VP, _U32, ctypes.POINTER(_U32), ctypes.POINTER(_F)],
     ctypes.c_int),
    ("astraea_gb300_debug_lookback_probe", [_U32, ctypes.POINTER(_U32)], ctypes.c_int),
]
EXPORTED_SYMBOLS = [name for name, _, _ in SIGNATURES]

_lib = None


def load_library(path=None):
    """Load libastraea_gb300.so (built by build_lib.py); raises when absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libastraea_gb300.so not built (%s); run __graft_entry__.build()" % p)
    lib = ctypes.CDLL(p)
    for name, args, res in SIGNATURES:
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.astraea_gb300_abi_version() != 1:
        raise RuntimeError("ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


class AstraeaError(RuntimeError):
    """Raised for a non-zero AstraeaStatus (the engine throws std::runtime_error)."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


def check(status):
    if status != 0:
        raise AstraeaError(status, load_library().astraea_gb300_last_error().decode(errors="replace"))
