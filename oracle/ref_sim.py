"""The reference engine's own Simulation on the CPU (TEST INFRASTRUCTURE ONLY).

Loads oracle/_ref/libref_sim.so (oracle/ref_sim_harness.cpp: engine/
simulation.cpp compiled from the reference checkout with a host stand-in for
the CUDA runtime and the oracle as its kernels; built by
oracle/build_oracle.py where the checkout exists).  Used to generate the
golden telemetry and relaxation vectors of tests/golden/sim_reference.npz
(tests/golden/make_sim_golden.py); nothing on the GPU machines needs it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_sim.so")

# TelemetrySnapshot (engine/types.hpp:81-111) flattened by the harness, in order.
SNAPSHOT_FIELDS = [
    "frameSeq", "simTimeSec", "dtSec", "outcome", "kineticEnergyJ", "potentialEnergyJ", "internalEnergyJ",
    "radiatedEnergyJ", "totalEnergyJ", "initialTotalEnergyJ", "energyDriftRel", "momentumX", "momentumY",
    "momentumZ", "angularMomentumX", "angularMomentumY", "angularMomentumZ", "virialRatio", "maxTempK",
    "maxPressureGPa", "boundMassFrac", "diskMassFrac", "ejectaMassFrac", "qRatioQrd", "livingBodyComKmX",
    "livingBodyComKmY", "livingBodyComKmZ", "livingBodyRadiusKm", "livingBodySpinRadS", "impactorComKmX",
    "impactorComKmY", "impactorComKmZ", "particleCount", "livingBodyPresent"]
CONTEXT_FIELDS = ["targetRadiusPsu", "impactorRadiusPsu", "livingBodyPresent", "hasImpacted", "qRatioQrd",
                  "impactParamB", "impactVelocityRatioVesc", "targetSpinOmegaRadS", "frameSeq", "simTimeSec",
                  "radiatedEnergyJ", "initialTotalEnergyJ", "sumRadPowerW"]

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import build_oracle
            if build_oracle.build_reference_sim() is None:
                return None
        lib = ctypes.CDLL(LIB)
        vp, u32, d = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double
        lib.refsim_create.restype = vp
        lib.refsim_create.argtypes = [u32]
        lib.refsim_destroy.argtypes = [vp]
        lib.refsim_last_error.restype = ctypes.c_char_p
        lib.refsim_load_preset.argtypes = [vp, ctypes.c_char_p, u32, ctypes.c_int, ctypes.c_uint64]
        lib.refsim_step.argtypes = [vp, d, vp]
        lib.refsim_compute_telemetry.argtypes = [vp, vp]
        lib.refsim_count.argtypes = [vp]
        lib.refsim_count.restype = u32
        lib.refsim_context.argtypes = [vp, vp]
        lib.refsim_get_particles.argtypes = [vp, vp]
        lib.refsim_set_particles.argtypes = [vp, vp]
        lib.refsim_relax_loaded.argtypes = [vp, vp, vp, d, u32, ctypes.POINTER(d)]
        _lib = lib
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference Simulation: %s" % _lib.refsim_last_error().decode())


class RefSimulation:
    """astraea::Simulation of the reference engine, running on the CPU."""

    def __init__(self, max_particles):
        import oracle
        self._oracle = oracle
        self.lib = load()
        if self.lib is None:
            raise RuntimeError("the reference Simulation harness is not built (no reference checkout)")
        self.h = self.lib.refsim_create(int(max_particles))
        if not self.h:
            raise RuntimeError(self.lib.refsim_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.refsim_destroy(self.h)
            self.h = None

    def load_preset(self, name, particles, relax_steps=-1, seed=42):
        _check(self.lib.refsim_load_preset(self.h, name.encode(), int(particles), int(relax_steps), int(seed)))

    def step(self, max_dt_sec=5.0):
        out = np.zeros(len(SNAPSHOT_FIELDS), np.float64)
        _check(self.lib.refsim_step(self.h, float(max_dt_sec), out.ctypes.data))
        return dict(zip(SNAPSHOT_FIELDS, out))

    def telemetry(self):
        out = np.zeros(len(SNAPSHOT_FIELDS), np.float64)
        _check(self.lib.refsim_compute_telemetry(self.h, out.ctypes.data))
        return dict(zip(SNAPSHOT_FIELDS, out))

    def context(self):
        out = np.zeros(len(CONTEXT_FIELDS), np.float64)
        self.lib.refsim_context(self.h, out.ctypes.data)
        return dict(zip(CONTEXT_FIELDS, out))

    def state(self):
        n = self.lib.refsim_count(self.h)
        hp = self._oracle.HostParticles({"posX": np.zeros(n, np.float32)}, max(n, 1))
        s = hp.struct()
        _check(self.lib.refsim_get_particles(self.h, ctypes.byref(s)))
        hp.count = n
        return hp.state()

    def set_state(self, state):
        hp = self._oracle.HostParticles(state)
        s = hp.struct()
        _check(self.lib.refsim_set_particles(self.h, ctypes.byref(s)))

    def relax_loaded(self, body, anchor_temp, nominal_radius_psu, steps):
        """relaxLoadedSingleBody on `body` (a state dict); returns (relaxed
        state, v_rms / v_esc)."""
        hp = self._oracle.HostParticles(body)
        s = hp.struct()
        anchors = np.ascontiguousarray(anchor_temp, np.float64)
        v = ctypes.c_double(0.0)
        _check(self.lib.refsim_relax_loaded(self.h, ctypes.byref(s), anchors.ctypes.data, float(nominal_radius_psu),
                                            int(steps), ctypes.byref(v)))
        return hp.state(), float(v.value)
