"""Python driver of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/liboracle.so (oracle/oracle.cpp, built by
oracle/build_oracle.py) and runs the reference algorithm on host numpy
particle states.  Used by tests/ as the checker, by __graft_entry__.smoke()
and by bench.py's CPU baseline; never by the product library.

A host state is a dict field -> numpy array with the ParticleBuffersDevice
field names (astraea_gb300.abi.FIELDS).  The BVH is a dict of numpy arrays
sized like the engine allocates them (engine/sph_gravity.cu:1812-1842).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "astraea-impact-sim_gb300"))
from astraea_gb300 import abi  # noqa: E402  (struct layout of include/astraea_gb300.h)

_lib = None
_ref = None


def load(build=True):
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if build or not os.path.exists(path):
            sys.path.insert(0, HERE)
            import build_oracle
            path = build_oracle.build_oracle()
        _lib = ctypes.CDLL(path)
        P, B = ctypes.POINTER(abi.Particles), ctypes.POINTER(abi.RadixBvh)
        vp, u32, f = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float
        sig = {
            "oracle_eos_batch": [u32, vp, vp, vp, vp, vp, vp, vp, vp],
            "oracle_clear_stats": [P],
            "oracle_scene_bounds": [u32, vp, vp, vp, vp],
            "oracle_morton": [u32, vp, vp, vp, vp, vp],
            "oracle_sort_pairs": [u32, vp, vp, vp],
            "oracle_karras": [u32, vp, vp, vp, vp],
            "oracle_sort_and_build": [P, P, B, vp],
            "oracle_sph_pass1": [P, B],
            "oracle_sph_pass1_f64": [P, B],
            "oracle_evaluate_eos": [P],
            "oracle_gravity": [P, B, f, vp],
            "oracle_gravity_ff": [P, B, f, vp, vp],
            "oracle_gravity_f64": [P, B, f, vp],
            "oracle_gravity_group_counts": [P, B, f, vp],
            "oracle_gravity_expand": [P, B, f, vp, u32, f, vp],
            "oracle_node_moments": [P, B, vp],
            "oracle_direct_gravity_f64": [u32, vp, vp, vp, vp, vp, u32, vp, vp, vp],
            "oracle_sph_pass2": [P, B],
            "oracle_sph_pass2_f64": [P, B],
            "oracle_kick_half": [P, f, ctypes.c_int],
            "oracle_drift": [P, f, B, ctypes.c_int],
            "oracle_drift_f64": [P, f, B, ctypes.c_int],
            "oracle_reduce_dt": [P, f, f, vp],
            "oracle_step": [P, P, B, f, f, f],
            "oracle_step_f64": [P, P, B, f, f, f],
            "oracle_pack_render_records": [P, vp, vp, f, f, f],
            "oracle_extract_tracers": [P, vp, u32, f, f, f, f, f, f],
            "oracle_pcls_frame": [P, ctypes.POINTER(abi.PclsFrameInfo), vp, ctypes.c_size_t],
            "oracle_telemetry": [P, ctypes.POINTER(abi.TelemetryParams), ctypes.POINTER(abi.Telemetry)],
            "oracle_solve_hydrostatic": [ctypes.POINTER(abi.BodySpec), ctypes.POINTER(abi.RadialSample), u32,
                                         ctypes.POINTER(u32), ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double)],
            "oracle_build_planet": [ctypes.POINTER(abi.BodySpec), u32, u32, u32, ctypes.c_uint64, ctypes.c_int, P,
                                    u32, ctypes.POINTER(abi.PlanetInfo)],
        }
        for name, args in sig.items():
            getattr(_lib, name).argtypes = args
        _lib.oracle_reduce_dt.restype = f
        _lib.oracle_step.restype = f
        _lib.oracle_step_f64.restype = f
        _lib.oracle_pcls_frame.restype = ctypes.c_size_t
        _lib.oracle_set_group_stride.argtypes = [ctypes.c_int]
        _lib.oracle_set_r2_form.argtypes = [ctypes.c_int]
        _lib.oracle_cold_energy.restype = ctypes.c_double
        _lib.oracle_cold_energy.argtypes = [ctypes.c_int, ctypes.c_double]
    return _lib


def load_reference_eos():
    """The reference's own eos.cu built as host C++ (None where absent)."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libref_eos.so")
        if not os.path.exists(path):
            sys.path.insert(0, HERE)
            import build_oracle
            path = build_oracle.build_reference_eos()
        if path is None or not os.path.exists(path):
            return None
        try:
            _ref = ctypes.CDLL(path)
        except OSError:
            return None
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        _ref.ref_eos_batch.argtypes = [u32, vp, vp, vp, vp, vp, vp, vp, vp]
        _ref.ref_cold_energy.argtypes = [ctypes.c_int, ctypes.c_double]
        _ref.ref_cold_energy.restype = ctypes.c_double
    return _ref


def load_reference_pcls():
    """The reference's PCLS frame builder (server/binary_protocol.cpp) as a
    host library (None where the checkout or zlib is absent)."""
    sys.path.insert(0, HERE)
    import build_oracle
    path = build_oracle.build_reference_pcls()
    if path is None or not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    lib.ref_build_frame.argtypes = [vp, sz, vp, sz, vp, sz, ctypes.c_double, ctypes.c_uint64, ctypes.c_float,
                                    ctypes.c_int, ctypes.c_uint32, ctypes.c_int, vp, sz]
    lib.ref_build_frame.restype = sz
    return lib


PROFILE_COLUMNS = ("r", "rho", "P", "M", "T", "material")
_SAMPLE_DTYPE = np.dtype([("r", "f8"), ("rho", "f8"), ("P", "f8"), ("M", "f8"), ("T", "f8"), ("material", "u4"),
                          ("reserved", "u4")])


def solve_hydrostatic(spec):
    """The oracle's PlanetBuilder::solveHydrostatic1D: (profile columns,
    radius [m], central pressure [Pa])."""
    lib = load()
    cap = 16384
    buf = (abi.RadialSample * cap)()
    n, r, pc = ctypes.c_uint32(0), ctypes.c_double(0.0), ctypes.c_double(0.0)
    st = lib.oracle_solve_hydrostatic(ctypes.byref(spec), buf, cap, ctypes.byref(n), ctypes.byref(r), ctypes.byref(pc))
    if st != 0:
        raise RuntimeError("oracle_solve_hydrostatic status %d" % st)
    a = np.frombuffer(buf, dtype=_SAMPLE_DTYPE, count=n.value)
    return {k: np.array(a[k]) for k in PROFILE_COLUMNS}, r.value, pc.value


PLANET_FIELDS = ("posX", "posY", "posZ", "velX", "velY", "velZ", "velHalfX", "velHalfY", "velHalfZ", "mass", "h",
                 "h0", "rho", "u", "tempK", "epsFail", "materialId", "bodyId", "originalId", "tracerIndex",
                 "tracerRestRadiusPsu", "tracerRestNormalX", "tracerRestNormalY", "tracerRestNormalZ",
                 "tracerIsOcean")


def build_planet(spec, n, body_id=0, grid=0, seed=42, stable_ties=False):
    """The oracle's PlanetBuilder::buildPlanet + body upload: (state dict of
    the fields the builder writes, info dict)."""
    lib = load()
    hp = HostParticles({"posX": np.zeros(n, np.float32)}, capacity=n)
    s = hp.struct()
    info = abi.PlanetInfo()
    st = lib.oracle_build_planet(ctypes.byref(spec), n, body_id, grid, seed & 0xFFFFFFFFFFFFFFFF,
                                 int(bool(stable_ties)), ctypes.byref(s), 0, ctypes.byref(info))
    if st != 0:
        raise RuntimeError("oracle_build_planet status %d" % st)
    out = {k: hp.arrays[k][:n].copy() for k in PLANET_FIELDS}
    return out, {f: getattr(info, f) for f, _ in abi.PlanetInfo._fields_ if f != "reserved"}


def load_reference_planet():
    """The reference's PlanetBuilder (engine/planet_builder.cpp) as a host
    library behind oracle/ref_planet_capi.cpp (None where absent)."""
    sys.path.insert(0, HERE)
    import build_oracle
    path = build_oracle.build_reference_planet()
    if path is None or not os.path.exists(path):
        return None
    return ctypes.CDLL(path)


def reference_solve_hydrostatic(lib, spec, cap=20000):
    D = ctypes.c_double
    cols = [np.zeros(cap) for _ in range(5)]
    mat = np.zeros(cap, np.uint8)
    R, Pc, sec = D(), D(), D()
    n = lib.ref_solve_hydrostatic(int(spec.archetype), D(spec.massKg), D(spec.surfaceTempK), D(spec.coreTempK),
                                  D(spec.spinOmegaRadS), ctypes.c_uint32(cap), *[_ptr(c) for c in cols], _ptr(mat),
                                  ctypes.byref(R), ctypes.byref(Pc), ctypes.byref(sec))
    prof = {k: c[:n].copy() for k, c in zip(PROFILE_COLUMNS[:5], cols)}
    prof["material"] = mat[:n].astype(np.uint32)
    return prof, R.value, Pc.value, sec.value


def reference_build_planet(lib, spec, n, body_id=0, grid=0, seed=42):
    """Runs the reference's PlanetBuilder::buildPlanet; returns (fields,
    info) in the layout of build_planet (velHalf = vel, h = h0 and the
    zeroed fields added as the engine's upload writes them), and the
    reference's own wall time in info['seconds']."""
    D = ctypes.c_double
    names = ("posX", "posY", "posZ", "velX", "velY", "velZ", "mass", "h0", "rho", "u", "tempK", "epsFail")
    f = {k: np.zeros(n, np.float32) for k in names}
    t4n = ("tracerRestRadiusPsu", "tracerRestNormalX", "tracerRestNormalY", "tracerRestNormalZ")
    t4 = {k: np.zeros(n, np.float32) for k in t4n}
    mat, body, oce = np.zeros(n, np.uint8), np.zeros(n, np.uint8), np.zeros(n, np.uint8)
    tidx = np.zeros(n, np.int32)
    info = np.zeros(5)
    fp = (ctypes.c_void_p * 12)(*[f[k].ctypes.data for k in names])
    tp = (ctypes.c_void_p * 4)(*[t4[k].ctypes.data for k in t4n])
    rc = lib.ref_build_planet(int(spec.archetype), D(spec.massKg), D(spec.surfaceTempK), D(spec.coreTempK),
                              D(spec.spinOmegaRadS), ctypes.c_uint32(n), ctypes.c_uint32(body_id),
                              ctypes.c_uint32(grid), ctypes.c_uint64(seed), fp, _ptr(mat), _ptr(body), _ptr(tidx), tp,
                              _ptr(oce), _ptr(info))
    if rc != 0:
        raise RuntimeError("ref_build_planet failed")
    out = dict(f)
    out.update(t4)
    out.update({"velHalfX": f["velX"].copy(), "velHalfY": f["velY"].copy(), "velHalfZ": f["velZ"].copy(),
                "h": f["h0"].copy(), "materialId": mat, "bodyId": body, "tracerIndex": tidx, "tracerIsOcean": oce,
                "originalId": np.arange(n, dtype=np.uint32)})
    return out, {"equatorialRadiusM": info[0], "actualMassKg": info[1], "centralPressurePa": info[2],
                 "tracerCount": int(info[3]), "seconds": info[4]}


def random_render_state(n, tracer_count, seed=7):
    """Seeded particle state for the packing kernels, with the edge cases
    their clamps handle: non-finite and negative temperatures, pressures below
    the 1 kPa cut, damage outside [0, 1], zero density, tracer indices that are
    negative or >= tracer_count, particles sitting on the living COM."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    st = {k: (rng.normal(0.0, 2.0, n)).astype(f32) for k in ("posX", "posY", "posZ")}
    for k in ("velX", "velY", "velZ"):
        st[k] = (rng.normal(0.0, 1.0, n) * 10.0 ** rng.uniform(-3, 1, n)).astype(f32)
    st["tempK"] = (10.0 ** rng.uniform(0.0, 6.0, n)).astype(f32)
    st["pressure"] = (np.sign(rng.normal(size=n)) * 10.0 ** rng.uniform(-10, 2, n)).astype(f32)
    st["damage"] = rng.uniform(-0.3, 1.3, n).astype(f32)
    st["mass"] = (10.0 ** rng.uniform(-12, -3, n)).astype(f32)
    st["rho"] = (10.0 ** rng.uniform(-4, 1.5, n)).astype(f32)
    st["divV"] = rng.normal(0.0, 5.0, n).astype(f32)
    st["h"] = (10.0 ** rng.uniform(-4, -1, n)).astype(f32)
    st["materialId"] = rng.integers(0, 5, n).astype(np.uint8)
    st["phaseId"] = rng.integers(0, 6, n).astype(np.uint8)
    st["bodyId"] = rng.integers(0, 20, n).astype(np.uint8)
    bad = rng.choice(n, max(n // 64, 8), replace=False)
    st["tempK"][bad[0::4]] = np.nan
    st["tempK"][bad[1::4]] = -5.0
    st["pressure"][bad[2::4]] = np.inf
    st["damage"][bad[3::4]] = np.nan
    st["rho"][bad[:4]] = 0.0
    tr = np.full(n, -1, np.int32)
    owners = rng.choice(n, min(n, tracer_count + 16), replace=False)
    slots = rng.permutation(tracer_count + 16).astype(np.int32)
    tr[owners] = slots[: len(owners)]                 # some slots >= tracer_count: skipped
    st["tracerIndex"] = tr
    r = np.sqrt(st["posX"].astype(np.float64) ** 2 + st["posY"] ** 2 + st["posZ"] ** 2)
    st["tracerRestRadiusPsu"] = (r * rng.uniform(0.8, 1.2, n)).astype(f32)
    nrm = rng.normal(size=(3, n))
    nrm /= np.linalg.norm(nrm, axis=0)
    st["tracerRestNormalX"], st["tracerRestNormalY"], st["tracerRestNormalZ"] = nrm.astype(f32)
    st["tracerIsOcean"] = (rng.uniform(size=n) < 0.3).astype(np.uint8)
    st["posX"][owners[0]] = st["posY"][owners[0]] = st["posZ"][owners[0]] = 0.0   # r = 0 at the living COM
    return st


def frame_info(sim_time=0.0, frame_seq=0, dt_sec=0.0, tracer_count=0, grid_res=0, living=False, speed=True,
               living_com=(0.0, 0.0, 0.0), sys_com=(0.0, 0.0, 0.0)):
    fi = abi.PclsFrameInfo()
    fi.simTimeSec, fi.frameSeq, fi.dtSec = sim_time, frame_seq, dt_sec
    fi.tracerCount, fi.tracerGridRes = tracer_count, grid_res
    fi.livingBodyPresent, fi.withSpeed = int(bool(living)), int(bool(speed))
    fi.livingCom[:] = list(living_com)
    fi.sysCom[:] = list(sys_com)
    return fi


def pack_render_records(state, sys_com, speed=True):
    """engine/sph_gravity.cu:1670-1743 on a host state: (records u8[20N], speed u8[N] or None)."""
    lib = load()
    hp = HostParticles(state)
    n = hp.count
    rec = np.zeros(20 * n, np.uint8)
    spd = np.zeros(n, np.uint8) if speed else None
    s = hp.struct()
    lib.oracle_pack_render_records(ctypes.byref(s), _ptr(rec), _ptr(spd) if speed else None, *map(float, sys_com))
    return rec, spd


def extract_tracers(state, tracer_count, living_com, sys_com):
    """engine/sph_gravity.cu:1586-1668 + 2163-2187 on a host state: u8[40 T]."""
    lib = load()
    hp = HostParticles(state)
    out = np.zeros(40 * tracer_count, np.uint8)
    s = hp.struct()
    lib.oracle_extract_tracers(ctypes.byref(s), _ptr(out), tracer_count, *map(float, living_com),
                               *map(float, sys_com))
    return out


def telemetry(state, target_radius_psu, living_body_present=True):
    """engine/simulation.cpp:567-582, 948-1285 loops on a host state (dict)."""
    lib = load()
    hp = HostParticles(state)
    s = hp.struct()
    prm = abi.TelemetryParams(float(target_radius_psu), int(bool(living_body_present)), 0)
    out = abi.Telemetry()
    lib.oracle_telemetry(ctypes.byref(s), ctypes.byref(prm), ctypes.byref(out))
    return out.as_dict()


def pcls_frame(state, info):
    """Uncompressed PCLS frame (server/binary_protocol.cpp:76-87, 155-217)."""
    lib = load()
    hp = HostParticles(state)
    n, t = hp.count, info.tracerCount
    cap = 40 + 20 * n + 40 * t + n
    out = np.zeros(cap, np.uint8)
    s = hp.struct()
    size = lib.oracle_pcls_frame(ctypes.byref(s), ctypes.byref(info), _ptr(out), cap)
    return out[:size]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class HostParticles:
    """Owns numpy arrays and a ctypes Particles struct pointing at them."""

    def __init__(self, state, capacity=None):
        n = len(state["posX"])
        cap = max(capacity or n, 1)
        self.arrays = {}
        for name, dt in abi.FIELDS:
            a = np.zeros(cap, dtype=dt)
            if name in state:
                a[:n] = state[name][:n]
            elif name == "tracerIndex":
                a[:] = -1
            self.arrays[name] = a
        self.count = n
        self.capacity = cap

    def struct(self):
        s = abi.Particles()
        s.capacity, s.count = self.capacity, self.count
        for name in abi.FIELD_NAMES:
            setattr(s, name, self.arrays[name].ctypes.data)
        return s

    def rebind(self, s, by_ptr):
        self.arrays = {name: by_ptr[getattr(s, name)] for name in abi.FIELD_NAMES}
        self.count = s.count

    def state(self):
        return {k: v[: self.count].copy() for k, v in self.arrays.items()}


class HostBvh:
    def __init__(self, capacity):
        n = max(int(capacity), 1)
        nodes = 2 * n - 1
        self.a = {
            "mortonCodes": np.zeros(n, np.uint64), "mortonCodesSorted": np.zeros(n, np.uint64),
            "indicesIn": np.zeros(n, np.uint32), "indicesSorted": np.zeros(n, np.uint32),
            "leftChild": np.zeros(n, np.int32), "rightChild": np.zeros(n, np.int32),
            "parent": np.zeros(nodes, np.int32), "atomicVisited": np.zeros(n, np.uint32),
            "livingFlags": np.zeros(2, np.uint32), "sceneBoundsFloat": np.zeros(6, np.float32),
        }
        for f in ("aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ", "nodeMass", "comX",
                  "comY", "comZ", "nodeMaxH"):
            self.a[f] = np.zeros(nodes, np.float32)
        self.s = abi.RadixBvh()
        self.s.capacity = n
        for k, v in self.a.items():
            setattr(self.s, k, v.ctypes.data)


class Oracle:
    """Stage-by-stage CPU restatement on one host state (p, alt, bvh)."""

    def __init__(self, state, capacity=None):
        self.lib = load()
        self.p = HostParticles(state, capacity)
        self.alt = HostParticles({"posX": np.zeros(0, np.float32)}, self.p.capacity)
        self.alt.count = self.p.count
        self.bvh = HostBvh(self.p.capacity)
        self.bounds = np.zeros(6, np.float32)
        self.prev_dt = 0.0

    def _pp(self):
        return self.p.struct(), self.alt.struct()

    def clear_stats(self):
        s = self.p.struct()
        self.lib.oracle_clear_stats(ctypes.byref(s))

    def sort_and_build(self):
        sp, sa = self._pp()
        self.lib.oracle_sort_and_build(ctypes.byref(sp), ctypes.byref(sa), ctypes.byref(self.bvh.s), _ptr(self.bounds))
        by_ptr = {}
        for hp in (self.p, self.alt):
            for a in hp.arrays.values():
                by_ptr[a.ctypes.data] = a
        self.p.rebind(sp, by_ptr)
        self.alt.rebind(sa, by_ptr)

    def pass1(self, f64=False):
        s = self.p.struct()
        (self.lib.oracle_sph_pass1_f64 if f64 else self.lib.oracle_sph_pass1)(ctypes.byref(s), ctypes.byref(self.bvh.s))

    def eos(self):
        s = self.p.struct()
        self.lib.oracle_evaluate_eos(ctypes.byref(s))

    def gravity(self, theta=0.5, far_field=0, f64=False):
        """far_field 0: the reference kernel; 1: + quadrupole of accepted nodes.
        f64: the same interaction set with FP64 pair arithmetic and sums."""
        s = self.p.struct()
        cnt = np.zeros(1, np.uint64)
        if f64:
            self.lib.oracle_gravity_f64(ctypes.byref(s), ctypes.byref(self.bvh.s), float(theta), _ptr(cnt))
        elif far_field == 0:
            self.lib.oracle_gravity(ctypes.byref(s), ctypes.byref(self.bvh.s), float(theta), _ptr(cnt))
        else:
            S6 = self.node_moments()
            self.lib.oracle_gravity_ff(ctypes.byref(s), ctypes.byref(self.bvh.s), float(theta), _ptr(S6), _ptr(cnt))
        return int(cnt[0])

    def gravity_expand(self, theta=0.7, leaf_bucket=16, gamma=0.3):
        """The library's far-field mode 3 (see oracle_gravity_expand); returns
        (member-evaluated terms, expansion terms, bucket P-P terms)."""
        s = self.p.struct()
        S6 = self.node_moments()
        cnt = np.zeros(3, np.uint64)
        self.lib.oracle_gravity_expand(ctypes.byref(s), ctypes.byref(self.bvh.s), float(theta), _ptr(S6),
                                       int(leaf_bucket), float(gamma), _ptr(cnt))
        return int(cnt[0]), int(cnt[1]), int(cnt[2])

    def gravity_group_counts(self, theta=0.5):
        """The reference kernel; returns each group's interaction count."""
        s = self.p.struct()
        out = np.zeros(max((self.p.count + 31) // 32, 1), np.uint32)
        self.lib.oracle_gravity_group_counts(ctypes.byref(s), ctypes.byref(self.bvh.s), float(theta), _ptr(out))
        return out[: (self.p.count + 31) // 32].astype(np.int64)

    def node_moments(self):
        """Central second moments of the internal nodes, float32 (n-1, 6)."""
        s = self.p.struct()
        S6 = np.zeros((max(self.p.count - 1, 1), 6), np.float32)
        self.lib.oracle_node_moments(ctypes.byref(s), ctypes.byref(self.bvh.s), _ptr(S6))
        return S6

    def pass2(self, f64=False):
        s = self.p.struct()
        (self.lib.oracle_sph_pass2_f64 if f64 else self.lib.oracle_sph_pass2)(ctypes.byref(s), ctypes.byref(self.bvh.s))

    def kick(self, half_dt, clamp_thermal=False):
        s = self.p.struct()
        self.lib.oracle_kick_half(ctypes.byref(s), float(half_dt), int(bool(clamp_thermal)))

    def drift(self, dt, f64=False):
        s = self.p.struct()
        use = 1 if self.p.count >= 2 else 0
        (self.lib.oracle_drift_f64 if f64 else self.lib.oracle_drift)(ctypes.byref(s), float(dt),
                                                                      ctypes.byref(self.bvh.s), use)

    def reduce_dt(self, prev_dt, max_dt):
        s = self.p.struct()
        raw = np.zeros(1, np.float32)
        dt = self.lib.oracle_reduce_dt(ctypes.byref(s), float(prev_dt), float(max_dt), _ptr(raw))
        return float(dt), float(raw[0])

    def initial_forces(self, theta=0.5):
        self.clear_stats()
        self.sort_and_build()
        self.pass1()
        self.eos()
        self.gravity(theta)
        self.pass2()

    def step_f64(self, max_dt, theta=0.5):
        """The FP64 host path of one step (oracle_step_f64), in C."""
        sp, sa = self._pp()
        dt = self.lib.oracle_step_f64(ctypes.byref(sp), ctypes.byref(sa), ctypes.byref(self.bvh.s),
                                      float(self.prev_dt), float(max_dt), float(theta))
        by_ptr = {}
        for hp in (self.p, self.alt):
            for a in hp.arrays.values():
                by_ptr[a.ctypes.data] = a
        self.p.rebind(sp, by_ptr)
        self.alt.rebind(sa, by_ptr)
        self.prev_dt = float(dt)
        return float(dt)

    def step(self, max_dt, theta=0.5):
        dt, _ = self.reduce_dt(self.prev_dt, max_dt)
        self.prev_dt = dt
        self.kick(0.5 * dt)
        self.drift(dt)
        self.sort_and_build()
        self.pass1()
        self.eos()
        self.gravity(theta)
        self.pass2()
        self.kick(0.5 * dt)
        self.eos()
        return dt

    def state(self):
        return self.p.state()


def set_group_stride(k):
    """Tree-walking stages visit every k-th group only (CPU timing sample)."""
    load().oracle_set_group_stride(int(k))


def set_r2_form(k):
    """Rounding of |d|^2 (and of the dt candidate's multiply-adds) at the
    engine's decision points: 1 fma(dz, dz, fma(dx, dx, dy^2)), as the
    engine's compiled kernels round it (the default); 0 the unfused sequence;
    2 fma(dz, dz, fma(dy, dy, dx^2))."""
    load().oracle_set_r2_form(int(k))


def eos_batch(mat, rho, u, dmg, reference=False):
    """(P, cs, T, phase) of the oracle EOS, or of the reference's own when
    reference=True (None if that library is unavailable)."""
    lib = load_reference_eos() if reference else load()
    if lib is None:
        return None
    n = len(rho)
    mat = np.ascontiguousarray(mat, np.uint8)
    rho = np.ascontiguousarray(rho, np.float32)
    u = np.ascontiguousarray(u, np.float32)
    dmg = np.ascontiguousarray(dmg, np.float32)
    P, cs, T = (np.zeros(n, np.float32) for _ in range(3))
    ph = np.zeros(n, np.uint8)
    fn = lib.ref_eos_batch if reference else lib.oracle_eos_batch
    fn(n, _ptr(mat), _ptr(rho), _ptr(u), _ptr(dmg), _ptr(P), _ptr(cs), _ptr(T), _ptr(ph))
    return P, cs, T, ph


def direct_gravity_f64(state, targets):
    lib = load()
    n = len(state["posX"])
    t = np.ascontiguousarray(targets, np.uint32)
    acc = np.zeros((len(t), 3), np.float64)
    phi = np.zeros(len(t), np.float64)
    arrs = [np.ascontiguousarray(state[k], np.float32) for k in ("posX", "posY", "posZ", "mass", "h0")]
    lib.oracle_direct_gravity_f64(n, *[_ptr(a) for a in arrs], len(t), _ptr(t), _ptr(acc), _ptr(phi))
    return acc, phi


def sort_pairs(keys):
    lib = load()
    keys = np.ascontiguousarray(keys, np.uint64)
    n = len(keys)
    ks = np.zeros(n, np.uint64)
    perm = np.zeros(n, np.uint32)
    lib.oracle_sort_pairs(n, _ptr(keys), _ptr(ks), _ptr(perm))
    return ks, perm


def morton(x, y, z):
    lib = load()
    x, y, z = (np.ascontiguousarray(a, np.float32) for a in (x, y, z))
    n = len(x)
    b = np.zeros(6, np.float32)
    lib.oracle_scene_bounds(n, _ptr(x), _ptr(y), _ptr(z), _ptr(b))
    codes = np.zeros(n, np.uint64)
    lib.oracle_morton(n, _ptr(x), _ptr(y), _ptr(z), _ptr(b), _ptr(codes))
    return codes, b


def karras(codes_sorted):
    lib = load()
    c = np.ascontiguousarray(codes_sorted, np.uint64)
    n = len(c)
    left = np.zeros(max(n - 1, 1), np.int32)
    right = np.zeros(max(n - 1, 1), np.int32)
    parent = np.zeros(2 * n - 1, np.int32)
    lib.oracle_karras(n, _ptr(c), _ptr(left), _ptr(right), _ptr(parent))
    return left, right, parent


# ------------------------------------------------ learned far field (mode 2)
# The network of astraea_gb300_ff_* restated in numpy FP64: 16 -> 64 -> 64 ->
# 16, SiLU, loss = mean over rows and the first 12 outputs of
# (y - label / scale)^2.  With bf16=True the operands are rounded to bfloat16
# (round to nearest even) where the GPU kernels round them: inputs, weights,
# the hidden activations, and the backward signals dY, dZ2, dZ1 before they
# enter a product; sums stay FP64 here (FP32 on the GPU).
FF_IN, FF_HID, FF_OUT, FF_USED = 16, 64, 16, 12
FF_SHAPES = [("W1", (FF_IN, FF_HID)), ("b1", (FF_HID,)), ("W2", (FF_HID, FF_HID)), ("b2", (FF_HID,)),
             ("W3", (FF_HID, FF_OUT)), ("b3", (FF_OUT,))]


def bf16_round(a):
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def ff_unpack(params):
    out, off = {}, 0
    for name, shp in FF_SHAPES:
        k = int(np.prod(shp))
        out[name] = np.asarray(params[off:off + k], np.float64).reshape(shp)
        off += k
    return out


def ff_pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in FF_SHAPES])


def _silu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return z * s, s * (1.0 + z * (1.0 - s))


def ff_forward(params, X, bf16=False):
    P = ff_unpack(params)
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    x = r(X)
    z1 = x @ r(P["W1"]) + P["b1"]
    h1 = r(_silu(z1)[0])
    z2 = h1 @ r(P["W2"]) + P["b2"]
    h2 = r(_silu(z2)[0])
    y = h2 @ r(P["W3"]) + P["b3"]
    return y, (x, z1, h1, z2, h2)


def ff_loss_grad(params, scale, X, T, bf16=False):
    """(loss, gradient over the packed parameters) of one batch."""
    P = ff_unpack(params)
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    y, (x, z1, h1, z2, h2) = ff_forward(params, X, bf16)
    n = X.shape[0]
    t = np.asarray(T, np.float64)[:, :FF_USED] / np.asarray(scale, np.float64)[:FF_USED]
    d = np.zeros_like(y)
    d[:, :FF_USED] = y[:, :FF_USED] - t
    loss = float(np.sum(d * d) / (n * FF_USED))
    dy = 2.0 * d / (n * FF_USED)
    dyr = r(dy)
    g = {"b3": dy.sum(0), "W3": h2.T @ dyr}
    dz2 = (dyr @ r(P["W3"]).T) * _silu(z2)[1]
    dz2r = r(dz2)
    g["b2"] = dz2.sum(0)
    g["W2"] = h1.T @ dz2r
    dz1 = (dz2r @ r(P["W2"]).T) * _silu(z1)[1]
    dz1r = r(dz1)
    g["b1"] = dz1.sum(0)
    g["W1"] = x.T @ dz1r
    return loss, ff_pack(g)
