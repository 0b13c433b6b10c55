"""Host-side mirror of the ASTRAEA kernel interface over the CUDA C-ABI.

The functions below have the names, argument meaning and error behaviour of
astraea::cuda::* in engine/sph_gravity.cuh:61-92 (launchSortAndBuildBvh ->
sort_and_build_bvh, ...): they enqueue work on the CUDA stream and raise
AstraeaError where the engine throws std::runtime_error.  Device memory is
held in torch tensors (one per SoA field), passed to the library as the
C descriptors of include/astraea_gb300.h.  Every call goes to
libastraea_gb300.so; there is no other implementation behind them.
"""
import ctypes

import numpy as np
import torch

from . import abi

_TORCH_DTYPES = {np.float32: torch.float32, np.uint8: torch.uint8, np.uint32: torch.int32, np.int32: torch.int32}


def _torch_dtype(np_dtype):
    return _TORCH_DTYPES[np_dtype]


def lib():
    return abi.load_library()


class DeviceParticles:
    """ParticleBuffersDevice in torch tensors (engine/types.hpp:114-161)."""

    def __init__(self, capacity, device="cuda"):
        self.capacity = int(capacity)
        self.count = 0
        self.device = torch.device(device)
        self.arrays = {
            name: torch.zeros(max(self.capacity, 1), dtype=_torch_dtype(dt), device=self.device)
            for name, dt in abi.FIELDS
        }
        self.arrays["tracerIndex"].fill_(-1)

    def struct(self):
        s = abi.Particles()
        s.capacity = self.capacity
        s.count = self.count
        for name in abi.FIELD_NAMES:
            setattr(s, name, self.arrays[name].data_ptr())
        return s

    def upload(self, host, count=None):
        """Copy host arrays (dict name -> numpy) into the first `count` slots."""
        n = int(count if count is not None else len(host["posX"]))
        if n > self.capacity:
            raise abi.AstraeaError(2, "upload: count %d > capacity %d" % (n, self.capacity))
        self.count = n
        for name, dt in abi.FIELDS:
            if name in host:
                a = np.ascontiguousarray(host[name][:n]).astype(dt, copy=False)
                if dt == np.uint32:
                    a = a.view(np.int32)
                self.arrays[name][:n].copy_(torch.from_numpy(a))

    def download(self, fields=None):
        out = {}
        n = self.count
        for name in fields or abi.FIELD_NAMES:
            t = self.arrays[name][:n].cpu().numpy()
            if abi.FIELD_DTYPES[name] == np.uint32:
                t = t.view(np.uint32)
            out[name] = t
        return out


def _rebind_after_swap(p, alt, sp, salt):
    """Follow the pointer swap the library made in the structs."""
    by_ptr = {}
    for dp in (p, alt):
        for name, t in dp.arrays.items():
            by_ptr[t.data_ptr()] = t
    for dp, s in ((p, sp), (alt, salt)):
        for name in abi.FIELD_NAMES:
            dp.arrays[name] = by_ptr[getattr(s, name)]
        dp.count = s.count


class DeviceBvh:
    """RadixBvhDevice allocated by the library (allocateRadixBvh)."""

    def __init__(self, capacity):
        self.s = abi.RadixBvh()
        abi.check(lib().astraea_gb300_allocate_radix_bvh(ctypes.byref(self.s), int(capacity)))

    @property
    def capacity(self):
        return self.s.capacity

    def free(self):
        if self.s.capacity:
            abi.check(lib().astraea_gb300_free_radix_bvh(ctypes.byref(self.s)))

    def __del__(self):
        try:
            if self.s.capacity and abi._lib is not None:
                abi._lib.astraea_gb300_free_radix_bvh(ctypes.byref(self.s))
        except Exception:
            pass



class TorchBvh:
    """RadixBvhDevice whose arrays are caller-owned torch tensors, the way
    tests/cpp/test_gravity_sph.cpp:178-236 builds one with raw cudaMalloc.
    packed=False leaves the packed node arrays and the scene scratch NULL,
    like that test (the library then uses its own scratch)."""

    def __init__(self, capacity, packed=True):
        n = int(capacity)
        nodes = 2 * n
        dev = "cuda"
        z = lambda k, dt: torch.zeros(max(k, 1), dtype=dt, device=dev)
        self.t = {
            "mortonCodes": z(n, torch.int64), "mortonCodesSorted": z(n, torch.int64),
            "indicesIn": z(n, torch.int32), "indicesSorted": z(n, torch.int32),
            "leftChild": z(n, torch.int32), "rightChild": z(n, torch.int32),
            "parent": z(nodes, torch.int32), "atomicVisited": z(n, torch.int32),
        }
        for f in ("aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ", "nodeMass", "comX",
                  "comY", "comZ", "nodeMaxH"):
            self.t[f] = z(nodes, torch.float32)
        if packed:
            self.t["sceneBoundsOrdered"] = z(6, torch.int32)
            self.t["sceneBoundsFloat"] = z(6, torch.float32)
            self.t["livingFlags"] = z(2, torch.int32)
            for f in ("nodeComMass", "nodeMinExtent", "nodeMaxHPacked"):
                self.t[f] = z(4 * nodes, torch.float32)
        self.s = abi.RadixBvh()
        self.s.capacity = n
        for name, t in self.t.items():
            setattr(self.s, name, t.data_ptr())

    @property
    def capacity(self):
        return self.s.capacity

    def release(self):
        if self.t:
            abi.check(lib().astraea_gb300_release_scratch(ctypes.byref(self.s)))
            self.t = {}

    def __del__(self):
        try:
            if self.t and abi._lib is not None:
                abi._lib.astraea_gb300_release_scratch(ctypes.byref(self.s))
        except Exception:
            pass


# -------------------------------------------------------- engine entry points
def clear_stats(p):
    s = p.struct()
    abi.check(lib().astraea_gb300_clear_stats(ctypes.byref(s)))


def sort_and_build_bvh(p, alt, bvh):
    sp, salt = p.struct(), alt.struct()
    abi.check(lib().astraea_gb300_sort_and_build_bvh(ctypes.byref(sp), ctypes.byref(salt), ctypes.byref(bvh.s)))
    _rebind_after_swap(p, alt, sp, salt)


def sph_pass1_neighbors(p, bvh):
    s = p.struct()
    abi.check(lib().astraea_gb300_sph_pass1_neighbors(ctypes.byref(s), ctypes.byref(bvh.s)))


def evaluate_eos(p):
    s = p.struct()
    abi.check(lib().astraea_gb300_evaluate_eos(ctypes.byref(s)))


def gravity_barnes_hut(p, bvh, theta=0.5):
    s = p.struct()
    abi.check(lib().astraea_gb300_gravity_barnes_hut(ctypes.byref(s), ctypes.byref(bvh.s), float(theta)))


def gravity_group_counts(p, bvh, theta=0.5):
    """The gravity stage with each group's interaction count (int64 numpy
    array, one entry per group of 32 sorted particles)."""
    groups = (p.count + 31) // 32
    out = torch.zeros(max(groups, 1), dtype=torch.int32, device=p.device)
    sp = p.struct()
    abi.check(lib().astraea_gb300_debug_gravity_group_counts(ctypes.byref(sp), ctypes.byref(bvh.s), float(theta),
                                                            out.data_ptr()))
    return out[:groups].cpu().numpy().view(np.uint32).astype(np.int64)


def gravity_group_trace(p, bvh, group, theta=0.5, capacity=1 << 16):
    """The gravity stage recording what one group takes: the nodes it accepts
    as monopoles (>= 0) and the leaves it reaches (~particle), in walk order."""
    out = torch.zeros(capacity + 1, dtype=torch.int32, device=p.device)
    sp = p.struct()
    abi.check(lib().astraea_gb300_debug_gravity_group_trace(ctypes.byref(sp), ctypes.byref(bvh.s), float(theta),
                                                           int(group), out.data_ptr(), int(capacity)))
    a = out.cpu().numpy()
    return a[1:1 + min(int(a[0]), capacity)].astype(np.int64)


def sph_pass2_forces(p, bvh):
    s = p.struct()
    abi.check(lib().astraea_gb300_sph_pass2_forces(ctypes.byref(s), ctypes.byref(bvh.s)))


def leapfrog_kick_half(p, half_dt, include_xsph=False, clamp_thermal=False):
    s = p.struct()
    abi.check(lib().astraea_gb300_leapfrog_kick_half(ctypes.byref(s), float(half_dt), int(bool(include_xsph)),
                                                     int(bool(clamp_thermal))))


def leapfrog_drift(p, dt, bvh):
    s = p.struct()
    abi.check(lib().astraea_gb300_leapfrog_drift(ctypes.byref(s), float(dt), ctypes.byref(bvh.s) if bvh else None))


def reduce_dt_psu(p, prev_dt, max_dt):
    s = p.struct()
    out = ctypes.c_float(0.0)
    abi.check(lib().astraea_gb300_reduce_dt_psu(ctypes.byref(s), float(prev_dt), float(max_dt), ctypes.byref(out)))
    return out.value


def step(p, alt, bvh, prev_dt, max_dt, theta=0.5, out_dt_ptr=None):
    """Fused Simulation::step kernel sequence; returns without a sync."""
    sp, salt = p.struct(), alt.struct()
    abi.check(lib().astraea_gb300_step(ctypes.byref(sp), ctypes.byref(salt), ctypes.byref(bvh.s), float(prev_dt),
                                       float(max_dt), float(theta), out_dt_ptr))
    _rebind_after_swap(p, alt, sp, salt)


def pack_render_records(p, records, speed=None, sys_com=(0.0, 0.0, 0.0)):
    """launchPackRenderRecords: 20-byte records (uint8 tensor of 20 N) and,
    when `speed` is given, one speed byte per particle."""
    s = p.struct()
    abi.check(lib().astraea_gb300_pack_render_records(ctypes.byref(s), records.data_ptr(),
                                                      speed.data_ptr() if speed is not None else None,
                                                      *map(float, sys_com)))


def extract_tracers(p, records, tracer_count, grid_res=0, living_com=(0.0, 0.0, 0.0), sys_com=(0.0, 0.0, 0.0)):
    """launchExtractTracers: 40-byte tracer records (uint8 tensor of 40 T)."""
    s = p.struct()
    abi.check(lib().astraea_gb300_extract_tracers(ctypes.byref(s), records.data_ptr(), int(tracer_count),
                                                  int(grid_res), *map(float, living_com), *map(float, sys_com)))


def pcls_frame_bytes(n, tracer_count, with_speed=True):
    out = ctypes.c_size_t(0)
    abi.check(lib().astraea_gb300_pcls_frame_bytes(int(n), int(tracer_count), int(bool(with_speed)),
                                                   ctypes.byref(out)))
    return out.value


def pack_pcls_frame(p, info, frame):
    """One uncompressed PCLS frame into `frame` (uint8 device tensor);
    `info` is an abi.PclsFrameInfo.  Returns the frame size in bytes."""
    s = p.struct()
    size = ctypes.c_size_t(0)
    abi.check(lib().astraea_gb300_pack_pcls_frame(ctypes.byref(s), ctypes.byref(info), frame.data_ptr(),
                                                  frame.numel(), ctypes.byref(size)))
    return size.value


def reduce_telemetry(p, target_radius_psu, living_body_present=True):
    """The O(N) telemetry loops on the device; returns a dict of
    AstraeaTelemetry fields (PSU, FP64)."""
    s = p.struct()
    prm = abi.TelemetryParams(float(target_radius_psu), int(bool(living_body_present)), 0)
    out = abi.Telemetry()
    abi.check(lib().astraea_gb300_reduce_telemetry(ctypes.byref(s), ctypes.byref(prm), ctypes.byref(out)))
    return out.as_dict()


def relax_single_body(p, alt, bvh, anchor_temp=None, nominal_radius=1.0, steps=20):
    """Simulation::Impl::relaxLoadedSingleBody on the device; `anchor_temp`
    is a float64 CUDA tensor indexed by originalId (None: 288 K).  Returns
    v_rms / v_esc after the 4 diagnostic steps."""
    sp, salt = p.struct(), alt.struct()
    out = ctypes.c_double(0.0)
    ptr = anchor_temp.data_ptr() if anchor_temp is not None else None
    cnt = anchor_temp.numel() if anchor_temp is not None else 0
    try:
        abi.check(lib().astraea_gb300_relax_single_body(ctypes.byref(sp), ctypes.byref(salt), ctypes.byref(bvh.s),
                                                        ptr, int(cnt), float(nominal_radius), int(steps),
                                                        ctypes.byref(out)))
    finally:
        _rebind_after_swap(p, alt, sp, salt)
    return out.value


def direct_gravity_f64(p, targets):
    """FP64 direct-sum accelerations (N, 3) and potentials at the listed
    target indices (an int CUDA tensor), as float64 CUDA tensors."""
    t = targets.to(device="cuda", dtype=torch.int32).contiguous()
    acc = torch.empty((t.numel(), 3), dtype=torch.float64, device="cuda")
    phi = torch.empty(t.numel(), dtype=torch.float64, device="cuda")
    s = p.struct()
    abi.check(lib().astraea_gb300_direct_gravity_f64(ctypes.byref(s), t.data_ptr(), t.numel(), acc.data_ptr(),
                                                     phi.data_ptr()))
    return acc, phi


# makeDefaultBodySpec (engine/presets.cpp:9-88): mass [kg], surface and core
# temperature [K], spin [rad/s] of each archetype.
ARCHETYPES = ("LivingTerra", "IronCore", "OceanIce", "LavaIo", "GasGiant", "ProtoTheia")
ARCHETYPE_DEFAULTS = {
    0: (5.97219e24, 288.0, 5500.0, 7.292115e-5),
    1: (3.3011e23, 440.0, 3200.0, 1.24e-6),
    2: (4.0e24, 275.0, 3800.0, 5.0e-5),
    3: (2.0e24, 1550.0, 4200.0, 4.11e-5),
    4: (1.2e26, 165.0, 18000.0, 1.76e-4),
    5: (6.417e23, 240.0, 2200.0, 7.09e-5),
}


def body_spec(archetype, mass_kg=None, surface_temp_k=None, core_temp_k=None, spin=None, relax_steps=80):
    """AstraeaBodySpec with the archetype's defaults for every field not given."""
    a = ARCHETYPES.index(archetype) if isinstance(archetype, str) else int(archetype)
    m, ts, tc, w = ARCHETYPE_DEFAULTS.get(a, (1.0, 0.0, 0.0, 0.0))
    return abi.BodySpec(a, int(relax_steps), m if mass_kg is None else mass_kg,
                        ts if surface_temp_k is None else surface_temp_k,
                        tc if core_temp_k is None else core_temp_k, w if spin is None else spin)


def solve_hydrostatic(spec):
    """PlanetBuilder::solveHydrostatic1D on the host: (profile dict of numpy
    columns r, rho, P, M, T, material; radius [m]; central pressure [Pa])."""
    n, r, pc = ctypes.c_uint32(0), ctypes.c_double(0.0), ctypes.c_double(0.0)
    cap = 16384                                    # the shooting makes at most ~12,000 steps
    buf = (abi.RadialSample * cap)()
    st = lib().astraea_gb300_solve_hydrostatic(ctypes.byref(spec), buf, cap, ctypes.byref(n), ctypes.byref(r),
                                               ctypes.byref(pc))
    if st == abi.ASTRAEA_ERR_CAPACITY and n.value > cap:
        buf = (abi.RadialSample * n.value)()
        st = lib().astraea_gb300_solve_hydrostatic(ctypes.byref(spec), buf, n.value, ctypes.byref(n),
                                                   ctypes.byref(r), ctypes.byref(pc))
    abi.check(st)
    a = np.frombuffer(buf, dtype=np.dtype([("r", "f8"), ("rho", "f8"), ("P", "f8"), ("M", "f8"), ("T", "f8"),
                                           ("material", "u4"), ("reserved", "u4")]), count=n.value)
    prof = {k: np.array(a[k]) for k in ("r", "rho", "P", "M", "T", "material")}
    return prof, r.value, pc.value


def build_planet(spec, particle_count, p, offset=0, body_id=0, tracer_grid_res=0, seed=42):
    """PlanetBuilder::buildPlanet written straight into particles
    [offset, offset + particle_count) of p (DeviceParticles); p.count is
    raised to cover the body.  Returns the AstraeaPlanetInfo as a dict."""
    info = abi.PlanetInfo()
    s = p.struct()
    abi.check(lib().astraea_gb300_build_planet(ctypes.byref(spec), int(particle_count), int(body_id),
                                               int(tracer_grid_res), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                               ctypes.byref(s), int(offset), ctypes.byref(info)))
    p.count = max(p.count, int(offset) + int(particle_count))
    return {f: getattr(info, f) for f, _ in abi.PlanetInfo._fields_ if f != "reserved"}


# ------------------------------------------------- learned far field (mode 2)
def ff_configure(theta_far=0.8, gamma=0.3, gate_tolerance=0.0, gate_targets=64, pairs_per_group=64,
                 gate_fp64_pairs=False):
    cfg = abi.FarFieldConfig(float(theta_far), float(gamma), float(gate_tolerance), int(gate_targets),
                             int(pairs_per_group), int(bool(gate_fp64_pairs)))
    abi.check(lib().astraea_gb300_ff_configure(ctypes.byref(cfg)))


def ff_collect(p, bvh, theta=0.5, group_stride=1, capacity=1 << 20):
    """Training rows (features, labels) as float32 CUDA tensors (rows x 16)
    from the current tree (built in far-field mode 2)."""
    feat = torch.empty((capacity, 16), dtype=torch.float32, device="cuda")
    lab = torch.empty((capacity, 16), dtype=torch.float32, device="cuda")
    cnt = ctypes.c_uint32(0)
    s = p.struct()
    abi.check(lib().astraea_gb300_ff_collect(ctypes.byref(s), ctypes.byref(bvh.s), float(theta), int(group_stride),
                                             feat.data_ptr(), lab.data_ptr(), capacity, ctypes.byref(cnt)))
    return feat[:cnt.value], lab[:cnt.value]


def ff_init(seed=1):
    abi.check(lib().astraea_gb300_ff_init(int(seed)))


def ff_fit_output_scale(labels):
    labels = labels.contiguous()
    abi.check(lib().astraea_gb300_ff_fit_output_scale(labels.data_ptr(), labels.shape[0]))


def ff_gradients(features, labels):
    """(gradient of the 6,288 parameters as float32 numpy, loss)."""
    g = np.zeros(abi.FF_PARAMS, np.float32)
    loss = ctypes.c_float(0.0)
    features, labels = features.contiguous(), labels.contiguous()
    abi.check(lib().astraea_gb300_ff_gradients(features.data_ptr(), labels.data_ptr(), features.shape[0],
                                               g.ctypes.data, ctypes.byref(loss)))
    return g, loss.value


def ff_train_step(features, labels, lr, want_loss=True):
    loss = ctypes.c_float(0.0)
    abi.check(lib().astraea_gb300_ff_train_step(features.data_ptr(), labels.data_ptr(), features.shape[0],
                                                float(lr), ctypes.byref(loss) if want_loss else None))
    return loss.value if want_loss else None


def ff_predict(features):
    features = features.contiguous()
    out = torch.empty((features.shape[0], 16), dtype=torch.float32, device="cuda")
    abi.check(lib().astraea_gb300_ff_predict(features.data_ptr(), features.shape[0], out.data_ptr()))
    return out


def ff_get_params():
    p = np.zeros(abi.FF_PARAMS, np.float32)
    sc = np.zeros(16, np.float32)
    abi.check(lib().astraea_gb300_ff_get_params(p.ctypes.data, abi.FF_PARAMS, sc.ctypes.data))
    return p, sc


def ff_set_params(params, scale=None):
    p = np.ascontiguousarray(params, np.float32)
    sc = None if scale is None else np.ascontiguousarray(scale, np.float32)
    abi.check(lib().astraea_gb300_ff_set_params(p.ctypes.data, p.size, None if sc is None else sc.ctypes.data))


def ff_profile(p, bvh, theta=0.5):
    """Times (ms) of the parts of one mode-2 gravity call: walk, network,
    correction, gate spot check, fallback walk."""
    out = (ctypes.c_float * 5)()
    sp = p.struct()
    abi.check(lib().astraea_gb300_ff_profile(ctypes.byref(sp), ctypes.byref(bvh.s), float(theta), out))
    return dict(zip(("walk", "network", "correct", "gate", "fallback"), list(out)))


def ff_stats():
    st = abi.FarFieldStats()
    abi.check(lib().astraea_gb300_ff_stats(ctypes.byref(st)))
    return {f: getattr(st, f) for f, _ in abi.FarFieldStats._fields_ if f != "reserved"}


def train_far_field(states, theta=0.5, group_stride=1, steps=600, batch=8192, lr=2e-3, seed=1, capacity=1 << 20):
    """Trains the mode-2 network on the GPU from the solver's own trees:
    every state is uploaded, built in mode 2, and its recorded pairs are
    labelled by FP64 direct sums; then `steps` Adam steps on random batches
    (the library's forward / backward kernels).  Leaves the far-field mode
    as it was.  Returns (rows, loss history)."""
    feats, labs = [], []
    for st in states:
        n = len(st["posX"])
        p, alt, bvh = DeviceParticles(n), DeviceParticles(n), DeviceBvh(n)
        p.upload(st)
        alt.count = n
        set_far_field(2)
        try:
            sort_and_build_bvh(p, alt, bvh)
            f, l = ff_collect(p, bvh, theta, group_stride, capacity)
        finally:
            set_far_field(0)
        feats.append(f.clone())
        labs.append(l.clone())
        del p, alt, bvh
    X = torch.cat(feats)
    T = torch.cat(labs)
    ff_init(seed)
    ff_fit_output_scale(T)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    hist = []
    for k in range(steps):
        idx = torch.randint(0, X.shape[0], (min(batch, X.shape[0]),), device="cuda", generator=gen)
        want = (k % 50 == 0) or k == steps - 1
        loss = ff_train_step(X[idx].contiguous(), T[idx].contiguous(), lr, want_loss=want)
        if want:
            hist.append((k, loss))
    return X.shape[0], hist


# ------------------------------------------------------------- autotuning
def _tuning_dict(t):
    return {f: getattr(t, f) for f, _ in abi.Tuning._fields_}


def autotune(p, bvh, theta=0.5):
    """Chooses the warps per block of the gravity and neighbour walks on the
    current tree (built for p) and keeps the choice for this particle-count
    bucket; returns it.  The gravity walk tuned is the one the current
    far-field mode runs at theta; the other walks keep their own shapes."""
    t = abi.Tuning()
    s = p.struct()
    abi.check(lib().astraea_gb300_autotune(ctypes.byref(s), ctypes.byref(bvh.s), float(theta), ctypes.byref(t)))
    return _tuning_dict(t)


def get_tuning(count):
    t = abi.Tuning()
    abi.check(lib().astraea_gb300_get_tuning(int(count), ctypes.byref(t)))
    return _tuning_dict(t)


def set_tuning(count, gravity_warps=4, neighbor_warps=4):
    t = abi.Tuning(int(gravity_warps), int(neighbor_warps), 0.0, 0.0)
    abi.check(lib().astraea_gb300_set_tuning(int(count), ctypes.byref(t)))


def get_gravity_warps(count, far_field_mode, theta):
    """Warps per block of the gravity walk of that far-field mode at theta."""
    w = ctypes.c_uint32(0)
    abi.check(lib().astraea_gb300_get_gravity_warps(int(count), int(far_field_mode), float(theta), ctypes.byref(w)))
    return int(w.value)


def invalidate_step_cache(bvh):
    abi.check(lib().astraea_gb300_invalidate_step_cache(ctypes.byref(bvh.s)))


def reserve(bvh, capacity):
    abi.check(lib().astraea_gb300_reserve(ctypes.byref(bvh.s), int(capacity)))


def radix_sort_pairs(keys, vals, end_bit=64):
    """Stable sort of (int64 keys as unsigned, int32 values) torch tensors."""
    n = keys.numel()
    k_in, v_in = keys.clone(), vals.clone()
    k_out, v_out = torch.empty_like(keys), torch.empty_like(vals)
    abi.check(lib().astraea_gb300_radix_sort_pairs(k_in.data_ptr(), k_out.data_ptr(), v_in.data_ptr(),
                                                   v_out.data_ptr(), n, int(end_bit)))
    return k_out, v_out


def read_device_status():
    flags = ctypes.c_uint32(0)
    counters = (ctypes.c_uint64 * 8)()
    abi.check(lib().astraea_gb300_read_device_status(ctypes.byref(flags), counters))
    return flags.value, dict(zip(abi.COUNTERS, list(counters)))


def read_device_counters():
    """Every device counter since the last reset (ASTRAEA_COUNTER_* order)."""
    out = (ctypes.c_uint64 * len(abi.ALL_COUNTERS))()
    cnt = ctypes.c_uint32(0)
    abi.check(lib().astraea_gb300_read_device_counters(out, len(abi.ALL_COUNTERS), ctypes.byref(cnt)))
    return dict(zip(abi.ALL_COUNTERS, list(out)[: cnt.value]))


def set_stage_timing(enable):
    """Events between the fused step's stages (off by default; not during graph capture)."""
    abi.check(lib().astraea_gb300_set_stage_timing(1 if enable else 0))


def read_stage_times(bvh):
    """Stage times (ms) of the last timed fused step on this BVH, by stage name."""
    out = (ctypes.c_float * len(abi.STAGES))()
    cnt = ctypes.c_uint32(0)
    abi.check(lib().astraea_gb300_read_stage_times(ctypes.byref(bvh.s), out, len(abi.STAGES), ctypes.byref(cnt)))
    return dict(zip(abi.STAGES, list(out)[: cnt.value]))


def measure_fp32_tflops():
    out = ctypes.c_float(0.0)
    abi.check(lib().astraea_gb300_measure_fp32_tflops(ctypes.byref(out)))
    return out.value


def measure_fp32_peaks():
    """(scalar fmaf, packed fma.rn.f32x2) FP32 throughput in TFLOP/s."""
    a, b = ctypes.c_float(0.0), ctypes.c_float(0.0)
    abi.check(lib().astraea_gb300_measure_fp32_peaks(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def reset_device_status():
    abi.check(lib().astraea_gb300_reset_device_status())


def set_stream(stream):
    """Launch stream of every later library call (a torch.cuda.Stream, or
    None for the legacy default stream)."""
    abi.check(lib().astraea_gb300_set_stream(stream.cuda_stream if stream is not None else None))


def set_far_field(mode):
    """0: monopole (the engine's kernel), 1: + quadrupole, 2: + learned
    correction, 3: quadrupole with leaf buckets and group expansion."""
    abi.check(lib().astraea_gb300_set_far_field(int(mode)))


def autotune_expansion(p, bvh, theta, candidates=(8, 16, 24, 32)):
    """Far-field mode 3: times the gravity for each candidate leaf bucket and
    keeps the fastest; returns (bucket, {candidate: ms})."""
    c = (ctypes.c_uint32 * len(candidates))(*candidates)
    ms = (ctypes.c_float * len(candidates))()
    out = ctypes.c_uint32(0)
    sp = p.struct()
    abi.check(lib().astraea_gb300_autotune_expansion(ctypes.byref(sp), ctypes.byref(bvh.s), float(theta), c,
                                                    len(candidates), ctypes.byref(out), ms))
    return out.value, dict(zip(candidates, list(ms)))


def set_node_rounding(mode):
    """0: node masses and COMs from exact moment sums (default); 1: the
    engine's FP32 bottom-up rounding (its exact node data and opening
    decisions).  Applies to later builds."""
    abi.check(lib().astraea_gb300_set_node_rounding(int(mode)))


def set_far_field_expansion(leaf_bucket=16, gamma=0.3):
    """Far-field mode 3: leaf bucket size (0..32) and the group-expansion gamma."""
    abi.check(lib().astraea_gb300_set_far_field_expansion(int(leaf_bucket), float(gamma)))


def set_lookback_spin_limit(limit):
    abi.check(lib().astraea_gb300_set_lookback_spin_limit(int(limit)))


class Simulation:
    """Device state + step driver, the part of engine/simulation.cpp that
    drives the hot path: upload (uploadHostStateToDevice :468-523), initial
    forces (evaluateInitialForcesOnDevice :525-536) and step() (:1711-1753)."""

    def __init__(self, capacity):
        self.p = DeviceParticles(capacity)
        self.alt = DeviceParticles(capacity)
        self.bvh = DeviceBvh(capacity)
        self.prev_dt = 0.0
        self.sim_time = 0.0
        self._dt_host = torch.zeros(1, dtype=torch.float32).pin_memory()

    def load_state(self, host):
        self.p.upload(host)
        self.alt.count = self.p.count
        for f in ("velHalfX", "velHalfY", "velHalfZ"):
            src = "vel" + f[-1]
            self.p.arrays[f][: self.p.count].copy_(self.p.arrays[src][: self.p.count])
        for f in ("pressure", "soundSpeed", "phaseId"):
            self.p.arrays[f].zero_()
        clear_stats(self.p)
        self.prev_dt = 0.0
        self.sim_time = 0.0

    def evaluate_initial_forces(self, theta=0.5):
        clear_stats(self.p)
        sort_and_build_bvh(self.p, self.alt, self.bvh)
        sph_pass1_neighbors(self.p, self.bvh)
        evaluate_eos(self.p)
        gravity_barnes_hut(self.p, self.bvh, theta)
        sph_pass2_forces(self.p, self.bvh)
        torch.cuda.synchronize()

    def step_stagewise(self, max_dt, theta=0.5):
        """The engine's step() as the sequence of stage entry points."""
        dt = reduce_dt_psu(self.p, self.prev_dt, max_dt)
        self.prev_dt = dt
        leapfrog_kick_half(self.p, 0.5 * dt, True, False)
        leapfrog_drift(self.p, dt, self.bvh)
        sort_and_build_bvh(self.p, self.alt, self.bvh)
        sph_pass1_neighbors(self.p, self.bvh)
        evaluate_eos(self.p)
        gravity_barnes_hut(self.p, self.bvh, theta)
        sph_pass2_forces(self.p, self.bvh)
        leapfrog_kick_half(self.p, 0.5 * dt, False, False)
        evaluate_eos(self.p)
        self.sim_time += dt
        return dt

    def step(self, max_dt, theta=0.5, sync=True):
        """Fused step; dt stays on the device.  Returns dt when sync."""
        step(self.p, self.alt, self.bvh, self.prev_dt, max_dt, theta, self._dt_host.data_ptr())
        if sync:
            torch.cuda.synchronize()
            dt = float(self._dt_host[0])
            self.prev_dt = dt
            self.sim_time += dt
            return dt
        return None

    def state(self, fields=None):
        return self.p.download(fields)


class Ensemble:
    """Independent impacts stepped together (the batched-ensemble workload).

    Each instance is a Simulation with its own BVH workspace.  `capture()`
    records two fused steps of every instance into one CUDA graph, each
    instance on its own stream (forked from and joined to the capture
    stream), so one `replay()` advances every instance by two steps with a
    single launch and the small instances run side by side.  Two steps are
    captured because a fused step flips the device dt slots and swaps the
    particle buffers: after two the graph's pointers and slots are where
    they started, so the same graph can be replayed again and again."""

    def __init__(self, states, max_dt, theta=0.5, autotune_walks=True):
        self.max_dt, self.theta = max_dt, theta
        self.sims = []
        self.tuning = {}
        for st in states:
            n = len(st["posX"])
            sim = Simulation(n)
            sim.load_state(st)
            reserve(sim.bvh, n)
            sim.evaluate_initial_forces(theta)
            bucket = n.bit_length() - 1
            if autotune_walks and bucket not in self.tuning:
                # the first instance of each power-of-two size tunes the walks for all of them
                self.tuning[bucket] = autotune(sim.p, sim.bvh, theta)
                sim.evaluate_initial_forces(theta)
            self.sims.append(sim)
        self.dt = torch.zeros(2 * len(states), dtype=torch.float32).pin_memory()
        self.streams = [torch.cuda.Stream() for _ in states]
        self.graph = None

    @property
    def particles(self):
        return sum(s.p.count for s in self.sims)

    def step_sequential(self, steps=1):
        """Eager fused steps, instance after instance, on the default stream."""
        for _ in range(steps):
            for k, sim in enumerate(self.sims):
                step(sim.p, sim.alt, sim.bvh, sim.prev_dt, self.max_dt, self.theta, self.dt[2 * k:].data_ptr())

    def capture(self):
        self.step_sequential(2)                   # step caches valid, device dt state primed
        torch.cuda.synchronize()
        cap = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(g, stream=cap):
                fork = torch.cuda.Event()
                fork.record(cap)
                for s in self.streams:           # every branch starts at the same point
                    s.wait_event(fork)
                for k, sim in enumerate(self.sims):
                    set_stream(self.streams[k])
                    for j in range(2):
                        step(sim.p, sim.alt, sim.bvh, sim.prev_dt, self.max_dt, self.theta,
                             self.dt[2 * k + j:].data_ptr())
                for s in self.streams:           # joined only after all branches are issued
                    cap.wait_stream(s)
        finally:
            set_stream(None)
        self.graph = g
        return g

    def replay(self, times=1):
        """Advance every instance by 2 * times steps."""
        for _ in range(times):
            self.graph.replay()
