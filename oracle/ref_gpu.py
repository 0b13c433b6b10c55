"""Runs the reference engine's own CUDA kernels on the GPU (TEST INFRASTRUCTURE ONLY).

oracle/_ref/ref_kernels_sm100.cubin is engine/eos.cu + engine/sph_gravity.cu
compiled for sm_100 from the reference checkout (oracle/build_oracle.py).
This module loads it with the CUDA driver API and launches its kernels with
the grids, blocks and argument lists of the reference's host launchers
(engine/sph_gravity.cu:1996-2161).  The one host-side piece it does not have
is CUB: the Morton codes are sorted with torch's stable sort (ties keep the
ascending original index -- the contract of cub::DeviceRadixSort::SortPairs
used at engine/sph_gravity.cu:2042).

Uses:
  python oracle/ref_gpu.py golden OUT.npz   -- stage-by-stage outputs of the
      reference on the small two-sphere scene (tests/golden/ref_stages.npz)
  python oracle/ref_gpu.py golden_render OUT.npz   -- the reference's render
      and tracer packing kernels on a seeded edge-case state
      (tests/golden/render_records.npz)
  python oracle/ref_gpu.py bench N STEPS WARMUP  -- the reference's GPU step
      time (gpuStepMs span, engine/simulation.cpp:1719-1739) on the
      differentiated-impact workload, one JSON line
"""
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "astraea-impact-sim_gb300"))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels_sm100.cubin")

KERNELS = {
    "init": "initSceneBoundsKernel", "reduce": "reduceSceneBoundsKernel", "finalize": "finalizeSceneBoundsKernel",
    "morton": "computeMortonCodesKernel", "permute": "permuteParticlesKernel",
    "karras": "initLeavesAndBuildKarrasKernel", "refit": "bottomUpBvhMomentsKernel", "clear": "clearStatsKernel",
    "pass1": "sphPass1KernelILb1E", "eos": "evaluateEosKernel", "gravity": "gravityBarnesHutKernelILb1E",
    "pass2": "sphPass2KernelILb1E", "kick": "leapfrogKickHalfKernel", "drift": "leapfrogDriftKernelILb1E",
    "dt": "reduceDtMinKernel", "render": "packRenderRecordsKernel", "tracers": "extractTracersKernel",
}


class RefKernels:
    def __init__(self, path=CUBIN):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")          # primary context current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        cnt = ctypes.c_uint()
        self._check(self.cu.cuModuleGetFunctionCount(ctypes.byref(cnt), self.mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * cnt.value)()
        self._check(self.cu.cuModuleEnumerateFunctions(funcs, cnt, self.mod), "cuModuleEnumerateFunctions")
        names = {}
        for f in funcs:
            nm = ctypes.c_char_p()
            self._check(self.cu.cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            names[nm.value.decode()] = f
        self.f = {}
        for key, frag in KERNELS.items():
            hits = [n for n in names if frag in n]
            if len(hits) != 1:
                raise RuntimeError("kernel %s: %d matches among %d functions" % (frag, len(hits), len(names)))
            self.f[key] = ctypes.c_void_p(names[hits[0]])

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed with CUresult %d" % (what, rc))

    def launch(self, key, grid, block, *args):
        holders = []
        ptrs = (ctypes.c_void_p * len(args))()
        for k, a in enumerate(args):
            holders.append(a)
            ptrs[k] = ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
        self._check(self.cu.cuLaunchKernel(self.f[key], grid, 1, 1, block, 1, 1, 0, None, ptrs, None),
                    "cuLaunchKernel " + key)


def grid(n, b):
    return (n + b - 1) // b


class RefEngine:
    """The reference's launch wrappers, restated host side over its kernels."""

    def __init__(self, n, kernels=None):
        import torch
        from astraea_gb300 import engine
        self.torch = torch
        self.K = kernels or RefKernels()
        self.p = engine.DeviceParticles(n)
        self.alt = engine.DeviceParticles(n)
        self.bvh = engine.TorchBvh(n, packed=True)
        self.dt_bits = torch.zeros(1, dtype=torch.int32, device="cuda")

    def U32(self, v):
        return ctypes.c_uint32(v)

    def sort_and_build(self):                                  # sph_gravity.cu:1996-2061
        from astraea_gb300 import engine
        torch = self.torch
        n = self.p.count
        b = self.bvh
        sp, salt = self.p.struct(), self.alt.struct()
        bo, bf, lf = (ctypes.c_void_p(b.s.sceneBoundsOrdered), ctypes.c_void_p(b.s.sceneBoundsFloat),
                      ctypes.c_void_p(b.s.livingFlags))
        self.K.launch("init", 1, 1, bo, lf)
        self.K.launch("reduce", min(grid(n, 256), 512), 256, ctypes.c_void_p(sp.posX), ctypes.c_void_p(sp.posY),
                      ctypes.c_void_p(sp.posZ), self.U32(n), bo)
        self.K.launch("finalize", 1, 8, bo, bf)
        self.K.launch("morton", grid(n, 256), 256, ctypes.c_void_p(sp.posX), ctypes.c_void_p(sp.posY),
                      ctypes.c_void_p(sp.posZ), bf, self.U32(n), ctypes.c_void_p(b.s.mortonCodes),
                      ctypes.c_void_p(b.s.indicesIn))
        codes = b.t["mortonCodes"][:n]
        ks, order = torch.sort(codes, stable=True)
        b.t["mortonCodesSorted"][:n] = ks
        b.t["indicesSorted"][:n] = b.t["indicesIn"][:n][order]
        self.K.launch("permute", grid(n, 256), 256, sp, salt, ctypes.c_void_p(b.s.indicesSorted), self.U32(n))
        # pointer swap p <-> alt (sph_gravity.cu:1745-1784, 2051-2052)
        self.p.arrays, self.alt.arrays = self.alt.arrays, self.p.arrays
        self.alt.count = self.p.count
        sp = self.p.struct()
        self.K.launch("karras", grid(n, 256), 256, sp, b.s, self.U32(n), lf)
        if n >= 2:
            self.K.launch("refit", grid(n, 256), 256, b.s, self.U32(n))

    def clear(self):
        self.K.launch("clear", grid(self.p.count, 256), 256, self.p.struct(), self.U32(self.p.count))

    def pass1(self):
        self.K.launch("pass1", grid(self.p.count, 128), 128, self.p.struct(), self.bvh.s, self.U32(self.p.count))

    def eos(self):
        self.K.launch("eos", grid(self.p.count, 256), 256, self.p.struct(), self.U32(self.p.count))

    def gravity(self, theta=0.5):
        t2 = max(0.0, theta) ** 2
        self.K.launch("gravity", grid(self.p.count, 128), 128, self.p.struct(), self.bvh.s, self.U32(self.p.count),
                      ctypes.c_float(np.float32(max(0.0, theta)) * np.float32(max(0.0, theta))))

    def pass2(self):
        self.K.launch("pass2", grid(self.p.count, 128), 128, self.p.struct(), self.bvh.s, self.U32(self.p.count),
                      ctypes.c_void_p(self.bvh.s.livingFlags))

    def kick(self, half_dt, include_xsph, clamp):
        self.K.launch("kick", grid(self.p.count, 256), 256, self.p.struct(), self.U32(self.p.count),
                      ctypes.c_float(half_dt), ctypes.c_bool(include_xsph), ctypes.c_bool(clamp))

    def drift(self, dt):
        n = self.p.count
        self.K.launch("drift", grid(n, 128), 128, self.p.struct(), self.bvh.s, self.U32(n), ctypes.c_float(dt),
                      ctypes.c_bool(n >= 2))

    def reduce_dt(self, prev_dt, max_dt):                      # sph_gravity.cu:2136-2161
        n = self.p.count
        floor_dt = min(np.float32(1e-5), np.float32(max_dt))
        upper = np.float32(min(np.float32(prev_dt) * np.float32(1.15), np.float32(max_dt))) if prev_dt > 0 else np.float32(max_dt)
        self.dt_bits.fill_(0x7f7f7f7f)
        self.K.launch("dt", min(grid(n, 256), 512), 256, self.p.struct(), self.U32(n),
                      ctypes.c_void_p(self.dt_bits.data_ptr()))
        bits = int(self.dt_bits.cpu().item()) & 0xFFFFFFFF   # the blocking D2H copy of the engine
        raw = np.array([bits], np.uint32).view(np.float32)[0]
        if bits == 0x7f7f7f7f or not np.isfinite(raw) or raw <= 0:
            raw = upper
        return float(min(upper, max(floor_dt, raw)))

    def step(self, prev_dt, max_dt, theta=0.5):               # engine/simulation.cpp:1721-1732
        dt = self.reduce_dt(prev_dt, max_dt)
        self.kick(0.5 * dt, True, False)
        self.drift(dt)
        self.sort_and_build()
        self.pass1()
        self.eos()
        self.gravity(theta)
        self.pass2()
        self.kick(0.5 * dt, False, False)
        self.eos()
        return dt

    def initial_forces(self, theta=0.5):                       # engine/simulation.cpp:525-536
        self.clear()
        self.sort_and_build()
        self.pass1()
        self.eos()
        self.gravity(theta)
        self.pass2()


STAGE_FIELDS = {
    "build": ["posX", "posY", "posZ", "velX", "mass", "h", "originalId"],
    "pass1": ["h", "shepardC", "surfFactor", "divV", "curlVX", "curlVY", "curlVZ"],
    "eos": ["pressure", "soundSpeed", "tempK", "phaseId"],
    "gravity": ["accX", "accY", "accZ", "phiGrav"],
    "pass2": ["accX", "accY", "accZ", "drhoDt", "duDt", "radPowerW", "dSXX", "dSYY", "dSZZ", "dSXY", "dSXZ", "dSYZ",
              "dDamageCbrtDt"],
    "kick": ["velX", "velY", "velZ", "rho", "u", "sXX", "sXY", "damage"],
    "drift": ["posX", "posY", "posZ"],
}


def ref_pack_render(K, p, records, speed, sys_com):         # sph_gravity.cu:2189-2201
    """Reference render packing into device buffers (torch uint8 tensors)."""
    n = p.count
    if n == 0:
        return
    K.launch("render", grid(n, 256), 256, p.struct(), ctypes.c_uint32(n), ctypes.c_void_p(records.data_ptr()),
             ctypes.c_void_p(speed.data_ptr() if speed is not None else None), *[ctypes.c_float(c) for c in sys_com])


def ref_extract_tracers(K, p, records, tracer_count, living_com, sys_com):   # sph_gravity.cu:2163-2187
    records.zero_()
    n = p.count
    if n == 0 or tracer_count == 0:
        return
    K.launch("tracers", grid(n, 256), 256, p.struct(), ctypes.c_uint32(n), ctypes.c_void_p(records.data_ptr()),
             ctypes.c_uint32(tracer_count), *[ctypes.c_float(c) for c in living_com],
             *[ctypes.c_float(c) for c in sys_com])


RENDER_CASE = dict(n=2048, tracers=384, seed=11, sys_com=(0.125, -0.25, 0.0625), living_com=(0.5, 0.25, -0.125))


def golden_render(out_path):
    """Reference packing kernels on a seeded edge-case state (tests/golden/render_records.npz)."""
    import torch
    sys.path.insert(0, HERE)
    import oracle
    from astraea_gb300 import engine
    c = RENDER_CASE
    st = oracle.random_render_state(c["n"], c["tracers"], c["seed"])
    K = RefKernels()
    p = engine.DeviceParticles(c["n"])
    p.upload(st)
    rec = torch.zeros(20 * c["n"], dtype=torch.uint8, device="cuda")
    spd = torch.zeros(c["n"], dtype=torch.uint8, device="cuda")
    trc = torch.zeros(40 * c["tracers"], dtype=torch.uint8, device="cuda")
    ref_pack_render(K, p, rec, spd, c["sys_com"])
    ref_extract_tracers(K, p, trc, c["tracers"], c["living_com"], c["sys_com"])
    torch.cuda.synchronize()
    np.savez_compressed(out_path, records=rec.cpu().numpy(), speed=spd.cpu().numpy(), tracers=trc.cpu().numpy())
    print("wrote", out_path)


def golden(out_path):
    """Reference outputs of every stage on the two-sphere scene (3,072 + 1,024)."""
    import torch
    from astraea_gb300 import scenarios
    st, _ = scenarios.two_granite_spheres(n_target=3072, n_impactor=1024, seed=42)
    n = len(st["posX"])
    e = RefEngine(n)
    e.p.upload(st)
    e.alt.count = n
    rec = {"input_" + k: v for k, v in st.items()}
    e.clear()
    e.sort_and_build()
    torch.cuda.synchronize()
    g = e.p.download()
    for f in STAGE_FIELDS["build"]:
        rec["build_" + f] = g[f]
    rec["build_codes"] = e.bvh.t["mortonCodesSorted"][:n].cpu().numpy().view(np.uint64)
    rec["build_perm"] = e.bvh.t["indicesSorted"][:n].cpu().numpy().view(np.uint32)
    rec["build_left"] = e.bvh.t["leftChild"][: n - 1].cpu().numpy()
    rec["build_right"] = e.bvh.t["rightChild"][: n - 1].cpu().numpy()
    rec["build_parent"] = e.bvh.t["parent"][: 2 * n - 1].cpu().numpy()
    for f in ("nodeMass", "comX", "comY", "comZ", "aabbMinX", "aabbMaxX", "nodeMaxH"):
        rec["build_node_" + f] = e.bvh.t[f][: 2 * n - 1].cpu().numpy()
    for stage, fn in (("pass1", e.pass1), ("eos", e.eos), ("gravity", e.gravity), ("pass2", e.pass2)):
        fn()
        torch.cuda.synchronize()
        g = e.p.download()
        for f in STAGE_FIELDS[stage]:
            rec[stage + "_" + f] = g[f]
    dt = e.reduce_dt(0.0, 5.0e-3)
    rec["dt"] = np.array([dt], np.float32)
    e.kick(0.5 * dt, True, False)
    torch.cuda.synchronize()
    g = e.p.download()
    for f in STAGE_FIELDS["kick"]:
        rec["kick_" + f] = g[f]
    e.drift(dt)
    torch.cuda.synchronize()
    g = e.p.download()
    for f in STAGE_FIELDS["drift"]:
        rec["drift_" + f] = g[f]
    # two full steps of the reference from here
    e.sort_and_build(); e.pass1(); e.eos(); e.gravity(); e.pass2(); e.kick(0.5 * dt, False, False); e.eos()
    prev = dt
    for _ in range(2):
        prev = e.step(prev, 5.0e-3)
    torch.cuda.synchronize()
    g = e.p.download()
    for f in ("posX", "posY", "posZ", "velX", "velY", "velZ", "rho", "u", "h", "accX", "accY", "accZ", "originalId"):
        rec["steps_" + f] = g[f]
    rec["steps_dt"] = np.array([prev], np.float32)
    np.savez_compressed(out_path, **rec)
    print("wrote", out_path, len(rec), "arrays")


def bench(n, steps, warmup, theta=0.5, st=None):
    """Step time of the reference's kernels on the workload; returns the
    record that `python ref_gpu.py bench` prints."""
    import torch
    from astraea_gb300 import scenarios
    if st is None:
        st, _ = scenarios.differentiated_impact(n_total=n, seed=42)
    e = RefEngine(n)
    e.p.upload(st)
    e.alt.count = n
    for f in ("velHalfX", "velHalfY", "velHalfZ"):
        e.p.arrays[f][:n].copy_(e.p.arrays["vel" + f[-1]][:n])
    e.initial_forces(theta)
    max_dt = 5.0e-3
    prev = 0.0
    for _ in range(warmup):
        prev = e.step(prev, max_dt, theta)
    torch.cuda.synchronize()
    times = []
    stage_ms = {}
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        prev = e.step(prev, max_dt, theta)
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    # per-stage split of one more step
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(11)]
    ev[0].record(); dt = e.reduce_dt(prev, max_dt); ev[1].record()
    e.kick(0.5 * dt, True, False); ev[2].record()
    e.drift(dt); ev[3].record()
    e.sort_and_build(); ev[4].record()
    e.pass1(); ev[5].record()
    e.eos(); ev[6].record()
    e.gravity(theta); ev[7].record()
    e.pass2(); ev[8].record()
    e.kick(0.5 * dt, False, False); ev[9].record()
    e.eos(); ev[10].record()
    torch.cuda.synchronize()
    names = ["reduce_dt", "kick1", "drift", "sort_build", "pass1", "eos1", "gravity", "pass2", "kick2", "eos2"]
    for k, nm in enumerate(names):
        stage_ms[nm] = ev[k].elapsed_time(ev[k + 1])
    med = float(np.median(times))
    return {"impl": "reference CUDA kernels (sm_100 cubin) on this GPU", "n": n, "steps": steps,
            "warmup": warmup, "ms_per_step_median": med, "ms_per_step_mean": float(np.mean(times)),
            "particle_steps_per_s": n / (med / 1e3), "stage_ms": stage_ms,
            "note": "CUB SortPairs replaced by torch.sort(stable=True), the same stable order"}


if __name__ == "__main__":
    if sys.argv[1] == "golden":
        golden(sys.argv[2])
    elif sys.argv[1] == "golden_render":
        golden_render(sys.argv[2])
    elif sys.argv[1] == "bench":
        print(json.dumps(bench(int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]))))
