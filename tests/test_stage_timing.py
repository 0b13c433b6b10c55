"""Stage timing of the fused step and the SPH pair counters.

astraea_gb300_set_stage_timing / _read_stage_times put CUDA events between
the stages of astraea_gb300_step (the engine times only the whole step,
gpuStepMs, engine/simulation.cpp:1719-1739); astraea_gb300_read_device_counters
adds the in-range pair counts of SPH pass 1, pass 2 and the drift to the
walk counters.  The pass-1 count is an integer result and must equal the
count of the engine's own FP32 test, r^2 < (2 max(h, 1e-6))^2 with
r^2 = (dx dx + dy dy) + dz dz (engine/sph_gravity.cu:713), evaluated here on
the host for every pair.
"""
import os
import re

import numpy as np
import pytest

from astraea_gb300 import abi, scenarios


def c1_state(seed=42):
    st, _ = scenarios.two_granite_spheres(n_target=12288, n_impactor=4096, seed=seed)
    return st


def host_pass1_pairs(st, rows=1024):
    """Pairs (i, j != i) with r_ij^2 < H_i^2 in the engine's FP32 arithmetic."""
    x = np.asarray(st["posX"], np.float32)
    y = np.asarray(st["posY"], np.float32)
    z = np.asarray(st["posZ"], np.float32)
    H = np.float32(2.0) * np.maximum(np.asarray(st["h"], np.float32), np.float32(1.0e-6))
    H2 = H * H
    n = len(x)
    total = 0
    for a in range(0, n, rows):
        b = min(n, a + rows)
        dx = x[a:b, None] - x[None, :]
        dy = y[a:b, None] - y[None, :]
        dz = z[a:b, None] - z[None, :]
        r2 = (dx * dx + dy * dy) + dz * dz
        inside = r2 < H2[a:b, None]
        inside[np.arange(b - a), np.arange(a, b)] = False
        total += int(inside.sum())
    return total


def test_stage_and_counter_names_match_header():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "include", "astraea_gb300.h")) as fh:
        hdr = fh.read()
    stages = dict(re.findall(r"#define ASTRAEA_STAGE_([A-Z0-9_]+)\s+(\d+)", hdr))
    counters = dict(re.findall(r"#define ASTRAEA_COUNTER_([A-Z0-9_]+)\s+(\d+)u", hdr))
    assert int(stages.pop("COUNT")) == len(abi.STAGES)
    assert int(counters.pop("COUNT")) == len(abi.ALL_COUNTERS)
    assert [k.lower() for k, _ in sorted(stages.items(), key=lambda kv: int(kv[1]))] == abi.STAGES
    assert [k.lower() for k, _ in sorted(counters.items(), key=lambda kv: int(kv[1]))] == abi.ALL_COUNTERS


@pytest.mark.gpu
def test_gpu_pass1_pair_counter_matches_host_count():
    from astraea_gb300 import engine
    st = c1_state()
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    engine.sort_and_build_bvh(p, alt, bvh)
    engine.reset_device_status()
    engine.sph_pass1_neighbors(p, bvh)
    c = engine.read_device_counters()
    assert c["pass1_pairs"] == host_pass1_pairs(st)
    assert 0 < c["pass1_pairs"] <= c["neighbor_entries"]
    engine.evaluate_eos(p)
    engine.gravity_barnes_hut(p, bvh, 0.5)
    engine.sph_pass2_forces(p, bvh)
    c2 = engine.read_device_counters()
    assert 0 < c2["pass2_pairs"] <= c2["neighbor_entries"]
    assert c2["pass1_pairs"] == c["pass1_pairs"]


@pytest.mark.gpu
def test_gpu_stage_times_cover_the_fused_step():
    import torch
    from astraea_gb300 import engine
    st, _ = scenarios.differentiated_impact(n_total=131072, seed=21)
    n = len(st["posX"])
    sim = engine.Simulation(n)
    sim.load_state(st)
    sim.evaluate_initial_forces(0.5)
    with pytest.raises(abi.AstraeaError):
        engine.read_stage_times(sim.bvh)            # no timed step yet
    for _ in range(2):
        sim.step(5.0e-3)
    engine.set_stage_timing(True)
    try:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        engine.reset_device_status()
        e0.record()
        sim.step(5.0e-3, sync=False)
        e1.record()
        torch.cuda.synchronize()
        whole = e0.elapsed_time(e1)
        t = engine.read_stage_times(sim.bvh)
        c = engine.read_device_counters()
        engine.invalidate_step_cache(sim.bvh)
        sim.step(5.0e-3)
        t_refresh = engine.read_stage_times(sim.bvh)
    finally:
        engine.set_stage_timing(False)
    assert list(t) == abi.STAGES
    assert all(v >= 0.0 for v in t.values())
    total = sum(t.values())
    assert 0.8 * whole <= total <= 1.05 * whole + 0.05
    assert t["gravity"] > 0.0 and t["pass2"] > 0.0 and t["neighbours"] > 0.0
    assert t["refresh"] < 0.1 * total                 # step cache valid: nothing rebuilt
    assert t_refresh["refresh"] > 0.5 * t_refresh["neighbours"]   # invalid cache: leaves + drift lists rebuilt
    assert c["pass1_pairs"] > 0 and c["pass2_pairs"] > 0 and c["drift_pairs"] > 0
    assert c["drift_pairs"] <= c["neighbor_entries"]
