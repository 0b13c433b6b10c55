"""The engine's scenario loading and conservation audits, run end to end on
the library's device path (astraea_gb300.headless): preset configuration
(engine/presets.cpp:147-210), bodies built and relaxed on the device,
Kepler approach orbit and merge (engine/simulation.cpp:1300-1470), fused
steps with the device telemetry reduction.

* AC-5 of tests/cpp/test_conservation.cpp:123-158: EarthTheiaMoonForming,
  20,000 particles, 150 steps of at most 5 s: |energy drift| < 1 %,
  |dP| / (M v_esc(1.4 R_earth)) < 1e-4, |dL| / |L0| < 0.5 %;
* the --verify-conservation thresholds of engine/headless_main.cpp:263-281
  on the runner's default preset;
* AC-9 of tests/cpp/test_conservation.cpp:197-258: the surface tracers of the
  LivingTerra target stay a permutation of 0 .. 6 G^2 - 1 across re-sorts.
CPU: the preset table and the Kepler placement's contact speed.
"""
import math
import os

import numpy as np
import pytest

from astraea_gb300 import headless


def test_presets_match_the_engine_table():
    cfg = headless.preset_config("LivingGaiaAsteroidCataclysm", 100000)
    assert cfg["target"].archetype == 0 and cfg["impactor"].archetype == 5
    assert cfg["impactor"].massKg == pytest.approx(0.025 * headless.M_EARTH)
    assert cfg["impactor"].coreTempK == 1800.0 and cfg["impactor"].spinOmegaRadS == 0.0
    assert cfg["target"].relaxSteps == 80 and cfg["grid"] == 16 and cfg["seed"] == 42
    assert (cfg["v_ratio"], cfg["b"], cfg["sep"]) == (1.65, 0.30, 3.2)
    m = headless.preset_config("MercuryMantleStrip", 10)
    assert m["target"].surfaceTempK == 440.0 and m["impactor"].archetype == 1
    assert headless.preset_config("EarthTheiaMoonForming", 10, relax_steps=3)["impactor"].relaxSteps == 3


def kepler_contact_speed(mtot, rc, d0, vrad, vperp):
    """Speed at separation rc on the two-body orbit starting at d0 with
    relative velocity (vrad, vperp): energy conservation."""
    v2 = vrad * vrad + vperp * vperp + 2.0 * headless.G_PSU * mtot * (1.0 / rc - 1.0 / d0)
    return math.sqrt(v2)


def test_kepler_placement_reaches_the_requested_contact_speed():
    G = headless.G_PSU
    mtot, rc, vr, b, sep = 6.1, 9.4, 1.65, 0.30, 3.2
    vesc = math.sqrt(2.0 * G * mtot / rc)
    vc = vr * vesc
    d0 = sep * rc
    v0 = math.sqrt(vc * vc - 2.0 * G * mtot * (1.0 / rc - 1.0 / d0))
    vperp = rc * vc * b / d0
    vrad = -math.sqrt(v0 * v0 - vperp * vperp)
    assert kepler_contact_speed(mtot, rc, d0, vrad, vperp) == pytest.approx(vc, rel=1e-12)


def ac5_drifts(e0, e1, e_rad, p0, p1, l0, l1):
    """The drifts tests/cpp/test_conservation.cpp:123-158 computes."""
    cfg = headless.preset_config("EarthTheiaMoonForming", 20000)
    m_kg = cfg["target"].massKg + cfg["impactor"].massKg
    v_esc = math.sqrt(2.0 * 6.67430e-11 * m_kg / (1.4 * 6.371e6))
    de = (e1 + e_rad - e0) / abs(e0)
    dp = float(np.linalg.norm(np.subtract(p1, p0))) / (m_kg * v_esc)
    dl = float(np.linalg.norm(np.subtract(l1, l0))) / float(np.linalg.norm(l0))
    return de, dp, dl


@pytest.mark.gpu
def test_gpu_conservation_audit_earth_theia_20k(golden_dir):
    """AC-5 on the device path, against the engine's own audit of the same
    scenario (tests/golden/sim_reference.npz: engine/simulation.cpp run on
    the CPU with the oracle's kernels): both pass the test's thresholds, the
    loaded scenarios have the same initial energy to 1e-3 and the drifts agree
    to within a tenth of each threshold."""
    res = headless.run_headless("EarthTheiaMoonForming", particles=20000, steps=150, dt_max_sec=5.0, verify=True)
    print(res)
    assert res["particles"] == 20000 and res["finite"]
    assert abs(res["energy_drift_rel"]) < 0.01
    assert res["dp_rel"] < 1.0e-4 and res["dl_rel"] < 0.005
    assert res["ok"]
    g = np.load(golden_dir + "/sim_reference.npz")
    names = ["frameSeq", "simTimeSec", "dtSec", "outcome", "kineticEnergyJ", "potentialEnergyJ", "internalEnergyJ",
             "radiatedEnergyJ", "totalEnergyJ", "initialTotalEnergyJ", "energyDriftRel", "momentumX", "momentumY",
             "momentumZ", "angularMomentumX", "angularMomentumY", "angularMomentumZ"]
    t0 = dict(zip(names, g["ac5_t0"]))
    t1 = dict(zip(names, g["ac5_t1"]))
    mom = lambda t: [t["momentumX"], t["momentumY"], t["momentumZ"]]
    ang = lambda t: [t["angularMomentumX"], t["angularMomentumY"], t["angularMomentumZ"]]
    engine_d = ac5_drifts(t0["totalEnergyJ"], t1["totalEnergyJ"], t1["radiatedEnergyJ"], mom(t0), mom(t1), ang(t0),
                          ang(t1))
    ours = ac5_drifts(res["energy_j_t0"], res["energy_j_t1"], res["radiated_j"], res["momentum_t0"],
                      res["momentum_t1"], res["angular_momentum_t0"], res["angular_momentum_t1"])
    print("AC-5 drifts (energy, dP, dL): device %s, engine %s" % (ours, engine_d))
    assert abs(res["energy_j_t0"] - t0["totalEnergyJ"]) <= 1e-3 * abs(t0["totalEnergyJ"])
    for mine, ref, thr in zip(ours, engine_d, (0.01, 1e-4, 0.005)):
        assert abs(ref) < thr and abs(mine) < thr
        assert abs(mine - ref) < 0.1 * thr


@pytest.mark.gpu
def test_gpu_verify_conservation_default_preset():
    res = headless.run_headless("LivingGaiaAsteroidCataclysm", particles=30000, steps=100, verify=True)
    print(res)
    assert res["ok"], res
    assert res["tracers"] == 6 * 16 * 16


@pytest.mark.gpu
def test_gpu_tracers_survive_resorts():
    cfg = headless.preset_config("LivingGaiaAsteroidCataclysm", 30000, relax_steps=5)
    sim, info = headless.load_scenario(cfg)
    T = info["tracers"]
    assert T == 6 * 16 * 16
    for _ in range(10):
        sim.step(5.0e-3)
    t = sim.state(["tracerIndex"])["tracerIndex"]
    assert np.array_equal(np.sort(t[t >= 0]), np.arange(T))


REF_CUBIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                         "ref_kernels_sm100.cubin")


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(REF_CUBIN),
                    reason="the reference kernels' cubin (built from the reference checkout) is absent")
def test_gpu_conservation_audit_matches_reference_kernels():
    """AC-5 (EarthTheiaMoonForming, 20,000 particles, 150 steps of at most
    5 s) from one loaded scenario, stepped by this library and by the
    reference's own kernels (oracle/ref_gpu.py) on the same GPU; both audited
    by the same telemetry and formulas: both pass the test's thresholds and
    the drifts agree within a tenth of each threshold."""
    import sys
    import torch
    from astraea_gb300 import engine
    sys.path.insert(0, os.path.dirname(os.path.dirname(REF_CUBIN)))
    import ref_gpu
    cfg = headless.preset_config("EarthTheiaMoonForming", 20000)
    m_tot, r_scale, v_esc = headless.scenario_scales(cfg)
    sim, info = headless.load_scenario(cfg)
    rt, living = info["target_radius_psu"], info["living_body_present"]
    state0 = sim.p.download()
    n = sim.p.count
    max_dt = 5.0 / headless.T_UNIT
    ours = headless.conservation_audit(lambda: sim.step(max_dt), lambda: sim.p, rt, living, 150, m_tot, r_scale, v_esc)
    e = ref_gpu.RefEngine(n)
    e.p.upload(state0)
    e.alt.count = n
    e.initial_forces(0.5)
    prev = [0.0]

    def ref_step():
        prev[0] = e.step(prev[0], max_dt, 0.5)
        return prev[0]
    ref = headless.conservation_audit(ref_step, lambda: e.p, rt, living, 150, m_tot, r_scale, v_esc)
    torch.cuda.synchronize()
    keys = ("energy_drift_rel", "dp_rel", "dl_rel")
    print("AC-5 drifts (energy, dP, dL): library %s, reference kernels %s"
          % ([float("%.3e" % ours[k]) for k in keys], [float("%.3e" % ref[k]) for k in keys]))
    assert abs(ours["energy_j_t0"] - ref["energy_j_t0"]) <= 1e-6 * abs(ref["energy_j_t0"])
    for k, thr in zip(keys, (0.01, 1e-4, 0.005)):
        assert abs(ours[k]) < thr and abs(ref[k]) < thr, k
        assert abs(ours[k] - ref[k]) < 0.1 * thr, k
