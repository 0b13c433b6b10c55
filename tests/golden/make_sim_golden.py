"""Generates tests/golden/sim_reference.npz from the reference engine's own
host code (TEST INFRASTRUCTURE; needs the reference checkout, so it runs on
the build machine, not the GPU machines).

oracle/ref_sim.py runs engine/simulation.cpp on the CPU (a host stand-in for
the CUDA runtime, the oracle as its kernels).  Recorded:

* telemetry: three states with the engine's TelemetrySnapshot and the engine
  state its scalar code reads (computeTelemetryFromDevice, :948-1285) --
  EarthTheiaMoonForming and LivingGaiaAsteroidCataclysm (a living target with
  surface tracers) after their load and four steps, and a post-impact state
  (the first with velocities and damage set so that every branch of the
  remnant classification and of the outcome rules is taken);
* relaxation: relaxLoadedSingleBody (:585-781) on two bodies built by the
  reference PlanetBuilder (the oracle's builder, bit-identical to it) and
  prepared as Simulation::relaxBody prepares them, 6 damped steps: the relaxed
  positions, velocities, density, energy, h and v_rms / v_esc;
* AC-2 (tests/cpp/test_planet_builder.cpp:329-361): relaxBody(0, 80) of each
  of the six archetypes in the test's own two-body scenario, the engine's
  v_rms / v_esc;
* AC-5 (tests/cpp/test_conservation.cpp:123-158): the engine's own
  conservation audit -- EarthTheiaMoonForming, 20,000 particles, loadScenario
  with its relaxation, 150 steps -- its snapshots at the start and the end and
  the drifts the test and --verify-conservation compute from them.

Usage: python tests/golden/make_sim_golden.py [out.npz]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "astraea-impact-sim_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import ref_sim  # noqa: E402
from astraea_gb300 import abi  # noqa: E402

TELEMETRY_FIELDS = ["posX", "posY", "posZ", "velX", "velY", "velZ", "mass", "rho", "u", "phiGrav", "tempK",
                    "pressure", "radPowerW", "damage", "bodyId", "materialId", "originalId"]
RELAX_OUT = ["posX", "posY", "posZ", "velX", "velY", "velZ", "rho", "u", "h"]
N_TELE = 3000
N_RELAX = 3000


def telemetry_case(out, tag, sim, state=None):
    if state is not None:
        sim.set_state(state)
    st = sim.state()
    ctx = sim.context()
    snap = sim.telemetry()
    for f in TELEMETRY_FIELDS:
        out["tele_%s_%s" % (tag, f)] = st[f]
    out["tele_%s_context" % tag] = np.array([ctx[k] for k in ref_sim.CONTEXT_FIELDS])
    out["tele_%s_snapshot" % tag] = np.array([snap[k] for k in ref_sim.SNAPSHOT_FIELDS])
    return st


def post_impact(st, seed=5):
    """The state with a fraction of particles flung out (ejecta), some set on
    tangential orbits (disk candidates), the impactor moved onto the target and
    some damage: every branch of the classification is taken."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = {k: v.copy() for k, v in st.items()}
    n = len(s["posX"])
    imp = s["bodyId"] != 0
    for k in ("posX", "posY", "posZ"):
        c0 = np.average(s[k][~imp], weights=s["mass"][~imp])
        c1 = np.average(s[k][imp], weights=s["mass"][imp])
        s[k][imp] = (s[k][imp] - 0.8 * (c1 - c0)).astype(np.float32)
    pick = rng.permutation(n)
    ej, disk = pick[: n // 10], pick[n // 10: n // 5]
    for k in ("velX", "velY", "velZ"):
        s[k][ej] = (s[k][ej] + rng.normal(0.0, 25.0, len(ej))).astype(np.float32)
    r = np.stack([s["posX"][disk], s["posY"][disk], s["posZ"][disk]], 1).astype(np.float64)
    t = np.cross(r, np.array([0.0, 1.0, 0.0]))
    t /= np.maximum(np.linalg.norm(t, axis=1, keepdims=True), 1e-9)
    for j, k in enumerate(("velX", "velY", "velZ")):
        s[k][disk] = (s[k][disk] + 6.0 * t[:, j]).astype(np.float32)
    for k in ("posX", "posY", "posZ"):
        s[k][disk] = (s[k][disk] * 1.8).astype(np.float32)
    s["damage"][pick[: n // 3]] = rng.uniform(0.0, 1.0, n // 3).astype(np.float32)
    return s


def prepared_body(archetype, n, grid, seed=42):
    """A body of the reference builder prepared as Simulation::relaxBody
    prepares it: COM and bulk velocity removed, velocities zero, h = h0,
    stresses and damage zero, originalId = index; anchors = tempK."""
    from astraea_gb300 import engine   # body specs only (no GPU work)
    spec = engine.body_spec(archetype)
    st, info = oracle.build_planet(spec, n, 0, grid, seed)
    m = st["mass"].astype(np.float64)
    for k in ("posX", "posY", "posZ"):
        c = np.sum(m * st[k].astype(np.float64)) / np.sum(m)
        st[k] = (st[k].astype(np.float64) - c).astype(np.float32)
    for k in ("velX", "velY", "velZ", "velHalfX", "velHalfY", "velHalfZ", "sXX", "sYY", "sZZ", "sXY", "sXZ", "sYZ",
              "damage", "damageCbrt", "pressure", "soundSpeed"):
        st[k] = np.zeros(n, np.float32)
    st["phaseId"] = np.zeros(n, np.uint8)
    st["h"] = st["h0"].copy()
    st["originalId"] = np.arange(n, dtype=np.uint32)
    radius = oracle.solve_hydrostatic(spec)[1] / 1.0e6
    return st, st["tempK"].astype(np.float64), radius


def main(out_path):
    out = {}
    sim = ref_sim.RefSimulation(N_TELE)
    sim.load_preset("EarthTheiaMoonForming", N_TELE, 10, 42)
    telemetry_case(out, "earth_t0", sim)
    for _ in range(4):
        sim.step(5.0)
    st = telemetry_case(out, "earth_s4", sim)
    telemetry_case(out, "post_impact", sim, post_impact(st))
    sim2 = ref_sim.RefSimulation(N_TELE)
    sim2.load_preset("LivingGaiaAsteroidCataclysm", N_TELE, 10, 42)
    for _ in range(4):
        sim2.step(5.0)
    telemetry_case(out, "gaia_s4", sim2)

    for arch, grid in ((1, 0), (0, 8)):        # IronCore; LivingTerra with surface tracers
        body, anchors, radius = prepared_body(arch, N_RELAX, grid)
        relaxed, vr = sim.relax_loaded(body, anchors, radius, 6)
        for f in RELAX_OUT:
            out["relax_a%d_%s" % (arch, f)] = relaxed[f]
        out["relax_a%d_vrms" % arch] = np.array([vr])
        out["relax_a%d_radius" % arch] = np.array([radius])

    ac2 = []
    for arch in range(6):
        body, anchors, radius = prepared_body(arch, 6400, 8)
        _, vr = sim.relax_loaded(body, anchors, radius, 80)
        ac2.append(vr)
        print("AC-2 archetype %d: v_rms / v_esc = %.3e" % (arch, vr))
    out["ac2_vrms"] = np.array(ac2)

    cons = ref_sim.RefSimulation(25000)
    cons.load_preset("EarthTheiaMoonForming", 20000, -1, 42)
    t0 = cons.telemetry()
    for _ in range(150):
        cons.step(5.0)
    t1 = cons.telemetry()
    out["ac5_t0"] = np.array([t0[k] for k in ref_sim.SNAPSHOT_FIELDS])
    out["ac5_t1"] = np.array([t1[k] for k in ref_sim.SNAPSHOT_FIELDS])
    print("AC-5 engine: energy drift %.3e, sim time %.1f s" % (t1["energyDriftRel"], t1["simTimeSec"]))
    np.savez_compressed(out_path, **out)
    print("wrote", out_path, len(out), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "sim_reference.npz"))
