"""Parity at the throughput workload: the differentiated Earth-Theia-like
impact at N = 1,000,000 (800k + 200k particles, Iron core + Granite mantle).

The GPU takes the seeded bodies through the initial forces and one fused
step; the state it reaches (velocities, stresses and damage no longer zero)
is the snapshot every stage below starts from.  Each stage runs on the GPU
through the C-ABI and in the oracle on identical inputs (the GPU's state
before the stage is copied into the oracle), over every particle:

* Morton codes, the sorted permutation, the Karras topology, node boxes,
  nodeMaxH and all 56 permuted fields: bit for bit;
* pass 1, EOS, gravity, pass 2, kick: within 1e-5 norm-relative RMS, drift
  within 1e-6;
* integer outputs exact: the EOS phase of every particle, the gravity
  interaction count (the same interaction set), the dt.

Where the reference's own kernels are present (oracle/_ref, compiled from
the reference checkout for sm_100), the same snapshot also runs through them
(oracle/ref_gpu.py) and the library is compared with the engine itself.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from astraea_gb300 import abi, engine, scenarios
from conftest import rel_rms

pytestmark = pytest.mark.gpu
REF_CUBIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                         "ref_kernels_sm100.cubin")
N = 1_000_000
TOL = 1e-5
MAX_DT = 5.0e-3


@pytest.fixture(scope="module")
def snapshot():
    st, _ = scenarios.differentiated_impact(N, seed=42)
    sim = engine.Simulation(N)
    sim.load_state(st)
    sim.evaluate_initial_forces()
    dt = sim.step(MAX_DT)
    s1 = sim.state()
    del sim
    torch.cuda.empty_cache()
    return s1, dt


def setup(state):
    p, alt = engine.DeviceParticles(N), engine.DeviceParticles(N)
    p.upload(state)
    alt.count = N
    bvh = engine.TorchBvh(N, packed=True)
    return p, alt, bvh


def into_oracle(o, g):
    """Copy a downloaded GPU state into the oracle's particle arrays (the
    oracle's tree, built from the same positions, is bit-identical)."""
    for name, a in g.items():
        o.p.arrays[name][:N] = a


def node_moments_into_oracle(o, bvh):
    """Give the oracle's tree the library's node masses and COMs.  The library
    forms them from exact fixed-point moment sums, the oracle (like the
    engine) from FP32 sums, so they differ in the last bit; a borderline
    opening test can then decide differently.  With the same node data the
    walks must make the same decisions."""
    for f in ("nodeMass", "comX", "comY", "comZ"):
        o.bvh.a[f][: 2 * N - 1] = bvh.t[f][: 2 * N - 1].cpu().numpy()


def report(tag, g, c, fields):
    errs = {f: rel_rms(g[f], c[f]) for f in fields}
    print("1M %s %s" % (tag, " ".join("%s=%.2e" % kv for kv in errs.items())))
    return errs


def test_1m_sort_and_tree_bit_exact(snapshot):
    s1, _ = snapshot
    p, alt, bvh = setup(s1)
    engine.sort_and_build_bvh(p, alt, bvh)
    torch.cuda.synchronize()
    o = oracle.Oracle(s1)
    o.sort_and_build()
    b = o.bvh.a
    t = lambda name, k, dt=None: bvh.t[name][:k].cpu().numpy().view(dt) if dt else bvh.t[name][:k].cpu().numpy()
    assert np.array_equal(t("mortonCodesSorted", N, np.uint64), b["mortonCodesSorted"])
    assert np.array_equal(t("indicesSorted", N, np.uint32), b["indicesSorted"])
    assert np.array_equal(t("leftChild", N - 1), b["leftChild"][: N - 1])
    assert np.array_equal(t("rightChild", N - 1), b["rightChild"][: N - 1])
    assert np.array_equal(t("parent", 2 * N - 1), b["parent"])
    for f in ("aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ", "nodeMaxH"):
        assert np.array_equal(t(f, 2 * N - 1), b[f]), f
    assert np.array_equal(t("sceneBoundsFloat", 6), o.bounds)
    g, c = p.download(), o.state()
    for f in abi.FIELD_NAMES:
        assert np.array_equal(g[f], c[f]), f


def test_1m_stages_on_identical_inputs(snapshot):
    s1, _ = snapshot
    p, alt, bvh = setup(s1)
    o = oracle.Oracle(s1)
    engine.sort_and_build_bvh(p, alt, bvh)
    o.sort_and_build()

    engine.sph_pass1_neighbors(p, bvh)
    o.pass1()
    g, c = p.download(), o.state()
    e = report("pass1", g, c, ["h", "shepardC", "surfFactor", "divV", "curlVX", "curlVY", "curlVZ"])
    assert max(e.values()) < TOL

    into_oracle(o, g)
    engine.evaluate_eos(p)
    o.eos()
    g, c = p.download(), o.state()
    e = report("eos", g, c, ["pressure", "soundSpeed", "tempK"])
    assert max(e.values()) < TOL
    flips = np.flatnonzero(g["phaseId"] != c["phaseId"])
    assert flips.size == 0, [(int(i), int(g["phaseId"][i]), int(c["phaseId"][i]), float(c["tempK"][i]),
                              float(g["rho"][i]), float(g["u"][i]), int(g["materialId"][i])) for i in flips[:10]]

    into_oracle(o, g)
    gpu_groups = engine.gravity_group_counts(p, bvh, 0.5)
    engine.reset_device_status()
    engine.gravity_barnes_hut(p, bvh, 0.5)
    _, counters = engine.read_device_status()
    own = o.gravity(0.5)                        # the oracle's own FP32 node COMs
    node_moments_into_oracle(o, bvh)
    cpu_groups = o.gravity_group_counts(0.5)
    count = o.gravity(0.5)
    print("1M gravity interactions gpu %d oracle %d (oracle with its own node COMs %d, %.1e relative)"
          % (counters["gravity_interactions"], count, own, abs(own - count) / count))
    bad = np.flatnonzero(gpu_groups != cpu_groups)
    assert bad.size == 0, [(int(k), int(gpu_groups[k]), int(cpu_groups[k])) for k in bad[:10]]
    assert counters["gravity_interactions"] == count == int(cpu_groups.sum())
    assert abs(own - count) <= 1e-6 * count
    g, c = p.download(), o.state()
    e = report("gravity", g, c, ["accX", "accY", "accZ", "phiGrav"])
    assert max(e.values()) < TOL

    into_oracle(o, g)
    engine.sph_pass2_forces(p, bvh)
    o.pass2()
    g, c = p.download(), o.state()
    e = report("pass2", g, c, ["accX", "accY", "accZ", "drhoDt", "duDt", "radPowerW", "dSXX", "dSYY", "dSZZ",
                               "dSXY", "dSXZ", "dSYZ", "dDamageCbrtDt"])
    assert max(e.values()) < TOL

    into_oracle(o, g)
    dt_g = engine.reduce_dt_psu(p, 0.0, MAX_DT)
    dt_c, _ = o.reduce_dt(0.0, MAX_DT)
    print("1M dt gpu %.9g oracle %.9g" % (dt_g, dt_c))
    assert dt_g == dt_c

    engine.leapfrog_kick_half(p, 0.5 * dt_g, True, False)
    o.kick(0.5 * dt_g)
    g, c = p.download(), o.state()
    e = report("kick", g, c, ["velX", "velY", "velZ", "rho", "u", "sXX", "sXY", "damage"])
    assert max(e.values()) < TOL

    into_oracle(o, g)
    engine.leapfrog_drift(p, dt_g, bvh)
    o.drift(dt_g)
    g, c = p.download(), o.state()
    e = report("drift", g, c, ["posX", "posY", "posZ"])
    assert max(e.values()) < 1e-6


def test_1m_fused_step_from_snapshot(snapshot):
    """One more fused step from the snapshot against the oracle's stage
    sequence from the same snapshot.  The dt of that step comes from the
    snapshot's fields on both sides, so it is exact.  After the drift the
    positions differ in the last bits (neighbour sums in another order), and
    a Morton code can change with one ulp, so the fields are compared particle
    by particle through originalId, within 1e-5."""
    s1, dt1 = snapshot
    sim = engine.Simulation(N)
    sim.p.upload(s1)
    sim.alt.count = N
    sim.prev_dt = dt1
    # the tree of the snapshot (its particles are already in Morton order:
    # the identity permutation) for the opening drift, on both sides
    engine.sort_and_build_bvh(sim.p, sim.alt, sim.bvh)
    engine.invalidate_step_cache(sim.bvh)
    o = oracle.Oracle(s1)
    o.sort_and_build()
    o.prev_dt = dt1
    dt_g = sim.step(MAX_DT)
    dt_c = o.step(MAX_DT)
    print("1M fused step dt gpu %.9g oracle %.9g" % (dt_g, dt_c))
    assert dt_g == dt_c
    g, c = sim.state(), o.state()
    og, oc = np.argsort(g["originalId"]), np.argsort(c["originalId"])
    assert np.array_equal(g["originalId"][og], c["originalId"][oc])
    fields = ["posX", "posY", "posZ", "velX", "velY", "velZ", "rho", "u", "h"]
    e = report("fused-step", {f: g[f][og] for f in fields}, {f: c[f][oc] for f in fields}, fields)
    assert max(e.values()) < TOL


@pytest.mark.skipif(not os.path.exists(REF_CUBIN),
                    reason="the reference kernels' cubin (built from the reference checkout) is absent")
def test_1m_against_reference_kernels(snapshot):
    """The snapshot through the reference's own kernels and through the
    library with the engine's node rounding (astraea_gb300_set_node_rounding):
    * the tree bit for bit, node masses and COMs included;
    * pass 1: h bit for bit (the neighbour counts are the engine's: the range
      test rounds |d|^2 as the engine's compiled kernel does), the other
      fields within 1e-5;
    * gravity: the oracle, whose node data and member test are the engine's
      bit for bit, makes exactly the library's interaction count in every
      group, and the accelerations agree with the reference kernels' to
      float summation order in every group;
    * dt of the reference's state after pass 2: the same float."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(REF_CUBIN), os.pardir))
    import ref_gpu
    s1, _ = snapshot
    e = ref_gpu.RefEngine(N)
    e.p.upload(s1)
    e.alt.count = N
    e.sort_and_build()
    p, alt, bvh = setup(s1)
    engine.set_node_rounding(1)
    try:
        engine.sort_and_build_bvh(p, alt, bvh)
    finally:
        engine.set_node_rounding(0)
    torch.cuda.synchronize()
    for name, k in (("mortonCodesSorted", N), ("indicesSorted", N), ("leftChild", N - 1), ("rightChild", N - 1),
                    ("parent", 2 * N - 1)):
        assert torch.equal(bvh.t[name][:k], e.bvh.t[name][:k]), name
    for f in ("aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ", "nodeMaxH", "nodeMass",
              "comX", "comY", "comZ"):
        assert torch.equal(bvh.t[f][: 2 * N - 1], e.bvh.t[f][: 2 * N - 1]), f
    g, r = p.download(), e.p.download()
    for f in abi.FIELD_NAMES:
        assert np.array_equal(g[f], r[f]), f

    engine.sph_pass1_neighbors(p, bvh)
    e.pass1()
    g, r = p.download(), e.p.download()
    hdiff = np.flatnonzero(g["h"] != r["h"])
    print("1M vs reference kernels: pass 1 h differs for %d particles" % hdiff.size)
    assert hdiff.size == 0, hdiff[:10]
    err = report("pass1 vs reference kernels", g, r, ["shepardC", "surfFactor", "divV", "curlVX", "curlVY", "curlVZ"])
    assert max(err.values()) < TOL

    engine.evaluate_eos(p)
    e.eos()
    engine.gravity_barnes_hut(p, bvh, 0.5)
    e.gravity(0.5)
    gg = engine.gravity_group_counts(p, bvh, 0.5)
    g, r = p.download(), e.p.download()
    o = oracle.Oracle(s1)
    o.sort_and_build()
    for f in ("nodeMass", "comX", "comY", "comZ"):       # the oracle's own node data is the engine's
        assert np.array_equal(o.bvh.a[f][: 2 * N - 1], e.bvh.t[f][: 2 * N - 1].cpu().numpy()), f
    cg = o.gravity_group_counts(0.5)
    bad = np.flatnonzero(gg != cg)
    assert bad.size == 0, [(int(k), int(gg[k]), int(cg[k])) for k in bad[:10]]
    # per particle, against the RMS acceleration (near the bodies' centres
    # |a| itself goes to zero): float summation order leaves ~1e-7, one
    # opening decision taken otherwise ~1e-4
    A = lambda d: np.stack([d["accX"], d["accY"], d["accZ"]], 1).astype(np.float64)
    ar = A(r)
    d = np.linalg.norm(A(g) - ar, axis=1) / np.sqrt(np.mean(np.sum(ar * ar, axis=1)))
    print("1M gravity vs reference kernels: per-particle difference / RMS |a|: median %.2e, p99.99 %.2e, max %.2e; "
          "interactions %d" % (np.median(d), np.percentile(d, 99.99), d.max(), int(gg.sum())))
    err = report("gravity vs reference kernels", g, r, ["accX", "accY", "accZ", "phiGrav"])
    assert max(err.values()) < 1e-6
    assert d.max() < 2e-5

    engine.sph_pass2_forces(p, bvh)
    e.pass2()
    g, r = p.download(), e.p.download()
    err = report("pass2 vs reference kernels", g, r, ["accX", "accY", "accZ", "drhoDt", "duDt", "radPowerW"])
    assert max(err.values()) < TOL
    q = engine.DeviceParticles(N)
    q.upload(r)
    dt_l = engine.reduce_dt_psu(q, 0.0, MAX_DT)
    dt_r = e.reduce_dt(0.0, MAX_DT)
    print("1M dt on the reference's state after pass 2: library %.9g, reference kernels %.9g" % (dt_l, dt_r))
    assert dt_l == dt_r


@pytest.mark.skipif(not os.path.exists(REF_CUBIN),
                    reason="the reference kernels' cubin (built from the reference checkout) is absent")
def test_1m_fused_step_against_reference_step(snapshot):
    """One fused step of the library (engine node rounding) against one step
    of the reference's own kernel sequence (engine/simulation.cpp:1721-1732)
    from the same snapshot.  The dt is the same float (it comes from the
    snapshot's fields).  The reference's drift reads neighbour positions that
    other threads are moving, so its positions after the drift differ from
    any race-free drift in the last bits; a pair that lands within an ulp of
    a range boundary then changes a neighbour count, an h and the SPH forces
    around it.  So: positions, density and energy within 1e-6 RMS; h equal
    for all but a few particles in 10^4; accelerations within 1e-4 of the RMS
    acceleration for 99.9 % of the particles and beyond it only around the
    particles whose h changed (compared through originalId)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(REF_CUBIN), os.pardir))
    import ref_gpu
    s1, dt1 = snapshot
    e = ref_gpu.RefEngine(N)
    e.p.upload(s1)
    e.alt.count = N
    e.sort_and_build()                   # the snapshot's tree, for the opening drift
    dt_r = e.step(dt1, MAX_DT)
    r = e.p.download()
    del e
    torch.cuda.empty_cache()
    sim = engine.Simulation(N)
    sim.p.upload(s1)
    sim.alt.count = N
    sim.prev_dt = dt1
    engine.set_node_rounding(1)
    try:
        engine.sort_and_build_bvh(sim.p, sim.alt, sim.bvh)
        engine.invalidate_step_cache(sim.bvh)
        dt_g = sim.step(MAX_DT)
    finally:
        engine.set_node_rounding(0)
    g = sim.state()
    print("1M fused step vs reference step: dt %.9g / %.9g" % (dt_g, dt_r))
    assert dt_g == dt_r
    og, orr = np.argsort(g["originalId"]), np.argsort(r["originalId"])
    assert np.array_equal(g["originalId"][og], r["originalId"][orr])
    G = {f: g[f][og] for f in g}
    R = {f: r[f][orr] for f in r}
    err = report("fused step vs reference step", G, R, ["posX", "posY", "posZ", "rho", "u", "velX", "velY", "velZ"])
    assert max(err[f] for f in ("posX", "posY", "posZ", "rho", "u")) < 1e-6
    hdiff = np.abs(G["h"].astype(np.float64) - R["h"]) / R["h"]
    A = lambda d: np.stack([d["accX"], d["accY"], d["accZ"]], 1).astype(np.float64)
    ar = A(R)
    da = np.linalg.norm(A(G) - ar, axis=1) / np.sqrt(np.mean(np.sum(ar * ar, axis=1)))
    print("1M fused step vs reference step: h differs (> 1e-6) for %d particles; acceleration difference / RMS "
          "|a|: median %.2e, p99.9 %.2e, p99.99 %.2e, max %.2e"
          % (int(np.sum(hdiff > 1e-6)), np.median(da), np.percentile(da, 99.9), np.percentile(da, 99.99), da.max()))
    nh = int(np.sum(hdiff > 1e-6))
    assert nh <= N // 10000
    # beyond float summation order only around the particles whose h changed
    # (a neighbourhood is ~60 particles)
    assert np.percentile(da, 99.9) < 1e-4
    assert int(np.sum(da > 1e-4)) <= 100 * (nh + 1)
