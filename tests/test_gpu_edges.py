"""Edge cases of the step pipeline on the GPU, against the oracle.

* count 0: every stage call is a no-op, as in the engine (sph_gravity.cu
  launchers return early for an empty buffer; reduce-dt returns its upper
  bound, sph_gravity.cu:2136-2160);
* counts around the 32-particle group width (31, 32, 64, 65, 97): partial
  groups in the gravity and neighbour walks;
* a fully coincident cloud: zero-extent scene (Morton span guard,
  sph_gravity.cu:350-355), all codes equal, the index tie-break builds the tree;
* neighbour-list overflow: with the per-particle list capacity forced to 32
  (below the ~56 neighbours of the scene) every particle is served by the
  per-thread fallback walk; pass 1 and pass 2 must still equal the oracle.
  The capacity is read once per process, so this runs in a child process.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from astraea_gb300 import scenarios
from conftest import rel_rms

pytestmark = pytest.mark.gpu
TOL = 1e-5
FIELDS = ("h", "shepardC", "divV", "accX", "accY", "accZ", "phiGrav", "drhoDt", "duDt", "dSXY")


def c1_state(n_t=3072, n_i=1024, seed=11):
    st, _ = scenarios.two_granite_spheres(n_target=n_t, n_impactor=n_i, seed=seed)
    return st


def run_pipeline(st):
    """Stage calls on the GPU and the oracle from the same state."""
    from astraea_gb300 import engine
    n = len(st["posX"])
    p, alt = engine.DeviceParticles(n), engine.DeviceParticles(n)
    p.upload(st)
    alt.count = n
    bvh = engine.DeviceBvh(n)
    o = oracle.Oracle(st)
    engine.clear_stats(p); o.clear_stats()
    engine.sort_and_build_bvh(p, alt, bvh); o.sort_and_build()
    engine.sph_pass1_neighbors(p, bvh); o.pass1()
    engine.evaluate_eos(p); o.eos()
    engine.gravity_barnes_hut(p, bvh); o.gravity()
    engine.sph_pass2_forces(p, bvh); o.pass2()
    return p.download(), o.state()


def check(g, c):
    assert np.array_equal(g["originalId"], c["originalId"])
    for f in FIELDS:
        assert np.all(np.isfinite(g[f])), f
        assert rel_rms(g[f], c[f]) < TOL or np.allclose(g[f], c[f], atol=1e-12), (f, rel_rms(g[f], c[f]))


def test_empty_count_is_a_no_op():
    import torch
    from astraea_gb300 import engine
    p, alt = engine.DeviceParticles(16), engine.DeviceParticles(16)
    bvh = engine.DeviceBvh(16)
    p.arrays["accX"].fill_(7.0)
    engine.clear_stats(p)
    engine.sort_and_build_bvh(p, alt, bvh)
    engine.sph_pass1_neighbors(p, bvh)
    engine.evaluate_eos(p)
    engine.gravity_barnes_hut(p, bvh)
    engine.sph_pass2_forces(p, bvh)
    engine.leapfrog_kick_half(p, 1e-3)
    engine.leapfrog_drift(p, 1e-3, bvh)
    assert engine.reduce_dt_psu(p, 0.0, 2.5e-3) == pytest.approx(2.5e-3)       # the upper bound
    assert engine.reduce_dt_psu(p, 1.0e-3, 2.5e-3) == pytest.approx(1.15e-3)
    rec = torch.full((40,), 3, dtype=torch.uint8, device="cuda")
    engine.pack_render_records(p, rec, None)
    torch.cuda.synchronize()
    assert torch.all(p.arrays["accX"] == 7.0) and torch.all(rec == 3)


@pytest.mark.parametrize("n", [31, 32, 64, 65, 97])
def test_group_boundary_counts(n):
    st = c1_state()
    small = {k: v[:n].copy() for k, v in st.items()}
    small["originalId"] = np.arange(n, dtype=np.uint32)
    check(*run_pipeline(small))


def test_fully_coincident_cloud():
    n = 300
    st = c1_state()
    small = {k: v[:n].copy() for k, v in st.items()}
    for k in ("posX", "posY", "posZ"):
        small[k][:] = small[k][0]
    small["originalId"] = np.arange(n, dtype=np.uint32)
    g, c = run_pipeline(small)
    assert np.array_equal(g["originalId"], c["originalId"])
    # Every separation is zero, so the true gravity and SPH accelerations are
    # zero.  The library's node COM comes from exact moment sums and equals the
    # common position: it opens every node and adds exact zeros.  The
    # engine's FP32 COM lands an ulp away, so its tiny nodes pass the opening
    # test and give a spurious monopole force (the oracle shows ~1.7e-6).
    for f in ("accX", "accY", "accZ"):
        assert np.all(g[f] == 0.0), f
        assert np.max(np.abs(c[f])) < 1e-5, f
    # the potential likewise: here all pairs with eps_ij softening, as the
    # FP64 direct sum; the oracle's spurious monopoles use eps_i instead
    _, phi64 = oracle.direct_gravity_f64(g, np.arange(n, dtype=np.uint32))
    assert rel_rms(g["phiGrav"], phi64) < TOL
    for f in ("h", "shepardC"):
        assert np.all(np.isfinite(g[f])), f
        assert rel_rms(g[f], c[f]) < TOL, f


def _overflow_child():
    """Runs in a child process with ASTRAEA_GB300_MAX_NEIGHBORS=32."""
    from astraea_gb300 import abi, engine
    st = c1_state()
    engine.reset_device_status()
    g, c = run_pipeline(st)
    flags, counters = engine.read_device_status()
    assert flags & abi.DEVFLAG_NEIGHBOR_OVERFLOW
    assert counters["fallback_walks"] > 0
    check(g, c)
    print("OVERFLOW-OK fallback_walks=%d" % counters["fallback_walks"])


def test_neighbour_overflow_falls_back_to_tree_walk():
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, ASTRAEA_GB300_MAX_NEIGHBORS="32")
    code = "import sys; sys.path.insert(0, %r); import conftest, test_gpu_edges as t; t._overflow_child()" % here
    res = subprocess.run([sys.executable, "-c", code], cwd=here, env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert "OVERFLOW-OK" in res.stdout
