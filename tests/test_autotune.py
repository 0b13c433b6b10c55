"""Autotuning of the tree walks' block shape (astraea_gb300_autotune).

The gravity walk and the neighbour-list walk give bit-identical results for
2, 4 and 8 warps per block (one warp walks one group of 32 particles
whatever the block size), so the autotuner may pick any of them; the tuned
choice is kept per power-of-two particle count and used by the stage calls
and the fused step; the gravity walk's choice is kept per walk variant
(monopole, quadrupole, expansion, each with and without the inside-box rule).
"""
import numpy as np
import pytest

from astraea_gb300 import abi, scenarios


@pytest.mark.gpu
def test_gpu_walk_results_do_not_depend_on_block_shape():
    from astraea_gb300 import engine
    st, _ = scenarios.differentiated_impact(n_total=131072, seed=17)
    n = len(st["posX"])
    outs = []
    for gw, nw in ((4, 4), (2, 2), (8, 8), (2, 8)):
        engine.set_tuning(n, gw, nw)
        p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
        p.upload(st)
        alt.count = n
        engine.sort_and_build_bvh(p, alt, bvh)
        engine.sph_pass1_neighbors(p, bvh)
        engine.evaluate_eos(p)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        engine.sph_pass2_forces(p, bvh)
        outs.append(p.download(["accX", "accY", "accZ", "phiGrav", "h", "shepardC", "drhoDt", "duDt"]))
    engine.set_tuning(n, 4, 4)
    for o in outs[1:]:
        for f, v in o.items():
            assert np.array_equal(v, outs[0][f]), f


@pytest.mark.gpu
def test_gpu_quadrupole_walk_does_not_depend_on_block_shape():
    from astraea_gb300 import engine
    st, _ = scenarios.differentiated_impact(n_total=131072, seed=19)
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    outs = []
    engine.set_far_field(1)
    try:
        engine.sort_and_build_bvh(p, alt, bvh)           # builds the second moments too
        for gw in (4, 2, 8):
            engine.set_tuning(n, gw, 4)
            engine.gravity_barnes_hut(p, bvh, 0.7)
            outs.append(p.download(["accX", "accY", "accZ", "phiGrav"]))
    finally:
        engine.set_far_field(0)
        engine.set_tuning(n, 4, 4)
    for o in outs[1:]:
        for f, v in o.items():
            assert np.array_equal(v, outs[0][f]), f


@pytest.mark.gpu
def test_gpu_autotune_records_a_valid_choice():
    from astraea_gb300 import engine
    st, _ = scenarios.differentiated_impact(n_total=65536, seed=18)
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    engine.sort_and_build_bvh(p, alt, bvh)
    t = engine.autotune(p, bvh, 0.5)
    assert t["gravityWarps"] in (2, 4, 8) and t["neighborWarps"] in (2, 4, 8)
    assert 0.0 < t["gravityMs"] < 1.0e3 and 0.0 < t["neighborMs"] < 1.0e3
    assert engine.get_tuning(n) == t
    assert engine.get_tuning(n + 1)["gravityWarps"] == t["gravityWarps"]       # same power-of-two bucket
    with pytest.raises(abi.AstraeaError):
        engine.set_tuning(n, 3, 4)
    engine.set_tuning(n, 4, 4)


@pytest.mark.gpu
def test_gpu_autotune_keeps_each_gravity_walk_its_own_shape():
    from astraea_gb300 import engine
    st, _ = scenarios.differentiated_impact(n_total=65536, seed=21)
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    engine.set_tuning(n, 2, 2)                   # a hand setting applies to every walk
    assert all(engine.get_gravity_warps(n, m, th) == 2 for m in (0, 1, 3) for th in (0.5, 0.7))
    try:
        engine.set_far_field(1)
        engine.sort_and_build_bvh(p, alt, bvh)
        t = engine.autotune(p, bvh, 0.7)             # the quadrupole walk with the inside-box rule
        assert engine.get_gravity_warps(n, 1, 0.7) == t["gravityWarps"]
        assert engine.get_gravity_warps(n, 1, 0.5) == 2      # the other walks keep theirs
        assert engine.get_gravity_warps(n, 0, 0.5) == 2
        assert engine.get_gravity_warps(n, 0, 0.7) == 2
        kept = engine.get_tuning(n)
        assert kept["gravityWarps"] == 2 and kept["neighborWarps"] == t["neighborWarps"]
    finally:
        engine.set_far_field(0)
        engine.set_tuning(n, 4, 4)
