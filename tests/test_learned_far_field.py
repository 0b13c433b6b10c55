"""Far-field mode 2: the learned correction (astraea_gb300_ff_*).

CPU: the oracle's FP64 network gradient against central finite differences.
GPU (through the C-ABI):
  * forward and backward of the tensor-core kernels against the oracle with
    the same bfloat16 rounding points (sums in FP32 on the GPU, FP64 here);
  * training on the solver's own trees lowers the loss;
  * with the trained network the mode-2 accelerations are closer to the FP64
    direct sum than the same walk without the correction (the gain of the
    network over the method without it), and the gate falls back to the plain
    walk when its tolerance is not met.
"""
import numpy as np
import pytest

import oracle
from astraea_gb300 import abi, scenarios
from conftest import rel_rms


def random_params(seed=3, scale=0.3):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(abi.FF_PARAMS) * scale).astype(np.float32)


def random_rows(n, seed=4):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.0, 1.0, (n, 16)).astype(np.float32)
    X[:, 11:] = 0.0
    T = rng.standard_normal((n, 16)).astype(np.float32)
    T[:, 12:] = 0.0
    return X, T


def test_oracle_gradient_matches_finite_differences():
    params = random_params().astype(np.float64)
    X, T = random_rows(24)
    scale = np.linspace(0.5, 2.0, 16)
    _, g = oracle.ff_loss_grad(params, scale, X, T)
    rng = np.random.default_rng(5)
    for k in rng.choice(len(params), 40, replace=False):
        e = np.zeros_like(params)
        e[k] = 1e-6
        num = (oracle.ff_loss_grad(params + e, scale, X, T)[0] - oracle.ff_loss_grad(params - e, scale, X, T)[0]) / 2e-6
        assert abs(num - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, num, g[k])


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_oracle():
    import torch
    from astraea_gb300 import engine
    params = random_params()
    X, T = random_rows(1000)
    engine.ff_set_params(params, np.ones(16, np.float32))
    Xd = torch.from_numpy(X).cuda()
    Td = torch.from_numpy(T).cuda()
    y = engine.ff_predict(Xd).cpu().numpy().astype(np.float64)
    yref, _ = oracle.ff_forward(params, X, bf16=True)
    assert np.max(np.abs(y - yref)) <= 2e-3 * np.max(np.abs(yref)), np.max(np.abs(y - yref))
    g, loss = engine.ff_gradients(Xd, Td)
    lref, gref = oracle.ff_loss_grad(params, np.ones(16), X, T, bf16=True)
    assert loss == pytest.approx(lref, rel=2e-3)
    rel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    assert rel < 5e-3, rel
    # against the unrounded FP64 network: the bfloat16 operands cost ~1e-2
    _, g64 = oracle.ff_loss_grad(params, np.ones(16), X, T, bf16=False)
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) < 5e-2


def impact(n, seed):
    st, _ = scenarios.differentiated_impact(n_total=n, seed=seed)
    return st


def rms_vs_direct(got, st, sel):
    ref, _ = oracle.direct_gravity_f64(st, sel)
    a = np.stack([got[k] for k in ("accX", "accY", "accZ")], 1)[sel].astype(np.float64)
    e = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return float(np.sqrt(np.mean(e * e)))


@pytest.mark.gpu
def test_gpu_trained_correction_gains_over_uncorrected_walk():
    from astraea_gb300 import engine
    engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
    rows, hist = engine.train_far_field([impact(65536, 11), impact(65536, 12)], steps=800, batch=4096, lr=2e-3)
    assert rows > 10000
    assert hist[-1][1] < 0.5 * hist[0][1], hist
    params, scale = engine.ff_get_params()
    st = impact(65536, 13)
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    try:
        engine.set_far_field(2)
        engine.sort_and_build_bvh(p, alt, bvh)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        learned = p.download()
        engine.ff_set_params(np.zeros_like(params), scale)      # same walk, no correction
        engine.gravity_barnes_hut(p, bvh, 0.5)
        uncorrected = p.download()
        engine.ff_set_params(params, scale)
    finally:
        engine.set_far_field(0)
    engine.gravity_barnes_hut(p, bvh, 0.5)
    plain = p.download()
    sorted_state = {k: learned[k] for k in ("posX", "posY", "posZ", "mass", "h0")}
    sel = np.random.default_rng(2).choice(n, 1024, replace=False).astype(np.uint32)
    e_l = rms_vs_direct(learned, sorted_state, sel)
    e_u = rms_vs_direct(uncorrected, sorted_state, sel)
    e_p = rms_vs_direct(plain, sorted_state, sel)
    print("RMS force error: plain theta 0.5 %.3e, mode-2 walk uncorrected %.3e, with the trained network %.3e"
          % (e_p, e_u, e_l))
    assert e_l < 0.8 * e_u


@pytest.mark.gpu
def test_gpu_gate_falls_back_to_plain_walk():
    from astraea_gb300 import engine
    st = impact(16384, 21)
    n = len(st["posX"])
    engine.ff_init(7)
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    before = engine.ff_stats()["fallbacks"]
    try:
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=1e-9, gate_targets=32)
        engine.set_far_field(2)
        engine.sort_and_build_bvh(p, alt, bvh)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        gated = p.download()
    finally:
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
        engine.set_far_field(0)
    stats = engine.ff_stats()
    assert stats["fallbacks"] == before + 1 and stats["lastGateRms"] > 1e-9
    engine.gravity_barnes_hut(p, bvh, 0.5)
    plain = p.download()
    for f in ("accX", "accY", "accZ", "phiGrav"):
        assert np.array_equal(gated[f], plain[f]), f


@pytest.mark.gpu
def test_gpu_gate_that_passes_keeps_the_learned_result():
    """A gate whose tolerance the spot check meets: the plain walk launched
    after it returns at once (the decision is on the device), so the result is
    the learned mode's own and no fallback is counted."""
    from astraea_gb300 import engine
    st = impact(16384, 23)
    n = len(st["posX"])
    engine.ff_init(7)
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    before = engine.ff_stats()["fallbacks"]
    try:
        engine.set_far_field(2)
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
        engine.sort_and_build_bvh(p, alt, bvh)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        ungated = p.download()
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=10.0, gate_targets=32, gate_fp64_pairs=True)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        gated = p.download()
    finally:
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
        engine.set_far_field(0)
    stats = engine.ff_stats()
    assert stats["fallbacks"] == before and 0.0 < stats["lastGateRms"] < 10.0
    # the gate's own RMS against the host's FP64 direct sum at its 32 evenly
    # spaced sorted targets.  The RMS is of relative errors, so a relative
    # difference d between the two reference sums moves it by about d: the
    # device softens with eps = 0.8 h0 rounded to float (the walk's value),
    # the host in FP64, which leaves d ~ 1e-8 for the FP64 spot check; the
    # default FP32 pair terms (FP64 sums) add ~1e-6
    targets = np.array([k * (n - 1) // 31 for k in range(32)], np.uint32)
    sorted_state = {k: gated[k] for k in ("posX", "posY", "posZ", "mass", "h0")}
    host_rms = rms_vs_direct(gated, sorted_state, targets)
    print("gate RMS: device FP64 %.9e, FP64 direct sum %.9e" % (stats["lastGateRms"], host_rms))
    assert abs(stats["lastGateRms"] - host_rms) <= 5e-8
    try:
        engine.set_far_field(2)
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=10.0, gate_targets=32)
        engine.gravity_barnes_hut(p, bvh, 0.5)
        rms32 = engine.ff_stats()["lastGateRms"]
    finally:
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
        engine.set_far_field(0)
    print("gate RMS: device FP32 pairs %.9e" % rms32)
    assert abs(rms32 - host_rms) <= 2e-6
    engine.gravity_barnes_hut(p, bvh, 0.5)                    # the plain walk (mode 0 tree is the same)
    plain = p.download()
    for f in ("accX", "accY", "accZ"):
        # the correction sums are float atomics (order-dependent in the last bits)
        assert rel_rms(gated[f], ungated[f]) < 1e-6, f
        assert rel_rms(gated[f], plain[f]) > 1e-5, f


@pytest.mark.gpu
def test_gpu_mode2_refuses_without_moments_tree():
    from astraea_gb300 import engine
    st = impact(4096, 22)
    n = len(st["posX"])
    p, alt, bvh = engine.DeviceParticles(n), engine.DeviceParticles(n), engine.DeviceBvh(n)
    p.upload(st)
    alt.count = n
    engine.sort_and_build_bvh(p, alt, bvh)                     # mode 0 tree
    try:
        engine.set_far_field(2)
        with pytest.raises(abi.AstraeaError):
            engine.gravity_barnes_hut(p, bvh, 0.5)
    finally:
        engine.set_far_field(0)
