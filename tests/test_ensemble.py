"""Batched ensemble: independent impacts advanced by one CUDA graph.

Two ensembles are built from the same seeded instances; one is stepped
eagerly instance after instance, the other captures two fused steps of every
instance (each on its own stream) into one graph and replays it.  The
instances are independent and every kernel is deterministic, so after the
same number of steps both hold bit-identical states.
"""
import numpy as np
import pytest

from astraea_gb300 import scenarios

FIELDS = ("posX", "posY", "posZ", "velX", "velY", "velZ", "rho", "u", "h", "accX", "accY", "accZ", "phiGrav",
          "pressure", "originalId")


def test_ensemble_configs_follow_the_workload():
    cfgs = scenarios.ensemble_configs()
    assert len(cfgs) == 64
    ns = np.array([c["n_total"] for c in cfgs])
    assert ns.min() >= 8192 and ns.max() <= 131072
    assert {c["material"] for c in cfgs} <= {0, 1, 2, 4}
    assert all(0.0 <= c["angle_deg"] <= 75.0 and 1.0 <= c["v_ratio"] <= 3.0 for c in cfgs)
    st, _ = scenarios.ensemble_impact(**cfgs[0])
    assert len(st["posX"]) == cfgs[0]["n_total"]


@pytest.mark.gpu
def test_graph_replay_matches_eager_steps():
    import torch
    from astraea_gb300 import engine
    cfgs = scenarios.ensemble_configs(count=5, n_min=3000, n_max=20000, seed=3)
    states = [scenarios.ensemble_impact(**c)[0] for c in cfgs]
    max_dt = 5.0e-3
    eager = engine.Ensemble(states, max_dt)
    graph = engine.Ensemble(states, max_dt)
    eager.step_sequential(2 + 4)
    graph.capture()                      # runs the same 2 priming steps, then records 2
    graph.replay(2)                      # 4 more steps
    torch.cuda.synchronize()
    for a, b in zip(eager.sims, graph.sims):
        da, db = a.p.download(FIELDS), b.p.download(FIELDS)
        for f in FIELDS:
            assert np.array_equal(da[f], db[f]), f


@pytest.mark.gpu
def test_graph_replay_gates_every_instance_in_learned_mode():
    """Far-field mode 2 in the ensemble graph.  Every BVH keeps its own pair
    records, corrections and gate state, so the instances' branches run
    concurrently and each is gated on its own spot check, on the device.
    A tolerance no spot check meets sends every gated call back to the plain
    walk: graph and eager stepping then give bit-identical states, and each
    instance counts one fallback per gravity call (the initial forces, two
    priming steps, four replayed steps).  A tolerance every check meets keeps
    the learned result without fallbacks (graph against eager within the
    float atomics of the correction sums)."""
    import torch
    from astraea_gb300 import engine
    cfgs = scenarios.ensemble_configs(count=4, n_min=3000, n_max=12000, seed=5)
    states = [scenarios.ensemble_impact(**c)[0] for c in cfgs]
    max_dt = 5.0e-3
    engine.ff_init(7)
    try:
        engine.set_far_field(2)
        results = {}
        for tag, tol in (("fail", 1e-9), ("pass", 10.0)):
            engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=tol, gate_targets=16)
            eager = engine.Ensemble(states, max_dt, autotune_walks=False)
            eager.step_sequential(2 + 4)
            before = engine.ff_stats()["fallbacks"]
            graph = engine.Ensemble(states, max_dt, autotune_walks=False)
            graph.capture()
            graph.replay(2)
            torch.cuda.synchronize()
            results[tag] = (eager, graph, engine.ff_stats()["fallbacks"] - before)
    finally:
        engine.ff_configure(theta_far=0.9, gamma=0.3, gate_tolerance=0.0)
        engine.set_far_field(0)
    eager, graph, fallbacks = results["fail"]
    assert fallbacks == len(states) * 7
    for a, b in zip(eager.sims, graph.sims):
        da, db = a.p.download(FIELDS), b.p.download(FIELDS)
        for f in FIELDS:
            assert np.array_equal(da[f], db[f]), f
    eager, graph, fallbacks = results["pass"]
    assert fallbacks == 0
    for a, b in zip(eager.sims, graph.sims):
        da, db = a.p.download(FIELDS), b.p.download(FIELDS)
        assert np.array_equal(da["originalId"], db["originalId"])
        for f in ("posX", "velX", "accX", "accY", "accZ"):
            err = np.sqrt(np.sum((da[f].astype(np.float64) - db[f]) ** 2) / np.sum(db[f].astype(np.float64) ** 2))
            assert err < 1e-5, (f, err)
