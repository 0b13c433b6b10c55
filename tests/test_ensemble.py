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
