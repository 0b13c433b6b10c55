"""Parity at the two large configurations of the workload table:

* the 4M Plummer sphere (gravity only): the tree bit for bit against the
  oracle; with the engine's node rounding the oracle's own node data equal
  to the library's bit for bit; on every 16th group of 32 the exact
  interaction count and the accelerations and potential within 1e-5;
* the 16M gas-giant core impact: the tree, node data and every permuted
  field bit for bit; the same gravity checks on every 256th group.

The oracle walks only the sampled groups (oracle.set_group_stride), so the
CPU side finishes in seconds; the GPU walks every group.
"""
import numpy as np
import pytest
import torch

import oracle
from astraea_gb300 import abi, engine, scenarios
from conftest import rel_rms

pytestmark = pytest.mark.gpu


def check(st, stride, tag):
    n = len(st["posX"])
    p, alt = engine.DeviceParticles(n), engine.DeviceParticles(n)
    p.upload(st)
    alt.count = n
    bvh = engine.TorchBvh(n, packed=True)
    engine.set_node_rounding(1)
    try:
        engine.sort_and_build_bvh(p, alt, bvh)
    finally:
        engine.set_node_rounding(0)
    torch.cuda.synchronize()
    o = oracle.Oracle(st)
    o.sort_and_build()
    b = o.bvh.a
    t = lambda name, k: bvh.t[name][:k].cpu().numpy()
    assert np.array_equal(t("mortonCodesSorted", n).view(np.uint64), b["mortonCodesSorted"])
    assert np.array_equal(t("indicesSorted", n).view(np.uint32), b["indicesSorted"])
    assert np.array_equal(t("leftChild", n - 1), b["leftChild"][: n - 1])
    assert np.array_equal(t("rightChild", n - 1), b["rightChild"][: n - 1])
    for f in ("aabbMinX", "aabbMinY", "aabbMinZ", "aabbMaxX", "aabbMaxY", "aabbMaxZ", "nodeMass", "comX", "comY",
              "comZ"):
        assert np.array_equal(t(f, 2 * n - 1), b[f]), f
    g, c = p.download(), o.state()
    for f in abi.FIELD_NAMES:
        assert np.array_equal(g[f], c[f]), f
    groups = engine.gravity_group_counts(p, bvh, 0.5)
    engine.gravity_barnes_hut(p, bvh, 0.5)
    g = p.download()
    try:
        oracle.set_group_stride(stride)
        cg = o.gravity_group_counts(0.5)
        o.gravity(0.5)
    finally:
        oracle.set_group_stride(1)
    c = o.state()
    sampled = np.arange(0, (n + 31) // 32, stride)
    bad = sampled[groups[sampled] != cg[sampled]]
    print("%s: %d sampled groups, interaction counts differ in %d" % (tag, sampled.size, bad.size))
    assert bad.size == 0, [(int(k), int(groups[k]), int(cg[k])) for k in bad[:10]]
    rows = (sampled[:, None] * 32 + np.arange(32)[None, :]).ravel()
    rows = rows[rows < n]
    errs = {f: rel_rms(g[f][rows], c[f][rows]) for f in ("accX", "accY", "accZ", "phiGrav")}
    print("%s gravity on the sampled groups: %s" % (tag, " ".join("%s=%.2e" % kv for kv in errs.items())))
    assert max(errs.values()) < 1e-5


def test_plummer_4m_tree_and_sampled_gravity():
    check(scenarios.plummer_sphere(4_000_000), 16, "4M Plummer")


def test_gas_giant_16m_tree_and_sampled_gravity():
    st, _ = scenarios.gas_giant_impact(n_total=16_000_000, n_impactor=2_000_000, seed=42)
    check(st, 256, "16M gas giant")
