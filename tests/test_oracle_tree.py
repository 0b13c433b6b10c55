"""Oracle Morton / sort / Karras / refit against independent restatements.

The reference's tests pin none of these bit for bit (its AC-9 only checks
tracer uniqueness across re-sorts, tests/cpp/test_conservation.cpp:197-258);
here the oracle is checked against direct numpy definitions: Morton codes by
explicit bit interleaving, the sort against numpy's stable argsort, and the
Karras tree by its defining properties (every internal node covers a
contiguous key range split at the highest differing bit).
"""
import numpy as np
import pytest

import oracle
from astraea_gb300 import scenarios


def morton_numpy(x, y, z):
    x, y, z = (np.asarray(a, np.float32) for a in (x, y, z))
    b = np.array([x.min(), y.min(), z.min(), x.max(), y.max(), z.max()], np.float32)
    codes = np.zeros(len(x), np.uint64)
    qs = []
    for k, a in enumerate((x, y, z)):
        span = np.float32(b[3 + k] - b[k])
        inv = np.float32(2097151.0) / span if span > np.float32(1e-6) else np.float32(0.0)
        f = np.minimum(np.maximum((a - b[k]).astype(np.float32) * np.float32(inv), np.float32(0)), np.float32(2097151.0))
        qs.append(f.astype(np.uint32).astype(np.uint64))
    for bit in range(21):
        for axis, shift in ((0, 2), (1, 1), (2, 0)):
            codes |= ((qs[axis] >> np.uint64(bit)) & np.uint64(1)) << np.uint64(3 * bit + shift)
    return codes, b


@pytest.mark.parametrize("seed", [0, 1])
def test_morton_matches_bit_interleave(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    x, y, z = (rng.normal(size=5000).astype(np.float32) for _ in range(3))
    c1, b1 = oracle.morton(x, y, z)
    c2, b2 = morton_numpy(x, y, z)
    assert np.array_equal(b1, b2)
    assert np.array_equal(c1, c2)
    assert int(c1.max()) < (1 << 63)


def test_morton_degenerate_span():
    x = np.full(100, 3.0, np.float32)
    codes, _ = oracle.morton(x, x, x)
    assert np.all(codes == 0)


def test_sort_is_stable_with_index_tiebreak():
    rng = np.random.Generator(np.random.PCG64(3))
    keys = rng.integers(0, 50, 10000).astype(np.uint64) << np.uint64(40)
    ks, perm = oracle.sort_pairs(keys)
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    assert np.array_equal(ks, np.sort(keys))


def _check_karras(codes, left, right, parent):
    n = len(codes)
    covered = np.zeros(n, np.int32)
    seen = np.zeros(n - 1, np.int32)

    def rng_of(c):
        if c < 0:
            return ~c, ~c
        return None

    # iterative: compute [first,last] of every internal node bottom-up via DFS
    first = np.zeros(n - 1, np.int64)
    last = np.zeros(n - 1, np.int64)
    order, st = [], [0]
    while st:
        v = st.pop()
        seen[v] += 1
        order.append(v)
        for c in (left[v], right[v]):
            if c >= 0:
                assert parent[c] == v
                st.append(c)
            else:
                covered[~c] += 1
                assert parent[n - 1 + ~c] == v
    for v in reversed(order):
        lf = (~left[v], ~left[v]) if left[v] < 0 else (first[left[v]], last[left[v]])
        rt = (~right[v], ~right[v]) if right[v] < 0 else (first[right[v]], last[right[v]])
        assert lf[1] + 1 == rt[0]          # children are adjacent key ranges
        first[v], last[v] = lf[0], rt[1]
    assert np.all(seen == 1) and np.all(covered == 1)
    assert first[0] == 0 and last[0] == n - 1 and parent[0] == -1


@pytest.mark.parametrize("n", [2, 3, 33, 1000])
def test_karras_tree_structure(n):
    rng = np.random.Generator(np.random.PCG64(n))
    keys = np.sort(rng.integers(0, 1 << 20, n).astype(np.uint64))   # duplicates included
    left, right, parent = oracle.karras(keys)
    _check_karras(keys, left, right, parent)


def test_sort_and_build_refit_conserves_mass_and_permutes():
    st, _ = scenarios.two_granite_spheres(n_target=768, n_impactor=256, seed=5)
    o = oracle.Oracle(st)
    o.sort_and_build()
    s = o.state()
    assert np.array_equal(np.sort(s["originalId"]), np.arange(1024))
    assert np.array_equal(s["posX"], st["posX"][s["originalId"]])
    b = o.bvh.a
    assert abs(float(b["nodeMass"][0]) - float(np.sum(st["mass"], dtype=np.float64))) < 1e-5 * float(b["nodeMass"][0])
    assert b["aabbMinX"][0] == st["posX"].min() and b["aabbMaxZ"][0] == st["posZ"].max()
