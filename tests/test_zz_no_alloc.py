"""The allocation-free radix sort entry point, through the C-ABI.

astraea_gb300_radix_sort_pairs_noalloc exists for callers that cannot let
the library call cudaMalloc (an arena or pool that owns the device memory,
or a host that forbids allocation after start-up).  Its scratch is a fixed
array inside the library image, shared by all calls.  These checks run it
twice in a row on different inputs and compare with the allocating
astraea_gb300_radix_sort_pairs (an integer sort: the outputs must be equal),
show that a repeated call leaves free device memory unchanged, that a call
above the fixed limit is refused with ASTRAEA_ERR_CAPACITY, and that a
look-back wait that gives up inside it is reported by the library's status
calls (its result is then unsorted, so it must not pass silently).

The file is named to be collected last, so a stop-at-first-failure run has
already run every other test when it gets here.
"""
import ctypes

import numpy as np
import pytest
import torch

from astraea_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu
MAX_KEYS = 1 << 20


def keys_and_values(seed, n, end_bit):
    rng = np.random.Generator(np.random.PCG64(seed))
    keys = rng.integers(0, 1 << 62, n, dtype=np.uint64) >> np.uint64(rng.integers(0, 40))
    keys[rng.integers(0, n, n // 3)] = keys[0]            # many equal keys: stability matters
    if end_bit == 64:
        keys |= rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63)
    vals = rng.permutation(n).astype(np.uint32)
    return (torch.from_numpy(keys.view(np.int64)).cuda(), torch.from_numpy(vals.view(np.int32)).cuda())


def sort_noalloc(keys, vals, end_bit):
    k_in, v_in = keys.clone(), vals.clone()
    k_out, v_out = torch.empty_like(keys), torch.empty_like(vals)
    abi.check(abi.load_library().astraea_gb300_radix_sort_pairs_noalloc(
        k_in.data_ptr(), k_out.data_ptr(), v_in.data_ptr(), v_out.data_ptr(), keys.numel(), end_bit))
    return k_out, v_out


def test_noalloc_sort_equals_allocating_sort_on_two_calls_in_a_row():
    for seed, n, end_bit in ((11, 300_001, 64), (12, MAX_KEYS, 63)):
        keys, vals = keys_and_values(seed, n, end_bit)
        k1, v1 = sort_noalloc(keys, vals, end_bit)
        k2, v2 = engine.radix_sort_pairs(keys, vals, end_bit)
        torch.cuda.synchronize()
        assert torch.equal(k1, k2) and torch.equal(v1, v2)
        kn = keys.cpu().numpy().view(np.uint64)
        mask = np.uint64((1 << end_bit) - 1) if end_bit < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
        order = np.argsort(kn & mask, kind="stable")
        assert np.array_equal(v1.cpu().numpy().view(np.uint32), vals.cpu().numpy().view(np.uint32)[order])


def test_noalloc_sort_allocates_nothing_per_call():
    keys, vals = keys_and_values(13, 200_000, 64)
    sort_noalloc(keys, vals, 64)                      # first call on this device: address set-up
    k_in, v_in = keys.clone(), vals.clone()
    k_out, v_out = torch.empty_like(keys), torch.empty_like(vals)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        abi.check(abi.load_library().astraea_gb300_radix_sort_pairs_noalloc(
            k_in.data_ptr(), k_out.data_ptr(), v_in.data_ptr(), v_out.data_ptr(), 200_000, 64))
        k_in.copy_(keys)
        v_in.copy_(vals)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_sort_refuses_more_than_its_limit():
    dummy = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = abi.load_library().astraea_gb300_radix_sort_pairs_noalloc(
        dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), MAX_KEYS + 1, 64)
    assert rc == 2
    assert b"limit" in abi.load_library().astraea_gb300_last_error()


def test_noalloc_sort_reports_a_lookback_timeout():
    """With a one-poll look-back limit some tiles give up waiting for their
    predecessors; every store stays inside the output (the sort checks each
    destination), the result is then not sorted, and the flag must reach
    read_device_status and the blocking dt call.  A result without the flag
    must be exactly sorted."""
    lib = abi.load_library()
    keys, vals = keys_and_values(14, MAX_KEYS, 64)
    kn = keys.cpu().numpy().view(np.uint64)
    expect = vals.cpu().numpy().view(np.uint32)[np.argsort(kn, kind="stable")]
    engine.reset_device_status()
    flagged_calls = 0
    try:
        abi.check(lib.astraea_gb300_set_lookback_spin_limit(1))
        for _ in range(20):
            _, v = sort_noalloc(keys, vals, 64)
            flags, _ = engine.read_device_status()
            if flags & abi.DEVFLAG_LOOKBACK_TIMEOUT:
                flagged_calls += 1
                break
            assert np.array_equal(v.cpu().numpy().view(np.uint32), expect)
    finally:
        abi.check(lib.astraea_gb300_set_lookback_spin_limit(0))   # back to the default limit
    assert flagged_calls == 1
    st, _ = scenarios.two_granite_spheres(n_target=48, n_impactor=16, seed=3)
    p = engine.DeviceParticles(64)
    p.upload(st)
    with pytest.raises(abi.AstraeaError) as ei:
        engine.reduce_dt_psu(p, 0.0, 1e-3)
    assert ei.value.status == 4
    engine.reset_device_status()
    flags, _ = engine.read_device_status()
    assert not flags & abi.DEVFLAG_LOOKBACK_TIMEOUT
    _, v = sort_noalloc(keys, vals, 64)
    flags, _ = engine.read_device_status()
    assert not flags & abi.DEVFLAG_LOOKBACK_TIMEOUT
    assert np.array_equal(v.cpu().numpy().view(np.uint32), expect)
