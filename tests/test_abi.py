"""The C-ABI library exists, loads, and exports what include/astraea_gb300.h
declares; the ctypes structs match the header's layout.  No device calls."""
import ctypes
import os
import re

import pytest

from astraea_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "astraea_gb300.h")) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(astraea_gb300_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(abi.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_covers_header():
    assert sorted(abi.EXPORTED_SYMBOLS) == declared_functions()


def test_library_loads_and_reports_abi():
    lib = abi.load_library()
    assert lib.astraea_gb300_abi_version() == 1


def test_struct_layouts_match_engine_descriptors():
    # 2 x u32 + 56 pointers (engine/types.hpp:114-161)
    assert ctypes.sizeof(abi.Particles) == 456
    assert abi.Particles.posX.offset == 8 and abi.Particles.tracerIsOcean.offset == 8 + 55 * 8
    # u32 + pad + 19 pointers + void* + size_t + 6 pointers (engine/sph_gravity.cuh:26-59)
    assert abi.RadixBvh.mortonCodes.offset == 8
    assert abi.RadixBvh.cubTempStorage.offset == 8 + 19 * 8
    assert ctypes.sizeof(abi.RadixBvh) == 8 + 19 * 8 + 16 + 48


def test_error_path_without_gpu_is_an_exception():
    # A stage call on a descriptor with no arrays must fail cleanly (status,
    # not a crash): count 0 is a no-op, a missing BVH is INVALID.
    lib = abi.load_library()
    p = abi.Particles()
    assert lib.astraea_gb300_clear_stats(ctypes.byref(p)) == 0
    b = abi.RadixBvh()
    p.count = 10
    rc = lib.astraea_gb300_sph_pass1_neighbors(ctypes.byref(p), ctypes.byref(b))
    assert rc == 3
    assert b"leftChild" in lib.astraea_gb300_last_error()


def test_mode_setters_reject_out_of_range_arguments():
    # process-wide settings are checked before anything touches a device
    lib = abi.load_library()
    assert lib.astraea_gb300_set_node_rounding(2) == 3
    assert b"node rounding" in lib.astraea_gb300_last_error()
    assert lib.astraea_gb300_set_node_rounding(-1) == 3
    assert lib.astraea_gb300_set_far_field(4) == 3
    assert lib.astraea_gb300_set_far_field_expansion(33, 0.3) == 3
    assert lib.astraea_gb300_set_far_field_expansion(8, 1.0) == 3
    assert lib.astraea_gb300_set_node_rounding(0) == 0
    assert lib.astraea_gb300_set_far_field(0) == 0
    assert lib.astraea_gb300_set_far_field_expansion(16, 0.3) == 0
    w = ctypes.c_uint32(0)
    assert lib.astraea_gb300_get_gravity_warps(1024, 4, 0.5, ctypes.byref(w)) == 3
    assert b"far-field mode" in lib.astraea_gb300_last_error()
    assert lib.astraea_gb300_get_gravity_warps(1024, 0, 0.5, None) == 3
