"""Render-record / crust-tracer packing and the PCLS frame.

Pins:
  * tests/golden/pcls_frames.npz -- frames built by the reference's own
    frame builder (server/binary_protocol.cpp:155-217) from oracle-packed
    records (tests/golden/make_pcls_golden.py); the oracle must rebuild them
    byte for byte;
  * tests/golden/render_records.npz -- the reference's packRenderRecordsKernel
    and extractTracersKernel (engine/sph_gravity.cu:1586-1743) run on a GB300
    over a seeded edge-case state (oracle/ref_gpu.py golden_render).

The GB300 kernels use the same expressions and CUDA math functions as the
reference kernels, so on the GPU every byte must match the golden records
and the reference kernels themselves.  The oracle computes with the host C
library and without multiply-add contraction, so against the GPU bytes it is
held to: positions and temperatures exact, quantised bytes within one step,
derived floats within a few ulp of their inputs (normalDelta, an arccos near
+-1, to 2e-3 rad; the radial displacement to a few ulp of the radius).
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from astraea_gb300 import abi

RENDER_CASE = dict(n=2048, tracers=384, seed=11, sys_com=(0.125, -0.25, 0.0625), living_com=(0.5, 0.25, -0.125))


def decode_records(b):
    b = np.asarray(b, np.uint8).reshape(-1, 20)
    f = b[:, :12].copy().view(np.float32).reshape(-1, 3)
    return {"xyz": f, "temp": b[:, 12:14].copy().view(np.uint16)[:, 0], "pres": b[:, 14:16].copy().view(np.uint16)[:, 0],
            "mat": b[:, 16], "phase_body": b[:, 17], "dmg": b[:, 18], "rad": b[:, 19]}


def decode_tracers(b):
    b = np.asarray(b, np.uint8).reshape(-1, 40)
    head = b[:, :4].copy().view(np.uint16).reshape(-1, 2)
    return {"anchor": head[:, 0], "flags": head[:, 1], "f": b[:, 4:].copy().view(np.float32).reshape(-1, 9)}


def assert_records_close(got, ref):
    g, r = decode_records(got), decode_records(ref)
    assert np.array_equal(g["xyz"], r["xyz"])
    for k in ("mat", "phase_body"):
        assert np.array_equal(g[k], r[k]), k
    for k in ("temp", "pres", "dmg", "rad"):
        d = np.abs(g[k].astype(np.int64) - r[k].astype(np.int64))
        assert d.max() <= 1, (k, int(d.max()))
        assert np.mean(d > 0) < 0.01, k


def assert_tracers_close(got, ref):
    g, r = decode_tracers(got), decode_tracers(ref)
    assert np.array_equal(g["anchor"], r["anchor"])
    assert np.mean(g["flags"] != r["flags"]) <= 0.005
    gf, rf = g["f"].astype(np.float64), r["f"].astype(np.float64)
    exact = [0, 1, 2, 5, 6]        # xKm, yKm, zKm, tempK, damage
    assert np.array_equal(g["f"][:, exact], r["f"][:, exact])
    # overpressure: a product chain, relative; dispKm = (r - r_rest) 1000 and
    # the tsunami height (dispKm x 1000 m) cancel, so their error is a few
    # ulp of r (|r| < 16 here: ulp 2e-6, x 1000 km) -- absolute bounds
    scale = np.maximum(np.abs(rf[:, 7]), 1e-3)
    assert np.max(np.abs(gf[:, 7] - rf[:, 7]) / scale) < 1e-5
    assert np.max(np.abs(gf[:, 3] - rf[:, 3])) < 8e-3
    assert np.max(np.abs(gf[:, 8] - rf[:, 8])) < 8.0
    assert np.max(np.abs(gf[:, 4] - rf[:, 4])) < 2e-3          # normalDelta [rad]


def render_inputs():
    c = RENDER_CASE
    return oracle.random_render_state(c["n"], c["tracers"], c["seed"])


# ------------------------------------------------------------------ CPU ----
def test_oracle_frames_match_reference_builder(golden_dir):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_pcls_golden", os.path.join(golden_dir, "make_pcls_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    gold = np.load(os.path.join(golden_dir, "pcls_frames.npz"))
    for k, c in enumerate(mk.CASES):
        st, info = mk.case_inputs(c)
        fr = oracle.pcls_frame(st, info)
        assert np.array_equal(fr, gold["frame%d" % k]), k


def test_frame_header_fields(golden_dir):
    gold = np.load(os.path.join(golden_dir, "pcls_frames.npz"))
    f = gold["frame0"]
    assert f[:4].tobytes() == b"SLCP"                   # magic 0x50434C53 little-endian
    hdr = f[:40].copy()
    assert hdr[4:6].view(np.uint16)[0] == 1
    flags = hdr[6:8].view(np.uint16)[0]
    assert flags == 2 | 4 | 8                           # tracers, living COM, speed array; no zlib
    n, t, grid, payload = hdr[24:40].view(np.uint32)
    assert (n, t, grid) == (600, 100, 16)
    assert payload == 20 * 600 + 40 * 100 + 600 == f.size - 40
    f1 = gold["frame1"][:40].copy()
    assert f1[6:8].view(np.uint16)[0] == 0 and f1[32:36].view(np.uint32)[0] == 0   # no tracers: grid res 0
    assert f1[16:20].view(np.uint32)[0] == 9            # frameSeq keeps its low 32 bits


def test_oracle_records_match_reference_kernel_golden(golden_dir):
    c = RENDER_CASE
    gold = np.load(os.path.join(golden_dir, "render_records.npz"))
    st = render_inputs()
    rec, spd = oracle.pack_render_records(st, c["sys_com"])
    assert_records_close(rec, gold["records"])
    d = np.abs(spd.astype(np.int64) - gold["speed"].astype(np.int64))
    assert d.max() <= 1 and np.mean(d > 0) < 0.01
    trc = oracle.extract_tracers(st, c["tracers"], c["living_com"], c["sys_com"])
    assert_tracers_close(trc, gold["tracers"])


def test_frame_size_query():
    lib = abi.load_library()
    out = ctypes.c_size_t(0)
    assert lib.astraea_gb300_pcls_frame_bytes(1000, 10, 1, ctypes.byref(out)) == 0
    assert out.value == 40 + 20000 + 400 + 1000
    assert lib.astraea_gb300_pcls_frame_bytes(0, 0, 1, ctypes.byref(out)) == 0
    assert out.value == 40


# ------------------------------------------------------------------ GPU ----
@pytest.fixture(scope="module")
def gpu_state():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from astraea_gb300 import engine
    st = render_inputs()
    p = engine.DeviceParticles(len(st["posX"]))
    p.upload(st)
    return st, p


@pytest.mark.gpu
def test_gpu_records_match_golden_and_reference_kernels(golden_dir, gpu_state):
    import torch
    from astraea_gb300 import engine
    import ref_gpu
    c = RENDER_CASE
    st, p = gpu_state
    gold = np.load(os.path.join(golden_dir, "render_records.npz"))
    n, t = c["n"], c["tracers"]
    rec = torch.zeros(20 * n, dtype=torch.uint8, device="cuda")
    spd = torch.zeros(n, dtype=torch.uint8, device="cuda")
    trc = torch.full((40 * t,), 0xAB, dtype=torch.uint8, device="cuda")
    engine.pack_render_records(p, rec, spd, c["sys_com"])
    engine.extract_tracers(p, trc, t, 16, c["living_com"], c["sys_com"])
    torch.cuda.synchronize()
    assert np.array_equal(rec.cpu().numpy(), gold["records"])
    assert np.array_equal(spd.cpu().numpy(), gold["speed"])
    assert np.array_equal(trc.cpu().numpy(), gold["tracers"])
    # and the reference kernels themselves, run now on this GPU
    K = ref_gpu.RefKernels()
    rrec = torch.zeros_like(rec)
    rspd = torch.zeros_like(spd)
    rtrc = torch.zeros_like(trc)
    ref_gpu.ref_pack_render(K, p, rrec, rspd, c["sys_com"])
    ref_gpu.ref_extract_tracers(K, p, rtrc, t, c["living_com"], c["sys_com"])
    torch.cuda.synchronize()
    assert torch.equal(rec, rrec) and torch.equal(spd, rspd) and torch.equal(trc, rtrc)


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [1, 2, 4, 8, 12])
def test_gpu_records_at_unaligned_destinations(gpu_state, offset):
    import torch
    from astraea_gb300 import engine
    c = RENDER_CASE
    st, p = gpu_state
    n, t = c["n"], c["tracers"]
    base = torch.zeros(20 * n, dtype=torch.uint8, device="cuda")
    engine.pack_render_records(p, base, None, c["sys_com"])
    buf = torch.full((20 * n + 64,), 0x5A, dtype=torch.uint8, device="cuda")
    view = buf[offset: offset + 20 * n]
    engine.pack_render_records(p, view, None, c["sys_com"])
    tb = torch.zeros(40 * t, dtype=torch.uint8, device="cuda")
    engine.extract_tracers(p, tb, t, 0, c["living_com"], c["sys_com"])
    tbuf = torch.full((40 * t + 64,), 0x5A, dtype=torch.uint8, device="cuda")
    engine.extract_tracers(p, tbuf[offset: offset + 40 * t], t, 0, c["living_com"], c["sys_com"])
    torch.cuda.synchronize()
    assert torch.equal(view, base)
    assert torch.all(buf[:offset] == 0x5A) and torch.all(buf[offset + 20 * n:] == 0x5A)
    assert torch.equal(tbuf[offset: offset + 40 * t], tb)
    assert torch.all(tbuf[:offset] == 0x5A) and torch.all(tbuf[offset + 40 * t:] == 0x5A)


@pytest.mark.gpu
def test_gpu_pcls_frame_matches_oracle_frame(gpu_state):
    import torch
    from astraea_gb300 import engine
    c = RENDER_CASE
    st, p = gpu_state
    n, t = c["n"], c["tracers"]
    info = oracle.frame_info(sim_time=86400.5, frame_seq=77, dt_sec=0.03, tracer_count=t, grid_res=16, living=True,
                             speed=True, living_com=c["living_com"], sys_com=c["sys_com"])
    size = engine.pcls_frame_bytes(n, t, True)
    frame = torch.zeros(size + 16, dtype=torch.uint8, device="cuda")
    got = engine.pack_pcls_frame(p, info, frame)
    torch.cuda.synchronize()
    assert got == size
    dev = frame[:size].cpu().numpy()
    ref = oracle.pcls_frame(st, info)
    assert dev.size == ref.size
    assert np.array_equal(dev[:40], ref[:40])
    assert_records_close(dev[40: 40 + 20 * n], ref[40: 40 + 20 * n])
    assert_tracers_close(dev[40 + 20 * n: 40 + 20 * n + 40 * t], ref[40 + 20 * n: 40 + 20 * n + 40 * t])
    ds = dev[40 + 20 * n + 40 * t:].astype(np.int64)
    rs = ref[40 + 20 * n + 40 * t:].astype(np.int64)
    assert np.abs(ds - rs).max() <= 1
    # a frame buffer one byte short is refused
    with pytest.raises(abi.AstraeaError):
        engine.pack_pcls_frame(p, info, frame[: size - 1])


@pytest.mark.gpu
def test_gpu_packing_no_ops(gpu_state):
    import torch
    from astraea_gb300 import engine
    st, p = gpu_state
    trc = torch.full((40,), 7, dtype=torch.uint8, device="cuda")
    engine.extract_tracers(p, trc, 0, 0)                 # tracerCount 0: untouched
    empty = engine.DeviceParticles(4)
    empty.count = 0
    rec = torch.full((80,), 9, dtype=torch.uint8, device="cuda")
    engine.pack_render_records(empty, rec, None)         # count 0: untouched
    engine.extract_tracers(empty, trc, 1, 0)             # count 0: zeroed record only
    torch.cuda.synchronize()
    assert torch.all(rec == 9)
    assert torch.all(trc == 0)
