"""Generates tests/golden/pcls_frames.npz: uncompressed PCLS frames built by
the reference's own frame builder (server/binary_protocol.cpp:155-217, via
oracle/ref_pcls_capi.cpp) from records packed by the oracle.

Run from the repository root in a checkout that has the reference sources
(oracle/build_oracle.py finds them) and zlib:
    python tests/golden/make_pcls_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "astraea-impact-sim_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

CASES = [
    dict(n=600, tracers=100, seed=3, sim_time=3605.25, frame_seq=41, dt_sec=0.0125, grid_res=16, living=True,
         speed=True, living_com=(0.5, -0.25, 0.125), sys_com=(0.0625, 0.03125, -0.5)),
    dict(n=257, tracers=0, seed=4, sim_time=1.0e7, frame_seq=(1 << 32) + 9, dt_sec=2.5, grid_res=16, living=False,
         speed=False, living_com=(0.0, 0.0, 0.0), sys_com=(1.0, 2.0, 3.0)),
    dict(n=0, tracers=0, seed=5, sim_time=0.0, frame_seq=0, dt_sec=0.0, grid_res=0, living=True, speed=True,
         living_com=(0.0, 0.0, 0.0), sys_com=(0.0, 0.0, 0.0)),
]


def case_inputs(c):
    st = oracle.random_render_state(max(c["n"], 64), c["tracers"], c["seed"])
    st = {k: v[: c["n"]] for k, v in st.items()}
    info = oracle.frame_info(c["sim_time"], c["frame_seq"], c["dt_sec"], c["tracers"], c["grid_res"], c["living"],
                             c["speed"], c["living_com"], c["sys_com"])
    return st, info


def main():
    ref = oracle.load_reference_pcls()
    if ref is None:
        raise SystemExit("reference sources or zlib not found")
    out = {}
    for k, c in enumerate(CASES):
        st, info = case_inputs(c)
        rec, spd = oracle.pack_render_records(st, c["sys_com"], speed=True)
        trc = oracle.extract_tracers(st, c["tracers"], c["living_com"], c["sys_com"])
        cap = 64 + rec.size + trc.size + spd.size
        buf = np.zeros(cap, np.uint8)
        sp = spd if c["speed"] else None
        size = ref.ref_build_frame(rec.ctypes.data, rec.size, trc.ctypes.data, trc.size,
                                   sp.ctypes.data if sp is not None else None, sp.size if sp is not None else 0,
                                   c["sim_time"], c["frame_seq"], c["dt_sec"], int(c["living"]), c["grid_res"], 0,
                                   buf.ctypes.data, cap)
        assert size > 0
        out["frame%d" % k] = buf[:size]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pcls_frames.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.size for k, v in out.items()})


if __name__ == "__main__":
    main()
