"""Regenerate tests/golden/*.npz from the reference implementation.

eos_reference.npz: (material, rho, u, damage) -> (P, cs, T, phase) evaluated
by the reference's own engine/eos.cu, compiled as host C++ from the reference
checkout by oracle/build_oracle.py into oracle/_ref/libref_eos.so.  The
states sweep every material over compressed, cold-expanded, two-phase,
hot-expanded and damaged-tension regimes (the regimes of
tests/cpp/test_eos.cpp:164-275) plus random states.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402

RHO0 = {0: 7800.0, 1: 2680.0, 2: 1000.0, 3: 0.178, 4: 2000.0}
CV = {0: 449.0, 1: 790.0, 2: 4184.0, 3: 8260.0, 4: 800.0}
ECV = {0: 8.67e6, 1: 1.8e7, 2: 2.68e6, 3: 1.0e7, 4: 1.8e7}


def eos_states(seed=7, per_mat=1200):
    rng = np.random.Generator(np.random.PCG64(seed))
    mats, rhos, us, ds = [], [], [], []
    for m in range(5):
        rho0 = RHO0[m] / 1e6
        eta = np.concatenate([
            rng.uniform(0.05, 0.95, per_mat // 4),        # expanded
            rng.uniform(0.95, 1.05, per_mat // 4),        # near rho0 (cancellation zone)
            rng.uniform(1.05, 4.0, per_mat // 4),         # compressed
            np.exp(rng.uniform(np.log(1e-4), np.log(20.0), per_mat - 3 * (per_mat // 4))),
        ])
        T = np.exp(rng.uniform(np.log(5.0), np.log(3e4), len(eta)))
        u = (CV[m] * T + rng.uniform(0.0, 1.5, len(eta)) * ECV[m] * (rng.uniform(size=len(eta)) < 0.3)) / 1e6
        d = np.where(rng.uniform(size=len(eta)) < 0.3, rng.uniform(0.0, 1.0, len(eta)), 0.0)
        mats.append(np.full(len(eta), m, np.uint8))
        rhos.append((eta * rho0).astype(np.float32))
        us.append(u.astype(np.float32))
        ds.append(d.astype(np.float32))
    return np.concatenate(mats), np.concatenate(rhos), np.concatenate(us), np.concatenate(ds)


def main():
    mat, rho, u, dmg = eos_states()
    res = oracle.eos_batch(mat, rho, u, dmg, reference=True)
    if res is None:
        raise SystemExit("reference EOS library unavailable (needs the reference checkout)")
    P, cs, T, ph = res
    out = os.path.join(HERE, "eos_reference.npz")
    np.savez_compressed(out, mat=mat, rho=rho, u=u, dmg=dmg, P=P, cs=cs, T=T, phase=ph)
    print("wrote", out, len(mat))


if __name__ == "__main__":
    main()
