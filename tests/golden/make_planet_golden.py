"""Generates tests/golden/planet_builder.npz: outputs of the reference's own
PlanetBuilder (engine/planet_builder.cpp, built as a host library by
oracle/build_oracle.py behind oracle/ref_planet_capi.cpp).

* profile_<a>_*: solveHydrostatic1D of archetype a (0..5) with its default
  BodyInitSpec (engine/presets.cpp:9-88): the six profile columns, the
  radius and the central pressure;
* body_<k>_*: buildPlanet of the cases in BODIES, every field it returns
  (positions, velocities, mass, h0, rho, u, tempK, epsFail, materialId,
  bodyId and the tracer fields).

Run from the repository root in a checkout that has the reference sources:
    python tests/golden/make_planet_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "astraea-impact-sim_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402
from astraea_gb300 import engine  # noqa: E402

# (archetype, particle count, body id, tracer grid, seed): the reference
# test's determinism case (tests/cpp/test_planet_builder.cpp:271-274), a
# gas giant, and an impactor body with the second seed.
BODIES = [(0, 4000, 0, 8, 42), (4, 2000, 0, 8, 42), (5, 1500, 1, 0, 43)]
BODY_FIELDS = ("posX", "posY", "posZ", "velX", "velY", "velZ", "mass", "h0", "rho", "u", "tempK", "epsFail",
               "materialId", "bodyId", "tracerIndex", "tracerRestRadiusPsu", "tracerRestNormalX",
               "tracerRestNormalY", "tracerRestNormalZ", "tracerIsOcean")


def main():
    lib = oracle.load_reference_planet()
    if lib is None:
        raise SystemExit("reference sources not found")
    out = {}
    for a in range(6):
        prof, r, pc, _ = oracle.reference_solve_hydrostatic(lib, engine.body_spec(a))
        for k, v in prof.items():
            out["profile_%d_%s" % (a, k)] = v
        out["profile_%d_radius" % a] = np.float64(r)
        out["profile_%d_pc" % a] = np.float64(pc)
    out["bodies"] = np.array(BODIES, dtype=np.int64)
    for k, (a, n, body, grid, seed) in enumerate(BODIES):
        fields, info = oracle.reference_build_planet(lib, engine.body_spec(a), n, body, grid, seed)
        for f in BODY_FIELDS:
            out["body_%d_%s" % (k, f)] = fields[f]
        out["body_%d_info" % k] = np.array([info["equatorialRadiusM"], info["actualMassKg"],
                                            info["centralPressurePa"], info["tracerCount"]])
    path = os.path.join(ROOT, "tests", "golden", "planet_builder.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
