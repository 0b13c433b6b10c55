"""GB300-native ASTRAEA per-step physics path (host side).

Import as `astraea_gb300` with this package's parent directory
(astraea-impact-sim_gb300/) on sys.path.  The compute lives in
libastraea_gb300.so (csrc/, sm_103a CUDA behind the C-ABI of
include/astraea_gb300.h); this package binds that library and mirrors the
engine's astraea::cuda launch interface (engine.py) and provides seeded
synthetic scenes (scenarios.py).
"""
from . import abi  # noqa: F401

__all__ = ["abi", "engine", "scenarios", "build"]


def build(force=False):
    """Compile libastraea_gb300.so for sm_103a (see build_lib.py)."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("astraea_gb300_build_lib", os.path.join(here, "build_lib.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)
