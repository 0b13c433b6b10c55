"""The C++ drop-in for engine/sph_gravity.cu (csrc/shim/sph_gravity_gb300.cpp).

Where the ASTRAEA engine's sources are available (their path comes from the
oracle's build recipe, oracle/build_oracle.py: ASTRAEA_REFERENCE_ENGINE, else
the checkout that recipe builds from), this compiles the shim against the engine's own headers -- its
static_asserts check the descriptor layouts -- links it with
libastraea_gb300, compiles the engine's Simulation (engine/simulation.cpp)
to an object file, and checks that every astraea::cuda symbol that object
needs is defined by the shim with the same C++ signature.  Compile and link
only: nothing runs on a GPU.
"""
import os
import re
import shutil
import subprocess

import pytest

from build_oracle import REFERENCE_ENGINE as ENGINE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"
SHIM = os.path.join(ROOT, "astraea-impact-sim_gb300", "csrc", "shim", "sph_gravity_gb300.cpp")
LIBDIR = os.path.join(ROOT, "astraea-impact-sim_gb300")


def _need():
    if not os.path.exists(os.path.join(ENGINE, "sph_gravity.cuh")):
        pytest.skip("engine sources not present")
    if shutil.which("g++") is None or shutil.which("nm") is None:
        pytest.skip("g++/nm missing")
    if not os.path.exists(os.path.join(LIBDIR, "libastraea_gb300.so")):
        pytest.skip("library not built")


def _symbols(path, defined):
    out = subprocess.run(["nm", "-C", "--defined-only" if defined else "--undefined-only", path],
                         capture_output=True, text=True, check=True).stdout
    # "<address> T name(args)" or "U name(args)"; names may contain spaces
    return {re.sub(r"^\s*[0-9a-fA-F]*\s*[A-Za-z]\s+", "", line).strip() for line in out.splitlines()
            if "astraea::cuda::" in line}


def test_shim_links_and_covers_the_engine(tmp_path):
    _need()
    shim_so = str(tmp_path / "libsph_gravity_gb300.so")
    subprocess.run(["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    "-I", ENGINE, "-I", CUDA_INC, SHIM, "-L", LIBDIR, "-lastraea_gb300",
                    "-Wl,-rpath," + LIBDIR, "-Wl,--no-undefined", "-o", shim_so],
                   check=True, capture_output=True, text=True)
    sim_o = str(tmp_path / "simulation.o")
    subprocess.run(["g++", "-std=c++20", "-c", "-I", ENGINE, "-I", CUDA_INC, os.path.join(ENGINE, "simulation.cpp"),
                    "-o", sim_o], check=True, capture_output=True, text=True)
    needed = _symbols(sim_o, defined=False)
    defined = _symbols(shim_so, defined=True)
    assert len(needed) >= 15
    missing = sorted(needed - defined)
    assert not missing, missing
    # and the BVH's member functions the engine's tests call
    assert "astraea::cuda::RadixBvhDevice::allocate(unsigned int)" in defined
    assert "astraea::cuda::RadixBvhDevice::free()" in defined
