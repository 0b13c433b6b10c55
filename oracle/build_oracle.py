"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* oracle/_build/liboracle.so -- the CPU restatement in oracle/oracle.cpp,
  compiled with OpenMP and with multiply-add contraction off
  (-ffp-contract=off) so its float arithmetic rounds like the reference
  expressions it restates, on x86_64 and aarch64 alike.
* oracle/_ref/libref_pcls.so -- the reference's server/binary_protocol.cpp
  (PCLS frame builder) behind oracle/ref_pcls_capi.cpp, same conditions.
* oracle/_ref/libref_eos.so -- the reference's own engine/eos.cu compiled as
  host C++ from the reference checkout where it lies (only when that checkout
  exists; it is absent on GPU machines, which use the committed golden
  vectors instead).  Nothing of the reference is copied into this tree.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# The reference checkout this recipe compiles from: ASTRAEA_REFERENCE_ENGINE
# when set, else the checkout's usual place on the build machine.  It is
# absent on GPU machines; every step that needs it is skipped there.
REFERENCE_ENGINE = os.environ.get("ASTRAEA_REFERENCE_ENGINE", "/root/reference/engine")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(ROOT, "include", "astraea_gb300.h")]
    if force or _stale(out, srcs):
        tmp = out + ".tmp%d" % os.getpid()
        _run(["g++"] + CXXFLAGS + ["-fopenmp", "-I", os.path.join(ROOT, "include"), srcs[0], "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_eos(force=False):
    """Compile the reference EOS as host C++; returns the path or None."""
    eos_cu = os.path.join(REFERENCE_ENGINE, "eos.cu")
    if not os.path.exists(eos_cu):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libref_eos.so")
    shim = os.path.join(HERE, "ref_eos_capi.cpp")
    if force or _stale(out, [eos_cu, shim]):
        tmp = out + ".tmp%d" % os.getpid()
        _run(["g++"] + CXXFLAGS + ["-I", REFERENCE_ENGINE, "-x", "c++", eos_cu, "-x", "none", shim, "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_cubin(force=False):
    """The reference kernels (engine/eos.cu + engine/sph_gravity.cu) as one
    sm_100 cubin, from the checkout where they lie; None where absent."""
    srcs = [os.path.join(REFERENCE_ENGINE, f) for f in ("eos.cu", "sph_gravity.cu", "sph_gravity.cuh", "eos.hpp")]
    if not all(os.path.exists(x) for x in srcs):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "ref_kernels_sm100.cubin")
    shim = os.path.join(HERE, "ref_cubin.cu")
    if force or _stale(out, srcs + [shim]):
        tmp = out + ".tmp%d" % os.getpid()
        _run(["nvcc", "-cubin", "-arch=sm_100", "-O3", "--expt-relaxed-constexpr", "-std=c++20",
              "-I", REFERENCE_ENGINE, shim, "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_pcls(force=False):
    """The reference's PCLS frame builder (server/binary_protocol.cpp, host
    C++ with zlib) behind a C entry point; None where the checkout or zlib is
    absent."""
    server = os.path.join(os.path.dirname(REFERENCE_ENGINE), "server")
    src = os.path.join(server, "binary_protocol.cpp")
    if not os.path.exists(src) or not os.path.exists("/usr/include/zlib.h"):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libref_pcls.so")
    shim = os.path.join(HERE, "ref_pcls_capi.cpp")
    if force or _stale(out, [src, shim]):
        tmp = out + ".tmp%d" % os.getpid()
        _run(["g++"] + CXXFLAGS + ["-I", REFERENCE_ENGINE, "-I", server, src, shim, "-lz", "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_planet(force=False):
    """The reference's PlanetBuilder (engine/planet_builder.cpp with
    engine/presets.cpp and engine/eos.cu as host C++) behind the C entry
    points of oracle/ref_planet_capi.cpp; None where the checkout is absent."""
    srcs = [os.path.join(REFERENCE_ENGINE, f) for f in ("planet_builder.cpp", "presets.cpp", "eos.cu")]
    if not all(os.path.exists(x) for x in srcs):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libref_planet.so")
    shim = os.path.join(HERE, "ref_planet_capi.cpp")
    if force or _stale(out, srcs + [shim]):
        tmp = out + ".tmp%d" % os.getpid()
        _run(["g++"] + CXXFLAGS + ["-I", REFERENCE_ENGINE, srcs[0], srcs[1], "-x", "c++", srcs[2], "-x", "none",
                                   shim, "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_sim(force=False):
    """The reference engine's own host code (engine/simulation.cpp with
    planet_builder.cpp, presets.cpp and eos.cu as host C++) run on the CPU
    behind oracle/ref_sim_harness.cpp: the CUDA runtime calls over host memory,
    the kernels from the oracle library.  None where the checkout is absent."""
    srcs = [os.path.join(REFERENCE_ENGINE, f) for f in ("simulation.cpp", "planet_builder.cpp", "presets.cpp",
                                                         "eos.cu")]
    cuda_inc = "/usr/local/cuda/include"
    if not all(os.path.exists(x) for x in srcs) or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        return None
    lib_dir = os.path.dirname(build_oracle())
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libref_sim.so")
    shim = os.path.join(HERE, "ref_sim_harness.cpp")
    if force or _stale(out, srcs + [shim, os.path.join(lib_dir, "liboracle.so")]):
        tmp = out + ".tmp%d" % os.getpid()
        flags = [f for f in CXXFLAGS if not f.startswith("-std=")] + ["-std=c++20"]
        _run(["g++"] + flags + ["-I", os.path.join(ROOT, "include"), "-I", REFERENCE_ENGINE, "-I", cuda_inc, shim,
                                srcs[1], srcs[2], "-x", "c++", srcs[3], "-x", "none", "-L", lib_dir, "-loracle",
                                "-Wl,-rpath," + lib_dir, "-Wl,-Bsymbolic", "-o", tmp])
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference_eos(force="--force" in sys.argv))
    print(build_reference_cubin(force="--force" in sys.argv))
    print(build_reference_pcls(force="--force" in sys.argv))
    print(build_reference_planet(force="--force" in sys.argv))
