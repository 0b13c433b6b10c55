"""Build recipe of the CUDA library libastraea_gb300.so (sm_103a).

Each translation unit under csrc/ is compiled by nvcc for
arch=compute_103a,code=sm_103a in parallel, then linked into one shared
library next to this file (in-tree, so the exact .so that runs is the one
built here).  Usage: python build_lib.py [--force] [--verbose-ptxas]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libastraea_gb300.so")
SOURCES = ["sort.cu", "build.cu", "gravity.cu", "sph.cu", "integrate.cu", "diag.cu", "render.cu", "telemetry.cu", "relax.cu", "planet.cu", "ff.cu", "noalloc.cu", "capi.cu"]
HEADERS = ["common.cuh", "internal.h", "kernels.h"]
# planet.cu reproduces the engine's host and device arithmetic operation for
# operation: no multiply-add contraction on either side.
EXTRA_FLAGS = {"planet.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]}

NVCC = os.environ.get("NVCC", "nvcc")
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr",
    "-I", os.path.join(ROOT, "include"),
    "-I", CSRC,
]


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res.stdout + res.stderr


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def build(force=False, verbose_ptxas=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "astraea_gb300.h"),
                                                        os.path.abspath(__file__)]
    dep_time = _newest(deps)
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(dep_time, os.path.getmtime(s)):
            flags = list(NVCC_FLAGS) + EXTRA_FLAGS.get(src, [])
            if verbose_ptxas:
                flags += ["-Xptxas", "-v"]
            jobs.append([NVCC] + flags + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if jobs or force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    return LIB, "".join(logs)


if __name__ == "__main__":
    lib, log = build(force="--force" in sys.argv, verbose_ptxas="--verbose-ptxas" in sys.argv)
    if log.strip():
        print(log)
    print(lib)
