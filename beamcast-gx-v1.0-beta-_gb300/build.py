"""Builds libbcgx.so (the C-ABI library) in-tree for sm_103a.

Every translation unit is compiled in parallel; CUDA sources get exactly one
-gencode (compute_103a -> sm_103a). Host C++ is compiled without
floating-point contraction so the fp64 scene builder rounds like the Go
reference. Usage: python build.py [--verbose] [--ptxas-v]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbcgx.so")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + CSRC] + GENCODE
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-I" + CSRC]


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "bc_gx.h"))
    deps.append(os.path.join(HERE, "..", "include", "bc_host_scene.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, ptxas_v: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cu, cpp = _sources()
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append([NVCC] + CU_FLAGS + extra + ["-c", src, "-o", obj])
    cxx = shutil.which("g++") or "g++"
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cxx] + CXX_FLAGS + ["-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            for out in ex.map(lambda c: _run(c, verbose), jobs):
                logs.append(out)
    if jobs or not os.path.exists(LIB):
        _run([NVCC, "-shared", "-o", LIB] + objs + GENCODE + ["-lpthread"], verbose)
    if ptxas_v:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, ptxas_v="--ptxas-v" in sys.argv, force="--force" in sys.argv))
