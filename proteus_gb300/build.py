"""Builds libgbjoin.so in-tree: every CUDA source compiled for sm_103a only.

Run as ``python -m proteus_gb300.build``.  Objects go to
``proteus_gb300/_build/``; the shared library to ``proteus_gb300/libgbjoin.so``.
Sources compile in parallel; no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbjoin.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, extra_nvcc=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    jobs = []
    for f in cu:
        obj = os.path.join(BUILD, f[:-3] + ".o")
        jobs.append([nvcc, *NVCC_FLAGS, *extra_nvcc, "-c", os.path.join(CSRC, f), "-o", obj])
    for f in cpp:
        obj = os.path.join(BUILD, f[:-4] + ".o")
        jobs.append(["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [j[-1] for j in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv,
                extra_nvcc=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
