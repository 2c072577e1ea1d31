"""Build recipe for the native parts: the CUDA library libbem_gb300.so (sm_103a)
and the drop-in NumCalc executable.  Plain nvcc/g++ invocations, translation
units compiled in parallel; outputs stay inside the package tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(LIBDIR, "libbem_gb300.so")
NUMCALC_DIR = os.path.join(PKG, "numcalc")
NUMCALC_BIN = os.path.join(NUMCALC_DIR, "bin", "NumCalc")
NUMCALC_SRC = os.path.join(NUMCALC_DIR, "src")

CU_SOURCES = ["bem_api.cu", "bem_engine.cu", "bem_gmres.cu", "bem_kernels.cu", "bem_precond.cu", "bem_server.cu", "bem_static.cu", "bem_peaks.cu", "bem_direct.cu", "bem_tune.cu", "bem_blr.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "bem_gb300.h"))
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), "-c", s, "-o", o, "-O3", "-std=c++17", *ARCH, "-lineinfo",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
                         "-I", os.path.join(ROOT, "include")])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stderr)
    if force or _stale(LIB, objs):
        _run([nvcc(), "-shared", *ARCH, "-o", LIB, *objs, "-Xcompiler", "-fPIC"])
    return LIB


def build_numcalc() -> str:
    """Build the drop-in NumCalc executable (links libbem_gb300.so by rpath)."""
    _run(["make", "-s", "-C", NUMCALC_SRC])
    return NUMCALC_BIN


def build_all(verbose: bool = False):
    build_library(verbose)
    build_numcalc()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
