"""Solve one synthetic scattering case on the GPU and print a JSON summary.

    python -m tests.solve_case [--n-tri 8000] [--freq 5000]
        [--precision mixed|fp64] [--repeat 2] [--head]
        [--krylov-copy fp16|complex64|blr] [--bench-batch B]

Sphere (radius 0.1 m, geodesic mesh with --n-tri = 20 n^2 triangles) or the
head-like scatterer (--head), point source at 1 m, 1000 evaluation points at
1.2 m.  --bench-batch B solves the benchmark's workload instead (head-like
mesh of --n-tri triangles with its seed, source 1 mm off bump 1, 1730-point
grid) for its first B frequencies as one bem_solve_batch, --repeat times,
and prints each solver's Krylov steps and Krylov-copy bytes.  A small, fixed
workload for profilers (the commands under profiles/) and quick checks of a
device; not part of the library.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from mesh2hrtf_gb300 import capi, meshes, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-tri", type=int, default=8000)
    ap.add_argument("--freq", type=float, default=5000.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--head", action="store_true")
    ap.add_argument("--krylov-copy", default="fp16", choices=["fp16", "complex64", "blr"])
    ap.add_argument("--bench-batch", type=int, default=0)
    a = ap.parse_args()
    kcopy = {"fp16": False, "complex64": True, "blr": capi.KRYLOV_BLR}[a.krylov_copy]
    if a.bench_batch > 0:
        bench_batch(a, kcopy)
        return
    if a.head:
        v, f, info = meshes.head_like(int(round((a.n_tri / 20) ** 0.5)))
        src = info["source"]
    else:
        v, f = meshes.icosphere(a.n_tri, 0.1)
        src = [1.0, 0.0, 0.0]
    pts = meshes.random_sphere_points(1000, 1.2, 20261203)
    mesh = capi.Mesh(v, f)
    prec = capi.PREC_MIXED if a.precision == "mixed" else capi.PREC_FP64
    s = capi.Solver(mesh, precision=prec, tol=1e-9, complex64_krylov=kcopy)
    k = 2 * np.pi * a.freq / 343.0
    amp = 0.1 / (1j * 1.21 * 2 * np.pi * a.freq)
    fr = capi.Frequency(k, len(f), point_sources=src, point_amps=[amp])
    out = []
    for _ in range(a.repeat):
        t = time.perf_counter()
        x, pot, _ = s.solve_frequency(fr, pts)
        info = s.info.as_dict()
        info["wall_ms"] = (time.perf_counter() - t) * 1000
        out.append(info)
    print(json.dumps({"n": len(f), "freq": a.freq, "precision": a.precision, "runs": out}))


def bench_batch(a, kcopy):
    """The benchmark's first --bench-batch frequencies as one batch."""
    v, f, src, pts, freqs = workloads.head_workload(20261204, int(round((a.n_tri / 20) ** 0.5)))
    n = len(f)
    mesh = capi.Mesh(v, f)
    prec = capi.PREC_MIXED if a.precision == "mixed" else capi.PREC_FP64
    B = a.bench_batch
    ss = [capi.Solver(mesh, precision=prec, tol=1e-9, max_iter=3000, complex64_krylov=kcopy) for _ in range(B)]
    Fs = [workloads.frequency(capi, n, float(fr), src) for fr in freqs[:B]]
    runs = []
    for _ in range(a.repeat):
        t = time.perf_counter()
        res = capi.solve_batch(ss, Fs, [pts] * B)
        runs.append({"wall_ms": (time.perf_counter() - t) * 1000, "iterations": [r[3]["iterations"] for r in res]})
    copy = [s.krylov_copy_info()["bytes_per_product"] for s in ss] if a.krylov_copy == "blr" else None
    print(json.dumps({"n": n, "freqs": [float(x) for x in freqs[:B]], "runs": runs, "krylov_copy_bytes": copy}))


if __name__ == "__main__":
    main()
