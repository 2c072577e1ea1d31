"""Large single solve with several sources (one matrix, many right-hand
sides) and print a JSON summary.

    python -m mesh2hrtf_gb300.large_case [--n 59] [--freq 16000] [--rhs 8]
        [--points 11950] [--fp64-check]

Mesh: the head-like scatterer (ellipsoid 0.09/0.075/0.11 m + two bumps,
graded) with 20 n^2 triangles (n = 59: 69620).  Sources: --rhs point
sources 1 mm off seeded surface points, one right-hand side each.  Grid:
--points quasi-uniform points (golden-angle spiral) on a 1.2 m sphere.
The product's roofline: each shared-matrix product reads A once
(N^2 * 8 bytes) for all right-hand sides; the engine's CUDA-event time of
the product launches over that.  --fp64-check also solves right-hand
side 0 in FP64 and reports the mixed solution's relative L2 difference.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import capi, meshes, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=59)
    ap.add_argument("--freq", type=float, default=16000.0)
    ap.add_argument("--rhs", type=int, default=8)
    ap.add_argument("--points", type=int, default=11950)
    ap.add_argument("--fp64-check", action="store_true")
    a = ap.parse_args()
    v, f, info = meshes.head_like(a.n)
    srcs = [meshes.surface_point_with_normal(v, f, 20261207 + r) for r in range(a.rhs)]
    pts = meshes.fibonacci_sphere(a.points, 1.2)
    n = len(f)
    t0 = time.perf_counter()
    mesh = capi.Mesh(v, f)
    t_mesh = time.perf_counter() - t0
    freqs = [workloads.frequency(capi, n, a.freq, s) for s in srcs]
    s = capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000, n_rhs=a.rhs)
    out = {"n_elements": n, "freq": a.freq, "rhs": a.rhs, "points": a.points, "mesh_upload_s": t_mesh}
    runs = []
    for rep in range(2):   # the first run includes one-time set-up (graph capture)
        t = time.perf_counter()
        xs, pots, grads, infos = s.solve_multi(freqs, pts)
        wall = time.perf_counter() - t
        i0 = infos[0]
        runs.append({"wall_s": wall, "assemble_ms": i0["assemble_ms"], "solve_ms": i0["solve_ms"],
                     "project_ms": i0["project_ms"], "matvec_ms": i0["matvec_ms"],
                     "iterations": [i["iterations"] for i in infos],
                     "rel_residual_max": max(i["rel_residual"] for i in infos)})
    r = runs[-1]
    steps = max(r["iterations"]) + 2 * 3   # Krylov products + refinement residuals (upper bound of launches)
    out["runs"] = runs
    out["matrix_bytes"] = n * n * 8.0
    out["product_launch_time_ms_mean"] = r["matvec_ms"] / max(1, steps)
    if a.fp64_check:
        s64 = capi.Solver(mesh, precision=capi.PREC_FP64, tol=1e-9, max_iter=3000)
        t = time.perf_counter()
        x64, p64, _ = s64.solve_frequency(freqs[0], pts)
        out["fp64_rhs0"] = {"wall_s": time.perf_counter() - t, **{k: s64.info.as_dict()[k] for k in
                            ("assemble_ms", "solve_ms", "project_ms", "iterations")}}
        out["mixed_rel_l2_err_rhs0"] = float(np.linalg.norm(xs[0] - x64) / np.linalg.norm(x64))
        out["mixed_rel_l2_err_pot_rhs0"] = float(np.linalg.norm(pots[0] - p64) / np.linalg.norm(p64))
        s64.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
