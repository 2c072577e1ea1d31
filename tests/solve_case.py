"""Solve one synthetic scattering case on the GPU and print a JSON summary.

    python -m tests.solve_case [--n-tri 8000] [--freq 5000]
        [--precision mixed|fp64] [--repeat 2] [--head]

Sphere (radius 0.1 m, geodesic mesh with --n-tri = 20 n^2 triangles) or the
head-like scatterer (--head), point source at 1 m, 1000 evaluation points at
1.2 m.  A small, fixed workload for profilers (the commands under profiles/) and
quick checks of a device; not part of the library.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from mesh2hrtf_gb300 import capi, meshes


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-tri", type=int, default=8000)
    ap.add_argument("--freq", type=float, default=5000.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--head", action="store_true")
    a = ap.parse_args()
    if a.head:
        v, f, info = meshes.head_like(int(round((a.n_tri / 20) ** 0.5)))
        src = info["source"]
    else:
        v, f = meshes.icosphere(a.n_tri, 0.1)
        src = [1.0, 0.0, 0.0]
    pts = meshes.random_sphere_points(1000, 1.2, 20261203)
    mesh = capi.Mesh(v, f)
    prec = capi.PREC_MIXED if a.precision == "mixed" else capi.PREC_FP64
    s = capi.Solver(mesh, precision=prec, tol=1e-9)
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


if __name__ == "__main__":
    main()
