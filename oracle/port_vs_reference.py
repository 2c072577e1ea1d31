"""Test infrastructure (oracle only): time the FP64 restatement ("port")
against the reference NumCalc, stage by stage, on the same project.

Both run single-threaded on one frequency of a head-like scatterer (the
benchmark's shape at 2420 and 5120 triangles: ellipsoid 0.09/0.075/0.11 m
with two seeded bumps, source 1 mm off bump 1, 1730-point 1.2 m grid), with
NumCalc's own solver settings: traditional BEM (methodBEM 0), threshold ILU
of scanning degree 0 (IPRECOND 0), CGS to 1e-9.

  reference  oracle/_ref/NumCalc (the reference's unmodified sources, built
             by oracle/Makefile); its NC.out stage times (whole seconds) and
             the process wall time
  port       oracle/bem_oracle.c: or_assemble, or_solve_cgs, or_project

Needs the reference build (MESH2HRTF_REFERENCE); prints a markdown table.

    python oracle/port_vs_reference.py [--sizes 11 16] [--freq 10000]
"""
from __future__ import annotations

import argparse
import os
import pathlib
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from mesh2hrtf_gb300 import meshes, project  # noqa: E402
from oracle import oracle_py as op  # noqa: E402
from oracle import refdump  # noqa: E402

RHO, C0 = 1.21, 343.0


def reference_run(wd):
    t0 = time.perf_counter()
    r = subprocess.run([refdump.REF_NUMCALC], cwd=wd, capture_output=True, text=True)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr)
    out = pathlib.Path(os.path.join(wd, "NC.out")).read_text()
    st = {}
    for key, name in (("Assembling the equation system", "assemble"), ("Solving the equation system", "solve"),
                      ("Post processing", "post")):
        m = re.search(re.escape(key) + r"\s*:\s*(\d+)", out)
        st[name] = int(m.group(1)) if m else None
    m = re.search(r"CGS solver: number of iterations = (\d+)", out)
    st["iterations"] = int(m.group(1)) if m else None
    st["wall"] = wall
    return st


def port_run(v, f, src, pts, fr):
    om = op.OracleMesh(v, f)
    k = 2 * np.pi * fr / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * fr)
    of = op.OracleFreq(k, src, [amp])
    t0 = time.perf_counter()
    A, b = op.assemble(om, of, nthreads=1)
    t1 = time.perf_counter()
    x, it, err, direct, stg = op.solve_cgs(A, b, precond=0, scan=0, nthreads=1, overwrite=True)
    t2 = time.perf_counter()
    phi, vel = op.boundary_fields(om, x)
    op.project(om, of, phi, vel, pts, nthreads=1)
    t3 = time.perf_counter()
    return {"assemble": t1 - t0, "solve": t2 - t1, "ilu": stg[0], "cgs": stg[1], "post": t3 - t2,
            "iterations": it, "wall": t3 - t0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=int, nargs="+", default=[11, 16])
    ap.add_argument("--freq", type=float, default=10000.0)
    a = ap.parse_args()
    if not refdump.available() and not refdump.build():
        raise SystemExit("reference build not available (set %s)" % refdump.REFERENCE_ENV)
    pts = meshes.equal_angle_grid(1.2, 5.0, 24)
    rows = []
    for n in a.sizes:
        v, f, info = meshes.head_like(n, seed=20261204)
        src = info["source"]
        tmp = tempfile.mkdtemp()
        p = project.Project(root=os.path.join(tmp, "p"), nodes=v, elems=f, eval_points=pts,
                            eval_elems=meshes.grid_triangles(pts), freqs=[a.freq],
                            point_sources=[(src[0], src[1], src[2], 0.1, 0.0)],
                            boundary=["ELEM 0 TO %d VELO 0.0 -1 0.0 -1" % (len(f) - 1)])
        wd = project.write_project(p)
        ref = reference_run(wd)
        port = port_run(v, f, src, pts, a.freq)
        rows.append((len(f), ref, port))
    print("| N | stage | reference NumCalc (s, NC.out) | port (s) | port / reference |")
    print("|---|---|---|---|---|")
    for n, ref, port in rows:
        for st in ("assemble", "solve", "post"):
            r = ref[st]
            print("| %d | %s | %s | %.2f | %s |" % (n, st, r, port[st], "%.2f" % (port[st] / r) if r else "-"))
        print("| %d | wall | %.2f | %.2f | %.2f |" % (n, ref["wall"], port["wall"], port["wall"] / ref["wall"]))
        print("| %d | CGS iterations | %s | %d | |" % (n, ref["iterations"], port["iterations"]))
        print("| %d | port solve split | | ILU %.2f + CGS %.2f | |" % (n, port["ilu"], port["cgs"]))


if __name__ == "__main__":
    main()
