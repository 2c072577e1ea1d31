"""Projects for the FMM -estimate_ram checks: each recipe writes a Mesh2HRTF
project (mesh2hrtf_gb300.project) whose NC.inp asks for single- or
multilevel FMM, so that NumCalc's cluster set-up runs on it.  Used by
tests/golden/make_fmm_estimate_golden.py (with the reference NumCalc) and
tests/test_fmm_estimate.py (with the drop-in)."""
from __future__ import annotations

import os
import pathlib

import numpy as np

from mesh2hrtf_gb300 import meshes, project


def _project(root, v, f, freqs, method, n_pts=40, **sym):
    pts = meshes.random_sphere_points(n_pts, 1.0, 7) + np.asarray(sym.get("sym_coords", (0.0, 0.0, 0.0)))
    return project.Project(root=str(root), nodes=v, elems=f, eval_points=pts,
                           eval_elems=meshes.grid_triangles(pts), freqs=list(freqs),
                           point_sources=[(0.31, 0.27, 0.22, 0.1, 0.0)],
                           boundary=["ELEM 0 TO %d VELO 0.0 -1 0.0 -1" % (len(f) - 1)], method=method, **sym)


def _main1(wd, token, value):
    """Set a token of NC.inp's Main Parameters I line."""
    inp = pathlib.Path(wd) / "NC.inp"
    lines = inp.read_text().split("\n")
    i = lines.index("## 1. Main Parameters I") + 1
    t = lines[i].split(" ")
    t[token] = str(value)
    lines[i] = " ".join(t)
    inp.write_text("\n".join(lines))


def _main2(wd, token, value):
    inp = pathlib.Path(wd) / "NC.inp"
    lines = inp.read_text().split("\n")
    i = lines.index("## 2. Main Parameters II") + 1
    t = lines[i].split(" ")
    t[token] = str(value)
    lines[i] = " ".join(t)
    inp.write_text("\n".join(lines))


def _groups(root, wd, n_groups):
    """Spread the boundary elements over n_groups element groups
    (interleaved, so the groups' boxes overlap); group 1 is the evaluation
    grid's, so the boundary groups are 0, 2, 3, ..."""
    el = pathlib.Path(root) / "ObjectMeshes" / "Reference" / "Elements.txt"
    lines = el.read_text().strip("\n").split("\n")
    out = [lines[0]]
    for i, ln in enumerate(lines[1:]):
        tok = ln.split()
        g = i % n_groups
        out.append(" ".join(tok[:-1] + [str(g if g == 0 else g + 1)]))
    el.write_text("\n".join(out) + "\n")
    _main1(wd, 0, n_groups + 1)


def write(name, root):
    """Write case `name` under root; returns the NumCalc working folder."""
    head = lambda: meshes.head_like(16)[:2]   # 5120 triangles
    if name == "sphere1280_ml":
        v, f = meshes.icosphere(1280, 0.1)
        return project.write_project(_project(root, v, f, [10.0, 100.0, 500.0, 1000.0, 2000.0, 4000.0,
                                                            8000.0, 12000.0, 16000.0, 20000.0], 4))
    if name == "head5120_ml":
        v, f = head()
        return project.write_project(_project(root, v, f, np.arange(200.0, 20001.0, 1650.0), 4))
    if name == "head5120_sl":
        v, f = head()
        return project.write_project(_project(root, v, f, [30.0, 100.0, 1000.0, 5000.0, 10000.0, 20000.0], 1))
    if name == "head5120_descending":
        v, f = head()
        return project.write_project(_project(root, v, f, [16000.0, 8000.0, 4000.0, 2000.0, 1000.0, 500.0], 4))
    if name == "quads2400_ml":
        v, f = meshes.cube_sphere(20, 0.1)
        return project.write_project(_project(root, v, f, [500.0, 2000.0, 8000.0, 16000.0], 4))
    if name == "groups3_ml":
        v, f = meshes.icosphere(5120, 0.1)
        wd = project.write_project(_project(root, v, f, [1000.0, 4000.0, 12000.0], 4))
        _groups(root, wd, 3)
        return wd
    if name == "min_terms5_ml":
        v, f = meshes.perturbed_ellipsoid(16, 3)
        wd = project.write_project(_project(root, v, f, [1000.0, 6000.0, 15000.0], 4))
        _main1(wd, 3, 5)
        return wd
    if name == "min_terms10_sl":
        v, f = meshes.perturbed_ellipsoid(16, 3)
        wd = project.write_project(_project(root, v, f, [1000.0, 6000.0, 15000.0], 1))
        _main1(wd, 3, 10)
        return wd
    if name == "cluster_edge_ml":
        v, f = meshes.perturbed_ellipsoid(16, 5)
        wd = project.write_project(_project(root, v, f, [2000.0, 9000.0, 18000.0], 4))
        _main2(wd, 3, 0.04)
        return wd
    if name == "half3456_sl":       # one symmetric plane x = 0
        v, f = meshes.sphere_sector(24, 0.1, (0,), triangles=True)
        return project.write_project(_project(root, v, f, [500.0, 2000.0, 8000.0, 16000.0], 1,
                                              nsym=1, sym_planes=(1, 0, 0)))
    if name == "quarter2400_ml":    # antisymmetric y = 0, symmetric z = 0
        v, q = meshes.sphere_sector(40, 0.1, (1, 2))
        return project.write_project(_project(root, v, q, [1000.0, 6000.0, 12000.0, 20000.0], 4,
                                              nsym=2, sym_planes=(0, 2, 1)))
    if name == "octant2400_ml":     # three planes through an off-origin point
        c = (0.01, -0.02, 0.03)
        v, f = meshes.sphere_sector(40, 0.1, (0, 1, 2), center=c, triangles=True)
        return project.write_project(_project(root, v, f, [3000.0, 9000.0, 20000.0], 4,
                                              nsym=3, sym_planes=(1, 2, 3), sym_coords=c))
    raise KeyError(name)


CASES = ("sphere1280_ml", "head5120_ml", "head5120_sl", "head5120_descending", "quads2400_ml", "groups3_ml",
         "min_terms5_ml", "min_terms10_sl", "cluster_edge_ml", "half3456_sl", "quarter2400_ml", "octant2400_ml")

COUNT_PREFIXES = ("TBEM:", "SLFMM:", "MLFMM:", "Nearfield", "T Matrix", "D Matrix", "S Matrix", "Tmatrix",
                  "Total Nr", "RAM Est", "Number of entries right hand side", "Number of Matrix entries")


def count_lines(stdout):
    """The estimate's count lines of a NumCalc -estimate_ram run."""
    return [ln for ln in stdout.splitlines() if ln.startswith(COUNT_PREFIXES)]


def memory_txt(wd):
    return pathlib.Path(os.path.join(wd, "Memory.txt")).read_text()
