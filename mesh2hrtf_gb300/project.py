"""Mesh2HRTF project folders: write NC.inp + mesh files, read be.out results.

The writer emits the dialect of the reference's exporter
(``mesh2hrtf/Mesh2Input/mesh2input.py:1170-1380``): the same section order,
frequency curve layout ("0 <nf+1>" then "t f/1e4e+04 0.0" lines), Main
Parameters I-IV and relative mesh paths, so the reference NumCalc and the
drop-in read identical inputs.  The reader follows the parser of the
reference's ``output2hrtf`` (``mesh2hrtf/Output2HRTF/output2hrtf.py:290-363``).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Project:
    root: str
    nodes: np.ndarray                 # (V, 3) boundary-mesh nodes
    elems: np.ndarray                 # (N, 3) or (N, 4) node indices
    eval_points: np.ndarray           # (M, 3)
    eval_elems: np.ndarray            # (Me, 3)
    freqs: list
    point_sources: list = field(default_factory=list)   # [(x, y, z, amp_re, amp_im)]
    plane_waves: list = field(default_factory=list)     # [(dx, dy, dz, amp_re, amp_im)]
    boundary: list = field(default_factory=lambda: [])  # raw "ELEM a TO b ..." lines
    method: int = 0                   # 0 TBEM, 1 SL-FMM, 4 ML-FMM
    precond: int = 0                  # Main Parameters II token 4
    solver: int = 0                   # 0 CGS, 4 direct
    speed_of_sound: float = 343.0
    density: float = 1.21
    node_id0: int = 0
    elem_id0: int = 0
    eval_node_id0: int = 200000
    eval_elem_id0: int = 200000
    grid_name: str = "Grid"
    title: str = "gb300 synthetic project"
    curves: list = field(default_factory=list)          # [(curve_id, [(f, v), ...])]
    nsym: int = 0
    sym_planes: tuple = (0, 0, 0)
    sym_coords: tuple = (0.0, 0.0, 0.0)


def _fmt(x: float) -> str:
    return "%.17e" % x


def write_project(p: Project, source_dir: str = "source_1") -> str:
    """Write the folder layout; returns the NumCalc working directory."""
    om = os.path.join(p.root, "ObjectMeshes", "Reference")
    eg = os.path.join(p.root, "EvaluationGrids", p.grid_name)
    nc = os.path.join(p.root, "NumCalc", source_dir)
    for d in (om, eg, nc):
        os.makedirs(d, exist_ok=True)
    nv = len(p.nodes)
    with open(os.path.join(om, "Nodes.txt"), "w", newline="\n") as fh:
        fh.write("%d\n" % nv)
        for i, (x, y, z) in enumerate(p.nodes):
            fh.write("%d %s %s %s\n" % (i + p.node_id0, _fmt(x), _fmt(y), _fmt(z)))
    with open(os.path.join(om, "Elements.txt"), "w", newline="\n") as fh:
        fh.write("%d\n" % len(p.elems))
        for e, con in enumerate(p.elems):
            ids = " ".join(str(int(c) + p.node_id0) for c in con)
            fh.write("%d %s 0 0 0\n" % (e + p.elem_id0, ids))
    with open(os.path.join(eg, "Nodes.txt"), "w", newline="\n") as fh:
        fh.write("%d\n" % len(p.eval_points))
        for i, (x, y, z) in enumerate(p.eval_points):
            fh.write("%d %s %s %s\n" % (i + p.eval_node_id0, _fmt(x), _fmt(y), _fmt(z)))
    with open(os.path.join(eg, "Elements.txt"), "w", newline="\n") as fh:
        fh.write("%d\n" % len(p.eval_elems))
        for e, con in enumerate(p.eval_elems):
            ids = " ".join(str(int(c) + p.eval_node_id0) for c in con)
            fh.write("%d %s 2 0 1\n" % (e + p.eval_elem_id0, ids))

    nf = len(p.freqs)
    n_el = len(p.elems) + len(p.eval_elems)
    n_nd = nv + len(p.eval_points)
    lines = [
        "##-------------------------------------------",
        "## This file was created by mesh2hrtf_gb300",
        "##-------------------------------------------",
        "Mesh2HRTF 1.0.0",
        "##",
        p.title,
        "##",
        "## Controlparameter I",
        "0 0 0 0 7 0",
        "##",
        "## Controlparameter II",
        "1 %d 0.000001 0.00e+00 1 0 0" % nf,
        "##",
        "## Load Frequency Curve ",
        "0 %d" % (nf + 1),
        "0.000000 0.000000e+00 0.0",
    ]
    for i, f in enumerate(p.freqs):
        lines.append("%f %fe+04 0.0" % (0.000001 * (i + 1), f / 10000.0))
    lines += [
        "##",
        "## 1. Main Parameters I",
        "2 %d %d 0 %d 2 1 %d %d" % (n_el, n_nd, p.nsym, p.method, p.solver),
        "##",
        "## 2. Main Parameters II",
        "%d %d 0 0.0000e+00 %d 0 0" % (len(p.plane_waves), len(p.point_sources), p.precond),
        "##",
        "## 3. Main Parameters III",
        "0 0 0 0",
        "##",
        "## 4. Main Parameters IV",
        "%s %se+00 1.0 0.0e+00 0.0 e+00 0.0e+00 0.0e+00" % (repr(float(p.speed_of_sound)), repr(float(p.density))),
        "##",
        "NODES",
        "../../ObjectMeshes/Reference/Nodes.txt",
        "../../EvaluationGrids/%s/Nodes.txt" % p.grid_name,
        "##",
        "ELEMENTS",
        "../../ObjectMeshes/Reference/Elements.txt",
        "../../EvaluationGrids/%s/Elements.txt" % p.grid_name,
        "##",
    ]
    if p.nsym > 0:
        lines += ["SYMMETRY", "%d %d %d" % tuple(p.sym_planes),
                  "%s %s %s" % tuple(_fmt(c) for c in p.sym_coords), "##"]
    lines += ["BOUNDARY"]
    lines += list(p.boundary)
    lines += ["RETU", "##"]
    if p.plane_waves:
        lines.append("PLANE WAVES")
        for i, (dx, dy, dz, ar, ai) in enumerate(p.plane_waves):
            lines.append("%d %s %s %s %s -1 %s -1" % (i, _fmt(dx), _fmt(dy), _fmt(dz), repr(float(ar)), repr(float(ai))))
        lines.append("##")
    if p.point_sources:
        lines.append("POINT SOURCES")
        for i, (x, y, z, ar, ai) in enumerate(p.point_sources):
            lines.append("%d %s %s %s %s -1 %s -1" % (i, _fmt(x), _fmt(y), _fmt(z), repr(float(ar)), repr(float(ai))))
        lines.append("##")
    if p.curves:
        lines.append("CURVES")
        lines.append("%d %d" % (len(p.curves), max(len(c[1]) for c in p.curves)))
        for cid, pts in p.curves:
            lines.append("%d %d" % (cid, len(pts)))
            for f, v in pts:
                lines.append("%s %s 0.0" % (repr(float(f)), repr(float(v))))
        lines.append("##")
    lines += ["POST PROCESS", "##", "END"]
    with open(os.path.join(nc, "NC.inp"), "w", newline="\n") as fh:
        fh.write("\n".join(lines) + "\n")
    return nc


def read_result(path: str):
    """Read one be.out/be.<k>/{p,v}{Boundary,EvalGrid} file.

    Returns (ids, values): ids as int array; values complex (M,) for the
    pressure/boundary files or complex (M, 3) for vEvalGrid.
    """
    ids, vals = [], []
    with open(path) as fh:
        for raw in fh:
            tok = raw.split()
            if len(tok) < 3 or tok[0].startswith("Mesh"):
                continue
            ids.append(int(tok[0]))
            nums = [float(t) for t in tok[1:]]
            if len(nums) == 2:
                vals.append(complex(nums[0], nums[1]))
            else:
                vals.append([complex(nums[2 * k], nums[2 * k + 1]) for k in range(len(nums) // 2)])
    return np.asarray(ids), np.asarray(vals)
