"""Generate the parser-parity fixtures under tests/golden/parser/.

Each case is a small, self-contained NumCalc project (NC.inp + mesh files)
exercising one part of the NC.inp dialect.  The reference NumCalc's dump
harness (oracle/_ref/NumCalc_dump, built from the reference's sources by
oracle/Makefile) parses each one; the SHA-256 of every parsed table is stored
in digests.json, together with the reference's exit code and, for
-estimate_ram, its Memory.txt.  The drop-in's parse-only mode must reproduce
them bit for bit.

    python tests/golden/make_parser_cases.py
"""
from __future__ import annotations

import hashlib
import json
import os
import pathlib
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from mesh2hrtf_gb300 import meshes, project  # noqa: E402
from oracle import refdump  # noqa: E402

OUT = os.path.join(HERE, "parser")
TABLES = ["scalars_i", "node_ext", "node_class", "node_xyz", "elem_ext", "elem_nvert", "elem_prop",
          "elem_group", "elem_conn", "elem_dof", "elem_ibval", "elem_center", "elem_normals", "elem_area",
          "group_index", "group_count", "group_prop"]


def digest(arr):
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def table_digests(d):
    """Digests of the parsed tables; the normals of a triangle's (absent)
    fourth node are never written by NumCalc and are masked out."""
    out = {}
    for k in TABLES:
        if k not in d:
            continue
        a = d[k]
        if k == "elem_normals":
            a = a.reshape(-1, 15).copy()
            tri = d["elem_nvert"] == 3
            a[tri, 12:] = 0.0
        out[k] = digest(a)
    return out


def _write(p, name, mutate=None):
    root = os.path.join(OUT, name)
    shutil.rmtree(root, ignore_errors=True)
    p.root = root
    wd = project.write_project(p)
    if mutate:
        mutate(root, wd)
    return wd


def case_plain():
    v, f = meshes.icosphere(80, 0.1)
    pts = meshes.random_sphere_points(12, 0.4, 1)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[500.0, 1000.0, 1500.0], point_sources=[(0.3, 0.0, 0.1, 0.1, 0.0)],
                        boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"])
    return _write(p, "plain")


def case_dialect():
    """Comments, blank lines, runs of spaces, trailing blanks, a last line
    without newline, jumps in the numbering and a duplicated node id."""
    v, f = meshes.icosphere(80, 0.1)
    pts = meshes.random_sphere_points(10, 0.5, 2)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[700.0, 1400.0], plane_waves=[(0.0, 1.0, 1.0, 1.0, 0.5)],
                        boundary=["ELEM 1000 TO 1039 VELO 0.0 -1 0.0 -1", "ELEM 1040 TO 1079 PRES 0.0 -1 0.0 -1"],
                        node_id0=5, elem_id0=1000, eval_node_id0=90000, eval_elem_id0=95000)

    def mutate(root, wd):
        inp = os.path.join(wd, "NC.inp")
        txt = pathlib.Path(inp).read_text().split("\n")
        out = []
        for ln in txt:
            if ln.startswith("BOUNDARY"):
                out += ["", "# a comment line", "##   another  # comment", ln]
            elif ln.startswith("ELEM"):
                out.append(ln.replace(" ", "   ") + "   ")
            else:
                out.append(ln)
        pathlib.Path(inp).write_text("\n".join(out).rstrip("\n") + "\nEND\n")
        nodes = os.path.join(root, "ObjectMeshes", "Reference", "Nodes.txt")
        lines = pathlib.Path(nodes).read_text().split("\n")
        lines[3] = lines[3].replace(" ", "  ")
        pathlib.Path(nodes).write_text("\n".join(lines).rstrip("\n") + " ")   # no newline at the end
    return _write(p, "dialect", mutate)


def case_dup_node():
    """A node id given twice: elements bind to the first match; here the
    second node is left unreferenced, which the reference rejects."""
    v, f = meshes.icosphere(20, 0.1)
    pts = meshes.random_sphere_points(6, 0.4, 5)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[1000.0], point_sources=[(0.3, 0.0, 0.0, 0.1, 0.0)],
                        boundary=["ELEM 0 TO 19 VELO 0.0 -1 0.0 -1"])

    def mutate(root, wd):
        nodes = os.path.join(root, "ObjectMeshes", "Reference", "Nodes.txt")
        lines = pathlib.Path(nodes).read_text().split("\n")
        tok = lines[4].split(" ")
        lines[4] = " ".join(["1"] + tok[1:])       # node id 3 becomes a second id 1
        pathlib.Path(nodes).write_text("\n".join(lines))
    return _write(p, "dup_node", mutate)


def case_quads_groups():
    """Quadrilaterals and triangles in one file, three element groups,
    admittance and impedance lines, frequency curves."""
    v, q = __import__("make_golden").cube_sphere(3, 0.1)
    tri = np.array([[q[0][0], q[0][1], q[0][2]], [q[0][0], q[0][2], q[0][3]]])
    elems = [list(e) for e in q[1:]] + [list(t) + [-1] for t in tri]
    pts = meshes.random_sphere_points(8, 0.3, 3)
    p = project.Project(root="", nodes=v, elems=np.array([e[:4] for e in elems]), eval_points=pts,
                        eval_elems=meshes.grid_triangles(pts), freqs=[1000.0, 2000.0, 4000.0],
                        point_sources=[(0.0, 0.0, 0.4, 0.1, 0.0)],
                        boundary=["ELEM 0 TO 20 ADMI 1.0 1 1.0 2", "ELEM 21 TO 30 IMPE 2.0 -1 0.5 -1",
                                  "ELEM 31 TO 40 VELO 0.2 -1 0.0 -1"],
                        curves=[(1, [(500.0, 0.1), (3000.0, 0.4), (8000.0, 0.2)]),
                                (2, [(500.0, 0.0), (5000.0, -0.3)])])

    def mutate(root, wd):
        el = os.path.join(root, "ObjectMeshes", "Reference", "Elements.txt")
        lines = pathlib.Path(el).read_text().strip("\n").split("\n")
        out = [lines[0]]
        for i, ln in enumerate(lines[1:]):
            tok = ln.split()
            ids = [t for t in tok[1:5] if int(t) >= 0]
            grp = str(i % 3)
            out.append(" ".join([tok[0]] + ids + ["0", "0", grp]))
        pathlib.Path(el).write_text("\n".join(out) + "\n")
        inp = os.path.join(wd, "NC.inp")
        s = pathlib.Path(inp).read_text().replace("2 %d" % (len(elems) + len(pts) * 2 - 4), "4 %d" % (len(elems) + len(pts) * 2 - 4), 1)
        pathlib.Path(inp).write_text(s)
    return _write(p, "quads_groups", mutate)


def case_crlf():
    """Windows line endings: the reference stops at the NODES keyword."""
    v, f = meshes.icosphere(20, 0.1)
    pts = meshes.random_sphere_points(6, 0.4, 4)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[1000.0], point_sources=[(0.3, 0.0, 0.0, 0.1, 0.0)],
                        boundary=["ELEM 0 TO 19 VELO 0.0 -1 0.0 -1"])

    def mutate(root, wd):
        inp = os.path.join(wd, "NC.inp")
        s = pathlib.Path(inp).read_text().replace("\n", "\r\n")
        pathlib.Path(inp).write_text(s, newline="")
    return _write(p, "crlf", mutate)


CASES = {"plain": case_plain, "dialect": case_dialect, "quads_groups": case_quads_groups, "crlf": case_crlf,
         "dup_node": case_dup_node}


def reference_result(wd):
    tmp = tempfile.mkdtemp()
    r = refdump.run(wd, dump_dir=tmp, args=("-nitermax", "1"))
    res = {"returncode": r.returncode, "stdout_tail": r.stdout.strip().split("\n")[-1]}
    tb = os.path.join(tmp, "tables.bin")
    if os.path.exists(tb):
        d = refdump.read_dump(tb)
        res["digests"] = table_digests(d)
    shutil.rmtree(tmp)
    est = subprocess.run([refdump.REF_NUMCALC, "-estimate_ram"], cwd=wd, capture_output=True, text=True)
    if est.returncode == 0 and os.path.exists(os.path.join(wd, "Memory.txt")):
        res["memory_txt"] = pathlib.Path(os.path.join(wd, "Memory.txt")).read_text()
    for junk in ("NC.out", "Memory.txt", "NCuntil1.out"):
        if os.path.exists(os.path.join(wd, junk)):
            os.remove(os.path.join(wd, junk))
    shutil.rmtree(os.path.join(wd, "be.out"), ignore_errors=True)
    return res


if __name__ == "__main__":
    if not refdump.available():
        refdump.build()
    os.makedirs(OUT, exist_ok=True)
    allres = {}
    for name, fn in CASES.items():
        wd = fn()
        allres[name] = reference_result(wd)
        print(name, allres[name].get("returncode"), allres[name].get("stdout_tail"))
    with open(os.path.join(OUT, "digests.json"), "w") as fh:
        json.dump(allres, fh, indent=1, sort_keys=True)
