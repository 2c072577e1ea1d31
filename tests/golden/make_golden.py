"""Generate the golden fixtures under tests/golden/ from the reference NumCalc.

Runs oracle/_ref/NumCalc_dump (the reference's unmodified sources, built by
oracle/Makefile) on small projects and stores, per case, the inputs (mesh,
evaluation points, frequency data), the reference's assembled matrix (full
or sampled rows/entries), right-hand side, CGS solution, a dense FP64 solve of
the same system, and the full-precision be.out results.  Needs the reference
sources; the committed .npz files are what the tests read.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mesh2hrtf_gb300 import meshes, project  # noqa: E402
from oracle import refdump  # noqa: E402

REF_FIXTURES = "/root/reference/tests/resources/test_numcalc"


def cube_sphere(n, radius):
    """Quadrilateral sphere: cube faces split n x n, projected (outward)."""
    pts, quads, idx = [], [], {}

    def vid(p):
        key = tuple(np.round(p, 12))
        if key not in idx:
            idx[key] = len(pts)
            pts.append(p)
        return idx[key]

    g = np.linspace(-1, 1, n + 1)
    for ax in range(3):
        for sgn in (-1, 1):
            for a in range(n):
                for b in range(n):
                    cs = []
                    for (u, v) in ((g[a], g[b]), (g[a + 1], g[b]), (g[a + 1], g[b + 1]), (g[a], g[b + 1])):
                        p = np.zeros(3)
                        p[ax] = sgn
                        p[(ax + 1) % 3] = u
                        p[(ax + 2) % 3] = v
                        cs.append(vid(p))
                    quads.append(cs)
    v = np.array(pts)
    v = v / np.linalg.norm(v, axis=1)[:, None] * radius
    q = np.array(quads)
    # NumCalc quad normal: dx/ds x dx/dt at the centre, outward wanted
    for e in range(len(q)):
        P = v[q[e]]
        dxs = 0.25 * (P[0] - P[1] - P[2] + P[3])
        dxt = 0.25 * (P[0] + P[1] - P[2] - P[3])
        if np.dot(np.cross(dxs, dxt), P.mean(axis=0)) < 0:
            q[e] = q[e][::-1]
    return v, q


def run_case(name, proj: project.Project, rows=None, n_entries=0, seed=0, full=False):
    tmp = tempfile.mkdtemp()
    proj.root = os.path.join(tmp, "p")
    wd = project.write_project(proj)
    dump = os.path.join(tmp, "dump")
    r = refdump.run(wd, dump_dir=dump)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr)
    out = {}
    tab = refdump.read_dump(os.path.join(dump, "tables.bin"))
    nsteps = len(proj.freqs)
    out["nodes"] = proj.nodes
    out["elems"] = proj.elems
    out["eval_points"] = proj.eval_points
    out["freqs"] = np.asarray(proj.freqs, float)
    out["point_sources"] = np.asarray(proj.point_sources, float).reshape(-1, 5)
    out["plane_waves"] = np.asarray(proj.plane_waves, float).reshape(-1, 5)
    out["speed_density"] = np.array([proj.speed_of_sound, proj.density])
    out["elem_center"] = tab["elem_center"].reshape(-1, 3)[: len(proj.elems)]
    out["elem_normal"] = tab["elem_normals"].reshape(-1, 15)[: len(proj.elems), :3]
    out["elem_area"] = tab["elem_area"][: len(proj.elems)]
    out["elem_ibval"] = tab["elem_ibval"][: len(proj.elems)]
    rng = np.random.default_rng(seed)
    for s in range(1, nsteps + 1):
        d = refdump.read_dump(os.path.join(dump, "step%d.bin" % s))
        n = int(d["n_method_precond"][0])
        A = d["A"].reshape(n, n)
        out["s%d_freq_k_rpfact" % s] = d["freq_k_rpfact"]
        out["s%d_zposoc" % s] = d["zposoc"]
        out["s%d_zinwav" % s] = d["zinwav"]
        out["s%d_zbval0" % s] = d["zbval0"].reshape(-1, 4)[:n]
        out["s%d_zbval1" % s] = d["zbval1"][:n]
        out["s%d_b" % s] = d["b"]
        out["s%d_x_cgs" % s] = d["x"]
        out["s%d_x_dense" % s] = np.linalg.solve(A, d["b"])
        if full:
            out["s%d_A" % s] = A
        else:
            rr = np.asarray(sorted(set(rows or [])), int)
            out["s%d_rows" % s] = rr
            out["s%d_A_rows" % s] = A[rr]
            ii = rng.integers(0, n, n_entries)
            jj = rng.integers(0, n, n_entries)
            out["s%d_ent_ij" % s] = np.stack([ii, jj], axis=1)
            out["s%d_ent_val" % s] = A[ii, jj]
        beo = os.path.join(wd, "be.out", "be.%d" % s)
        for f in ("pBoundary", "vBoundary", "pEvalGrid", "vEvalGrid"):
            if os.path.exists(os.path.join(beo, f)):
                ids, vals = project.read_result(os.path.join(beo, f))
                out["s%d_%s" % (s, f)] = vals
                out["s%d_%s_ids" % (s, f)] = ids
    shutil.rmtree(tmp)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, {k: v.shape for k, v in out.items() if hasattr(v, "shape")})


def case_sphere80():
    v, f = meshes.icosphere(80, 0.1)
    sh = [meshes.random_sphere_points(24, 0.3, 5), meshes.random_sphere_points(8, 0.104, 6)]
    pts = np.vstack(sh)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.shells_triangles(sh),
                        freqs=[1000.0, 5000.0], point_sources=[(0.5, 0.1, 0.0, 1.0, 0.0)],
                        boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"])
    run_case("sphere80", p, full=True)


def case_quad_soft():
    v, q = cube_sphere(4, 0.1)
    sh = [meshes.random_sphere_points(24, 0.25, 7), meshes.random_sphere_points(6, 0.106, 8)]
    pts = np.vstack(sh)
    p = project.Project(root="", nodes=v, elems=q, eval_points=pts, eval_elems=meshes.shells_triangles(sh),
                        freqs=[2000.0], plane_waves=[(0.0, -1.0, 0.0, 1.0, 0.0)],
                        boundary=["ELEM 0 TO %d PRES 0.0 -1 0.0 -1" % (len(q) - 1)])
    run_case("quad96_soft_plane", p, full=True)


def case_admittance():
    v, f = meshes.icosphere(320, 0.1)
    pts = meshes.random_sphere_points(40, 0.5, 9)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[3000.0],
                        boundary=["ELEM 0 TO 319 ADMI 0.5 -1 0.2 -1", "ELEM 10 TO 12 VELO 0.1 -1 0.0 -1"])
    run_case("sphere320_adm_velo", p, rows=[0, 10, 11, 12, 160, 319], n_entries=600, seed=3)


def case_sphere1280():
    v, f = meshes.icosphere(1280, 0.1)
    pts = meshes.random_sphere_points(1000, 1.2, 20261203)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[1000.0], point_sources=[(1.0, 0.0, 0.0, 1.0, 0.0)],
                        boundary=["ELEM 0 TO 1279 VELO 0.0 -1 0.0 -1"])
    run_case("sphere1280_1k", p, rows=[0, 1, 640, 1279], n_entries=2000, seed=1)


def _load_ref_mesh(folder):
    nodes = np.loadtxt(os.path.join(folder, "Nodes.txt"), skiprows=1)
    el = np.loadtxt(os.path.join(folder, "Elements.txt"), skiprows=1, dtype=np.int64)
    idmap = {int(i): k for k, i in enumerate(nodes[:, 0])}
    con = np.vectorize(idmap.get)(el[:, 1:4])
    return nodes[:, 1:], con


def case_pspw():
    """The reference's own TBEM fixture: 2412-element sphere (a = 0.0875 m),
    point source at 0.2 m, 4 kHz, 7560 evaluation points from 0.09 m."""
    base = os.path.join(REF_FIXTURES, "project_folder_pspw")
    v, f = _load_ref_mesh(os.path.join(base, "ObjectMeshes", "Reference"))
    pts, ptri = _load_ref_mesh(os.path.join(base, "EvaluationGrids", "HorPlane"))
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=ptri, freqs=[4000.0],
                        point_sources=[(0.2, 0.0, 0.0, 0.1, 0.0)], speed_of_sound=343.0, density=1.1839,
                        boundary=["ELEM 0 TO 2411 VELO 0.0 -1 0.0 -1"])
    run_case("pspw2412_4k", p, rows=[0, 1205, 2411], n_entries=1000, seed=2)


CASES = {"sphere80": case_sphere80, "quad": case_quad_soft, "adm": case_admittance,
         "sphere1280": case_sphere1280, "pspw": case_pspw}

if __name__ == "__main__":
    if not refdump.available():
        refdump.build()
    for c in (sys.argv[1:] or list(CASES)):
        CASES[c]()
