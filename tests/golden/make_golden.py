"""Generate the golden fixtures under tests/golden/ from the reference NumCalc.

Runs oracle/_ref/NumCalc_dump (the reference's unmodified sources, built by
oracle/Makefile) on small projects and stores, per case, the inputs (mesh,
evaluation points, frequency data), the reference's assembled matrix (full
or sampled rows/entries), right-hand side, CGS solution, a dense FP64 solve of
the same system, and the full-precision be.out results.  Needs the reference
sources (MESH2HRTF_REFERENCE = root of a Mesh2HRTF checkout); the committed
.npz files are what the tests read.

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



def ref_fixtures() -> str:
    """The reference's test_numcalc resources (needs MESH2HRTF_REFERENCE)."""
    root = refdump.reference_root()
    if not root:
        raise SystemExit("set %s to the root of a Mesh2HRTF checkout" % refdump.REFERENCE_ENV)
    return os.path.join(root, "tests", "resources", "test_numcalc")


def cube_sphere(n, radius):
    return meshes.cube_sphere(n, radius)


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
    if proj.nsym:
        out["sym_planes"] = np.asarray(proj.sym_planes, np.int32)   # NC.inp codes
        out["sym_coords"] = np.asarray(proj.sym_coords, float)
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
    base = os.path.join(ref_fixtures(), "project_folder_pspw")
    v, f = _load_ref_mesh(os.path.join(base, "ObjectMeshes", "Reference"))
    pts, ptri = _load_ref_mesh(os.path.join(base, "EvaluationGrids", "HorPlane"))
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=ptri, freqs=[4000.0],
                        point_sources=[(0.2, 0.0, 0.0, 0.1, 0.0)], speed_of_sound=343.0, density=1.1839,
                        boundary=["ELEM 0 TO 2411 VELO 0.0 -1 0.0 -1"])
    run_case("pspw2412_4k", p, rows=[0, 1205, 2411], n_entries=1000, seed=2)


def case_sym1():
    """Half sphere (x >= 0) of 216 triangles, one symmetric plane x = 0,
    rigid, point source off the plane; two frequencies."""
    v, f = meshes.sphere_sector(6, 0.1, (0,), triangles=True)
    sh = [meshes.random_sphere_points(24, 0.3, 31), meshes.random_sphere_points(8, 0.104, 32)]
    pts = np.vstack(sh)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.shells_triangles(sh),
                        freqs=[1500.0, 4000.0], point_sources=[(0.25, 0.05, 0.02, 1.0, 0.0)],
                        boundary=["ELEM 0 TO %d VELO 0.0 -1 0.0 -1" % (len(f) - 1)],
                        nsym=1, sym_planes=(1, 0, 0))
    run_case("sym1_half216", p, rows=[0, 5, 60, 107, 108, 150, 215], n_entries=1500, seed=4)


def case_sym2():
    """Quarter sphere (y, z >= 0) of 54 quads: antisymmetric plane y = 0,
    symmetric plane z = 0; admittance everywhere, a vibrating patch, a
    sound-soft patch, a plane wave and a point source."""
    v, q = meshes.sphere_sector(6, 0.1, (1, 2))
    pts = meshes.random_sphere_points(30, 0.35, 33)
    d = np.array([0.3, -0.5, 0.81])
    d /= np.linalg.norm(d)
    p = project.Project(root="", nodes=v, elems=q, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[2500.0], point_sources=[(0.05, 0.2, 0.1, 1.0, 0.5)],
                        plane_waves=[(d[0], d[1], d[2], 0.7, -0.2)],
                        boundary=["ELEM 0 TO 53 ADMI 0.3 -1 0.1 -1", "ELEM 4 TO 7 VELO 0.2 -1 -0.1 -1",
                                  "ELEM 30 TO 32 PRES 0.05 -1 0.02 -1"],
                        nsym=2, sym_planes=(0, 2, 1))
    run_case("sym2_quarter54", p, full=True)


def case_sym3():
    """Octant of 54 triangles moved off the origin: three planes through
    (0.02, -0.01, 0.03) - symmetric x, antisymmetric y, hard reflecting z
    (NC.inp code 3, the reference treats it as symmetric); rigid with a
    point source and a plane wave."""
    c = (0.02, -0.01, 0.03)
    v, f = meshes.sphere_sector(6, 0.1, (0, 1, 2), center=c, triangles=True)
    pts = meshes.random_sphere_points(24, 0.3, 34) + np.asarray(c)
    d = np.array([-0.4, 0.2, -0.9])
    d /= np.linalg.norm(d)
    p = project.Project(root="", nodes=v, elems=f, eval_points=pts, eval_elems=meshes.grid_triangles(pts),
                        freqs=[3000.0], point_sources=[(0.12, 0.09, 0.15, 1.0, 0.0)],
                        plane_waves=[(d[0], d[1], d[2], 0.5, 0.0)],
                        boundary=["ELEM 0 TO %d VELO 0.0 -1 0.0 -1" % (len(f) - 1)],
                        nsym=3, sym_planes=(1, 2, 3), sym_coords=c)
    run_case("sym3_octant54", p, full=True)


CASES = {"sphere80": case_sphere80, "quad": case_quad_soft, "adm": case_admittance,
         "sphere1280": case_sphere1280, "pspw": case_pspw, "sym1": case_sym1, "sym2": case_sym2,
         "sym3": case_sym3}

if __name__ == "__main__":
    if not refdump.available():
        refdump.build()
    for c in (sys.argv[1:] or list(CASES)):
        CASES[c]()
