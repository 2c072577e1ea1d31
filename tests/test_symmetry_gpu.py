"""Symmetry planes on the GPU path (NumCalc's SYMMETRY block): every element
is integrated with its 1, 2, 4 or 8 images in the planes, incident waves
with theirs (NC_ReflectElement / NC_ReflectPointVector,
NC_3dFunctions.cpp:181-452; NC_EquationSystem.cpp:277-300,1731-1812;
NC_PostProcessing.cpp:776-975).

Against the reference run on the same projects (tests/golden/sym*.npz, made
by tests/golden/make_golden.py) with the tolerances of the plain-mesh parity
tests: FP64 entries within 1e-12 of the matrix scale, FP64 solution within
1e-9 of the reference's dense solve, mixed precision within the metric's
1e-4.  At larger sizes, where no reference output exists, a half sphere
with its plane must give the full sphere's solution (the images of the
half are the other half's elements, integrated with the same quadrature).
"""
import os
import subprocess

import numpy as np
import pytest

from mesh2hrtf_gb300 import build, capi, meshes, project
from oracle import oracle_py as op
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def _mesh(c):
    return capi.Mesh(c.nodes, c.elems, sym_planes=c.sym, sym_coords=c.sym_coords)


def _freq(c, s):
    st = c.step(s)
    f = capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                       admittance=st["admittance"], point_sources=st["point_sources"],
                       point_amps=st["point_amps"], plane_dirs=st["plane_dirs"],
                       plane_amps=st["plane_amps"])
    return st, f


@pytest.mark.parametrize("name", gc.SYM_CASES)
def test_fp64_matrix_and_rhs(name):
    c = gc.load(name)
    m = _mesh(c)
    s = capi.Solver(m, precision=capi.PREC_FP64, tol=1e-12)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        s.assemble(f)
        A, b = s.system()
        if c.has("s%d_A" % k):
            Aref = c["s%d_A" % k]
            assert np.abs(A - Aref).max() <= 1e-12 * np.abs(Aref).max()
        else:
            rr, Ar = c["s%d_rows" % k], c["s%d_A_rows" % k]
            assert np.abs(A[rr] - Ar).max() <= 1e-12 * np.abs(Ar).max()
            ij = c["s%d_ent_ij" % k]
            assert np.abs(A[ij[:, 0], ij[:, 1]] - c["s%d_ent_val" % k]).max() <= 1e-12 * np.abs(Ar).max()
        assert gc.rel_err(b, c["s%d_b" % k]) < 1e-12


@pytest.mark.parametrize("name", gc.SYM_CASES)
def test_fp64_solve_and_fields(name):
    c = gc.load(name)
    m = _mesh(c)
    s = capi.Solver(m, precision=capi.PREC_FP64, tol=1e-12)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        x, pot, grad = s.solve_frequency(f, c.pts)
        assert s.info.rel_residual < 1e-12
        assert gc.rel_err(x, c["s%d_x_dense" % k]) < 1e-9
        om = op.OracleMesh(c.nodes, c.elems, bc_type=st["bc_type"], bc_val=st["bc_value"],
                           adm=st["admittance"], sym=c.sym, sym_coord=c.sym_coords)
        of = op.OracleFreq(st["k"], st["point_sources"], st["point_amps"], st["plane_dirs"], st["plane_amps"])
        phi, vel = op.boundary_fields(om, x)
        pot_o, grad_o = op.project(om, of, phi, vel, c.pts, nthreads=8)
        assert gc.rel_err(pot, pot_o) < 1e-12
        assert gc.rel_err(grad, grad_o) < 1e-12
        assert gc.rel_err(1j * st["rpfact"] * pot, c["s%d_pEvalGrid" % k]) < 1e-6


@pytest.mark.parametrize("name", gc.SYM_CASES)
def test_mixed_precision_meets_1e4(name):
    c = gc.load(name)
    m = _mesh(c)
    s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-10)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        x, pot, grad = s.solve_frequency(f, c.pts)
        assert gc.rel_err(x, c["s%d_x_dense" % k]) < 1e-4
        assert gc.rel_err(pot, c["s%d_pEvalGrid" % k] / (1j * st["rpfact"])) < 1e-4


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_batch_with_and_without_planes_equals_alone(prec):
    """A batch mixing meshes with and without images: each result is the
    one it gets alone, bit for bit."""
    c = gc.load("sym2_quarter54")
    v, f = meshes.icosphere(320, 0.1)
    plain = capi.Mesh(v, f)
    sym = _mesh(c)
    _, fs = _freq(c, 1)
    fp = capi.Frequency(2 * np.pi * 2000 / 343.0, len(f), point_sources=[0.3, 0.1, 0.0], point_amps=[1.0])
    pts = meshes.random_sphere_points(40, 0.4, 5)
    alone = []
    for m, fr in ((sym, fs), (plain, fp)):
        s = capi.Solver(m, precision=prec, tol=1e-9)
        alone.append(s.solve_frequency(fr, pts))
    solvers = [capi.Solver(sym, precision=prec, tol=1e-9), capi.Solver(plain, precision=prec, tol=1e-9)]
    res = capi.solve_batch(solvers, [fs, fp], [pts, pts])
    for (x0, p0, g0), (x1, p1, g1, info, st) in zip(alone, res):
        assert st == capi.BEM_OK
        assert np.array_equal(x1, x0) and np.array_equal(p1, p0) and np.array_equal(g1, g0)


@pytest.mark.parametrize("code,sign", [(1, 1.0), (2, -1.0)])
@pytest.mark.parametrize("prec,tol", [(capi.PREC_FP64, 1e-9), (capi.PREC_MIXED, 1e-4)])
def test_half_sphere_equals_full_sphere(code, sign, prec, tol):
    """1536-quad sphere against its 768-quad half with the plane x = 0: a
    symmetric (antisymmetric) source pair on the full sphere gives, on the
    half, the solution of the half with a symmetric (antisymmetric) plane."""
    vf, qf = meshes.cube_sphere(16, 0.1)
    vh, qh = meshes.sphere_sector(16, 0.1, (0,))
    k = 2 * np.pi * 3000 / 343.0
    src = np.array([0.25, 0.05, 0.02])
    img = src * np.array([-1.0, 1.0, 1.0])
    pts = meshes.random_sphere_points(64, 0.4, 8)
    full = capi.Solver(capi.Mesh(vf, qf), precision=prec, tol=1e-11)
    xf, pf, gf = full.solve_frequency(
        capi.Frequency(k, len(qf), point_sources=np.vstack([src, img]), point_amps=[1.0, sign]), pts)
    half = capi.Solver(capi.Mesh(vh, qh, sym_planes=(code, 0, 0)), precision=prec, tol=1e-11)
    xh, ph, gh = half.solve_frequency(capi.Frequency(k, len(qh), point_sources=src, point_amps=[1.0]), pts)
    # element correspondence by centre
    cf = vf[qf].mean(axis=1)
    ch = vh[qh].mean(axis=1)
    key = {tuple(np.round(p, 9)): i for i, p in enumerate(cf)}
    idx = np.array([key[tuple(np.round(p, 9))] for p in ch])
    assert gc.rel_err(xh, xf[idx]) < tol
    assert gc.rel_err(ph, pf) < tol
    assert gc.rel_err(gh, gf) < tol


@pytest.fixture(scope="module")
def numcalc():
    build.build_all()
    return build.NUMCALC_BIN


@pytest.mark.parametrize("precision,tol", [("fp64", 2e-6), ("mixed", 1e-5)])
def test_numcalc_drop_in_with_planes(numcalc, tmp_path, precision, tol):
    """The drop-in on a project with two planes (antisymmetric y, symmetric
    z), admittance, vibrating and sound-soft patches, a plane wave and a
    point source: be.out against the reference's."""
    c = gc.load("sym2_quarter54")
    ps, pw = c["point_sources"], c["plane_waves"]
    p = project.Project(root=str(tmp_path / "p"), nodes=c.nodes, elems=c.elems, eval_points=c.pts,
                        eval_elems=meshes.grid_triangles(c.pts), freqs=list(c.freqs),
                        point_sources=[tuple(ps[0])], plane_waves=[tuple(pw[0])],
                        boundary=["ELEM 0 TO 53 ADMI 0.3 -1 0.1 -1", "ELEM 4 TO 7 VELO 0.2 -1 -0.1 -1",
                                  "ELEM 30 TO 32 PRES 0.05 -1 0.02 -1"],
                        nsym=2, sym_planes=c.sym, sym_coords=c.sym_coords)
    wd = project.write_project(p)
    env = dict(os.environ, NUMCALC_GB300_PRECISION=precision)
    r = subprocess.run([numcalc], cwd=wd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    for f in ("pBoundary", "vBoundary", "pEvalGrid", "vEvalGrid"):
        ids, vals = project.read_result(os.path.join(wd, "be.out", "be.1", f))
        assert np.array_equal(ids, c["s1_%s_ids" % f])
        assert gc.rel_err(vals, c["s1_%s" % f]) < tol, (f, gc.rel_err(vals, c["s1_%s" % f]))
