"""The FP64 C restatement (oracle/bem_oracle.c) against the reference's own
outputs stored in tests/golden (CPU only).  This pins the oracle before it is
used to check the CUDA library."""
import numpy as np
import pytest

from oracle import analytic, oracle_py as op
from tests import golden_cases as gc


def _mesh(case):
    s = case.step(1)
    return op.OracleMesh(case.nodes, case.elems, bc_type=s["bc_type"], bc_val=s["bc_value"],
                         adm=s["admittance"], sym=case.sym, sym_coord=case.sym_coords)


def _freq(s):
    return op.OracleFreq(s["k"], s["point_sources"], s["point_amps"], s["plane_dirs"], s["plane_amps"])


@pytest.mark.parametrize("name", gc.CASES + gc.SYM_CASES)
def test_geometry_matches_reference(name):
    c = gc.load(name)
    m = _mesh(c)
    np.testing.assert_allclose(m.centers, c["elem_center"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(m.normals[:, :3], c["elem_normal"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(m.areas, c["elem_area"], rtol=1e-14)


@pytest.mark.parametrize("name", ["sphere80", "quad96_soft_plane"])
def test_full_matrix_matches_reference(name):
    c = gc.load(name)
    m = _mesh(c)
    for s in range(1, len(c.freqs) + 1):
        st = c.step(s)
        A, b = op.assemble(m, _freq(st), nthreads=4)
        Aref = c["s%d_A" % s]
        assert np.abs(A - Aref).max() <= 1e-13 * np.abs(Aref).max()
        assert gc.rel_err(b, c["s%d_b" % s]) < 1e-13


@pytest.mark.parametrize("name", ["sphere320_adm_velo", "sphere1280_1k", "pspw2412_4k"])
def test_sampled_matrix_matches_reference(name):
    c = gc.load(name)
    m = _mesh(c)
    st = c.step(1)
    rows = c["s1_rows"]
    scale = np.abs(c["s1_A_rows"]).max()
    for k, r in enumerate(rows):
        A, _ = op.assemble(m, _freq(st), rows=(int(r), int(r) + 1), nthreads=4)
        assert np.abs(A[0] - c["s1_A_rows"][k]).max() <= 1e-13 * scale
    ij = c["s1_ent_ij"][:64]
    for (i, j), v in zip(ij, c["s1_ent_val"][:64]):
        A, _ = op.assemble(m, _freq(st), rows=(int(i), int(i) + 1), nthreads=4)
        assert abs(A[0, j] - v) <= 1e-13 * scale


@pytest.mark.parametrize("name", ["sphere80", "quad96_soft_plane", "sphere320_adm_velo"])
def test_projection_matches_reference(name):
    """Reference be.out (17 digits) from its own CGS solution."""
    c = gc.load(name)
    m = _mesh(c)
    for s in range(1, len(c.freqs) + 1):
        st = c.step(s)
        phi, vel = op.boundary_fields(m, c["s%d_x_cgs" % s])
        pot, grad = op.project(m, _freq(st), phi, vel, c.pts, nthreads=4)
        p = 1j * st["rpfact"] * pot
        assert gc.rel_err(p, c["s%d_pEvalGrid" % s]) < 1e-12
        assert gc.rel_err(grad, c["s%d_vEvalGrid" % s]) < 1e-12
        pb = 1j * st["rpfact"] * phi
        assert gc.rel_err(pb, c["s%d_pBoundary" % s]) < 1e-13
        assert gc.rel_err(vel[:, 0], c["s%d_vBoundary" % s]) < 1e-13 or np.abs(c["s%d_vBoundary" % s]).max() == 0


def test_dense_solve_matches_reference_cgs():
    c = gc.load("sphere80")
    m = _mesh(c)
    st = c.step(1)
    A, b = op.assemble(m, _freq(st))
    x = op.solve_dense(A, b)
    assert gc.rel_err(x, c["s1_x_dense"]) < 1e-12
    assert gc.rel_err(x, c["s1_x_cgs"]) < 1e-8


@pytest.mark.parametrize("name", ["sphere80", "sphere1280_1k", "pspw2412_4k"])
def test_cgs_ilu_reproduces_reference_cgs(name):
    """The restatement of NumCalc's solver (threshold ILU of scanning degree 0,
    CGS to 1e-9, NC_CommonFunctions.cpp:1066-1721) on the oracle's matrix
    gives the reference's own CGS solution bit for bit, at any thread count."""
    c = gc.load(name)
    m = _mesh(c)
    st = c.step(1)
    A, b = op.assemble(m, _freq(st), nthreads=8)
    x1, it, err, direct, _ = op.solve_cgs(A, b, precond=0, scan=0, nthreads=1)
    x8, it8, _, _, _ = op.solve_cgs(A, b, precond=0, scan=0, nthreads=8)
    assert not direct and err < 1e-9 and it == it8
    assert np.array_equal(x1, x8)
    assert np.array_equal(x1, c["s1_x_cgs"])


def test_analytic_series_vs_reference_bem():
    """Discretisation error of the reference BEM on the 1280-triangle sphere
    (a = 0.1 m, 1 kHz, point source at 1 m) against the FP64 series."""
    c = gc.load("sphere1280_1k")
    st = c.step(1)
    pa = analytic.point_source_sphere(c.pts, [1.0, 0, 0], 0.1, st["k"], Q=1.0)
    assert gc.rel_err(c["s1_pEvalGrid"], pa) < 1e-3


@pytest.mark.parametrize("name", gc.SYM_CASES)
def test_symmetry_planes_match_reference(name):
    """Images of the elements, sources and waves in one to three symmetry
    planes (symmetric, antisymmetric, reflecting; planes off the origin):
    matrix, right-hand side and evaluation-grid fields against the
    reference run on the same project."""
    c = gc.load(name)
    m = _mesh(c)
    assert any(c.sym)
    for s in range(1, len(c.freqs) + 1):
        st = c.step(s)
        A, b = op.assemble(m, _freq(st), nthreads=4)
        if c.has("s%d_A" % s):
            Aref = c["s%d_A" % s]
            assert np.abs(A - Aref).max() <= 1e-13 * np.abs(Aref).max()
        else:
            rr, Ar = c["s%d_rows" % s], c["s%d_A_rows" % s]
            assert np.abs(A[rr] - Ar).max() <= 1e-13 * np.abs(Ar).max()
            ij = c["s%d_ent_ij" % s]
            assert np.abs(A[ij[:, 0], ij[:, 1]] - c["s%d_ent_val" % s]).max() <= 1e-13 * np.abs(Ar).max()
        assert gc.rel_err(b, c["s%d_b" % s]) < 1e-13
        assert gc.rel_err(op.solve_dense(A, b), c["s%d_x_dense" % s]) < 1e-12
        phi, vel = op.boundary_fields(m, c["s%d_x_cgs" % s])
        pot, grad = op.project(m, _freq(st), phi, vel, c.pts, nthreads=4)
        assert gc.rel_err(1j * st["rpfact"] * pot, c["s%d_pEvalGrid" % s]) < 1e-12
        assert gc.rel_err(grad, c["s%d_vEvalGrid" % s]) < 1e-12
