"""CUDA library vs the reference (golden fixtures) and vs the FP64 oracle.

Tolerances: the FP64 path assembles and projects in FP64 and solves with
GMRES to a relative residual of 1e-12, so entries agree with the reference to
1e-12 of the matrix scale and the solution with the reference's dense solve
to 1e-9.  The mixed path (FP32 assembly with exact subdivision decisions,
refined solve) must meet the metric's bar: boundary pressure within 1e-4
relative L2 of the FP64 solution.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi
from oracle import oracle_py as op
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def _gpu(case, prec, tol=1e-12):
    m = capi.Mesh(case.nodes, case.elems)
    return m, capi.Solver(m, precision=prec, tol=tol)


def _freq(case, s):
    st = case.step(s)
    f = capi.Frequency(st["k"], case.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                       admittance=st["admittance"], point_sources=st["point_sources"],
                       point_amps=st["point_amps"], plane_dirs=st["plane_dirs"],
                       plane_amps=st["plane_amps"])
    return st, f


@pytest.mark.parametrize("name", ["sphere80", "quad96_soft_plane"])
def test_fp64_full_matrix(name):
    c = gc.load(name)
    m, s = _gpu(c, capi.PREC_FP64)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        s.assemble(f)
        A, b = s.system()
        Aref = c["s%d_A" % k]
        assert np.abs(A - Aref).max() <= 1e-12 * np.abs(Aref).max()
        assert gc.rel_err(b, c["s%d_b" % k]) < 1e-12


@pytest.mark.parametrize("name", ["sphere320_adm_velo", "sphere1280_1k", "pspw2412_4k"])
def test_fp64_sampled_matrix(name):
    c = gc.load(name)
    m, s = _gpu(c, capi.PREC_FP64)
    st, f = _freq(c, 1)
    s.assemble(f)
    A, b = s.system()
    scale = np.abs(c["s1_A_rows"]).max()
    assert np.abs(A[c["s1_rows"]] - c["s1_A_rows"]).max() <= 1e-12 * scale
    ij = c["s1_ent_ij"]
    assert np.abs(A[ij[:, 0], ij[:, 1]] - c["s1_ent_val"]).max() <= 1e-12 * scale
    assert gc.rel_err(b, c["s1_b"]) < 1e-12


@pytest.mark.parametrize("name", gc.CASES)
def test_fp64_solve_and_fields(name):
    c = gc.load(name)
    m, s = _gpu(c, capi.PREC_FP64)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        x, pot, grad = s.solve_frequency(f, c.pts)
        assert s.info.rel_residual < 1e-12
        assert gc.rel_err(x, c["s%d_x_dense" % k]) < 1e-9
        # field projection from this x: the FP64 oracle on the same x
        om = op.OracleMesh(c.nodes, c.elems, bc_type=st["bc_type"], bc_val=st["bc_value"],
                           adm=st["admittance"])
        of = op.OracleFreq(st["k"], st["point_sources"], st["point_amps"], st["plane_dirs"], st["plane_amps"])
        phi, vel = op.boundary_fields(om, x)
        pot_o, grad_o = op.project(om, of, phi, vel, c.pts, nthreads=8)
        assert gc.rel_err(pot, pot_o) < 1e-12
        assert gc.rel_err(grad, grad_o) < 1e-12
        # end to end against the reference's be.out (its CGS stops at 1e-9)
        assert gc.rel_err(1j * st["rpfact"] * pot, c["s%d_pEvalGrid" % k]) < 1e-6


@pytest.mark.parametrize("name", gc.CASES)
def test_mixed_precision_meets_1e4(name):
    c = gc.load(name)
    m, s = _gpu(c, capi.PREC_MIXED, tol=1e-10)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        x, pot, grad = s.solve_frequency(f, c.pts)
        xr = c["s%d_x_dense" % k]
        phi_ref = np.where(st["bc_type"] == 1, st["bc_value"][:, 0], xr)
        phi = np.where(st["bc_type"] == 1, st["bc_value"][:, 0], x)
        # boundary pressure p = i rho w phi; for pressure-prescribed elements
        # the unknown is the velocity, compared separately
        if np.any(st["bc_type"] != 1):
            assert gc.rel_err(phi, phi_ref) < 1e-4
        assert gc.rel_err(x, xr) < 1e-4
        assert gc.rel_err(pot, c["s%d_pEvalGrid" % k] / (1j * st["rpfact"])) < 1e-4


def test_subdivision_limit_reported():
    """An evaluation point on the surface: NumCalc stops with its subdivision
    error; the library returns BEM_ERR_SUBDIVISION instead of faulting."""
    c = gc.load("sphere80")
    m, s = _gpu(c, capi.PREC_FP64)
    st, f = _freq(c, 1)
    s.assemble(f)
    s.solve()
    on_surface = c.nodes[:1] * 1.0
    with pytest.raises(capi.BemError) as e:
        s.project(on_surface)
    assert e.value.status == capi.BEM_ERR_SUBDIVISION
