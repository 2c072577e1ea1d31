"""The preconditioner's window correction (bem_solver_params.no_precond = 0,
the default): M = X (2 I - A_w X) with X the block-Jacobi inverse of the
128-unknown diagonal blocks and A_w the 1024-unknown diagonal windows of A.
It changes how GMRES gets there, not where: every preconditioner mode meets
the same residual target on the same system, so the solutions agree to about
the target times the condition number (bar: 1e-6 relative), and the
corrected preconditioner needs fewer iterations than block-Jacobi alone.
The modes include NumCalc's own scaling preconditioner (no_precond = 3,
NC_ComputeScalingVector, NC_CommonFunctions.cpp:1322-1351) and none.

Covers both matrix paths of the correction (complex128 for FP64, complex64
and its fp16 copy for mixed precision), partial windows (n not a multiple of
1024, n below 1024) and several right-hand sides on one matrix.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

MODES = (True, "block-jacobi", "scaling", False)


def _freq(c, step=1):
    st = c.step(step)
    return capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                          admittance=st["admittance"], point_sources=st["point_sources"],
                          point_amps=st["point_amps"], plane_dirs=st["plane_dirs"], plane_amps=st["plane_amps"])


@pytest.mark.parametrize("name", ["quad96_soft_plane", "sphere1280_1k", "pspw2412_4k"])
@pytest.mark.parametrize("prec,c64", [(capi.PREC_FP64, False), (capi.PREC_MIXED, False), (capi.PREC_MIXED, True)])
def test_modes_reach_the_same_solution(name, prec, c64):
    c = gc.load(name)
    f = _freq(c)
    m = capi.Mesh(c.nodes, c.elems)
    out = {}
    for mode in MODES:
        s = capi.Solver(m, precision=prec, tol=1e-9, precond=mode, complex64_krylov=c64)
        x, pot, _ = s.solve_frequency(f, c.pts, with_grad=False)
        assert s.info.rel_residual <= 1e-9
        assert gc.rel_err(x, c["s1_x_dense"]) < (1e-8 if prec == capi.PREC_FP64 else 1e-4)
        out[mode] = (x, pot, s.info.iterations)
        s.close()
    for mode in MODES[1:]:
        assert gc.rel_err(out[True][0], out[mode][0]) < 1e-6
        assert gc.rel_err(out[True][1], out[mode][1]) < 1e-6


def test_window_correction_saves_iterations_on_the_head_mesh():
    """5120-triangle head-like mesh (5 windows), source 1 mm off a bump:
    fewer Krylov iterations than block-Jacobi alone at every frequency, in
    both precisions, and the same solution."""
    v, f, info = meshes.head_like(16)
    m = capi.Mesh(v, f)
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        for fh in (500.0, 4000.0, 16000.0):
            fr = workloads.frequency(capi, len(f), fh, info["source"])
            res = {}
            for mode in (True, "block-jacobi"):
                s = capi.Solver(m, precision=prec, tol=1e-9, precond=mode)
                s.assemble(fr)
                s.solve()
                assert s.info.rel_residual <= 1e-9
                res[mode] = (s.solution(), s.info.iterations)
                s.close()
            assert res[True][1] < res["block-jacobi"][1], (prec, fh, res[True][1], res["block-jacobi"][1])
            assert gc.rel_err(res[True][0], res["block-jacobi"][0]) < 1e-6


def test_window_correction_with_several_right_hand_sides():
    """Right-hand sides sharing one complex64 matrix (grouped products, no fp16
    copy) agree with single solves of the same preconditioner."""
    v, f, info = meshes.head_like(12)
    n = len(f)
    srcs = [meshes.surface_point_with_normal(v, f, 7 + r) for r in range(3)]
    m = capi.Mesh(v, f)
    pts = meshes.fibonacci_sphere(64, 1.2)
    freqs = [workloads.frequency(capi, n, 6000.0, sp) for sp in srcs]
    s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, n_rhs=3)
    xs, pots, _, infos = s.solve_multi(freqs, pts, with_grad=False)
    assert all(i["rel_residual"] <= 1e-9 for i in infos)
    s.close()
    for r in range(3):
        s1 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, precond="block-jacobi")
        x1, p1, _ = s1.solve_frequency(freqs[r], pts, with_grad=False)
        s1.close()
        assert gc.rel_err(xs[r], x1) < 1e-6
        assert gc.rel_err(pots[r], p1) < 1e-6


def test_invalid_preconditioner_mode_is_rejected():
    c = gc.load("sphere80")
    m = capi.Mesh(c.nodes, c.elems)
    with pytest.raises(ValueError):
        capi.Solver(m, precond="ilu")
    p = capi.SolverParams(capi.PREC_MIXED, 0, 0, 0.0, 0.0, 4, 0, 0)
    h = capi.C.c_void_p()
    rc = capi.load().bem_solver_create(m.handle, capi.C.byref(p), capi.C.byref(h))
    assert rc == capi.BEM_ERR_INVALID
