"""The dense direct solver on the GPU (bem_solve_direct): NumCalc's
Tfactor_usy / Tfbelim (NC_TypeDefinition.h:543-594), LU without pivoting,
which the reference runs for ISOLVER 4 and after a failed CGS.

Bars: FP64 within 1e-9 of the reference's own dense solve of the same
system (golden fixtures; LU without pivoting in FP64 agrees to ~1e-12);
mixed precision (complex64 factors, FP64 substitutions) within the metric's
1e-4; the drop-in with ISOLVER 4 writes the reference's be.out within the
7-digit print bar (2e-6 FP64, 1e-5 mixed).
"""
import os
import pathlib
import subprocess

import numpy as np
import pytest

from mesh2hrtf_gb300 import build, capi, meshes, project
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def _freq(c, s):
    st = c.step(s)
    return st, capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                              admittance=st["admittance"], point_sources=st["point_sources"],
                              point_amps=st["point_amps"], plane_dirs=st["plane_dirs"],
                              plane_amps=st["plane_amps"])


@pytest.mark.parametrize("name", ["sphere80", "quad96_soft_plane", "sphere320_adm_velo", "pspw2412_4k"])
@pytest.mark.parametrize("prec,tol", [(capi.PREC_FP64, 1e-9), (capi.PREC_MIXED, 1e-4)])
def test_direct_matches_reference_dense_solve(name, prec, tol):
    c = gc.load(name)
    m = capi.Mesh(c.nodes, c.elems)
    s = capi.Solver(m, precision=prec)
    for k in range(1, len(c.freqs) + 1):
        st, f = _freq(c, k)
        s.assemble(f)
        info = s.solve_direct()
        assert info["iterations"] == 0 and info["solve_ms"] > 0
        x = s.solution()
        assert gc.rel_err(x, c["s%d_x_dense" % k]) < tol, gc.rel_err(x, c["s%d_x_dense" % k])
        pot, _ = s.project(c.pts)
        assert gc.rel_err(1j * st["rpfact"] * pot, c["s%d_pEvalGrid" % k]) < max(tol, 1e-6)
    s.close()
    m.close()


def test_factored_matrix_needs_a_new_assembly():
    c = gc.load("sphere320_adm_velo")
    m = capi.Mesh(c.nodes, c.elems)
    s = capi.Solver(m, precision=capi.PREC_FP64, tol=1e-12)
    st, f = _freq(c, 1)
    s.assemble(f)
    s.solve_direct()
    x_direct = s.solution()
    for call in (s.solve, s.solve_direct):
        with pytest.raises(capi.BemError) as e:
            call()
        assert e.value.status == capi.BEM_ERR_INVALID and "assemble" in str(e.value)
    s.assemble(f)
    s.solve()
    assert gc.rel_err(s.solution(), x_direct) < 1e-10
    s.close()
    m.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 2e-6), ("mixed", 1e-5)])
def test_numcalc_isolver4(tmp_path, precision, tol):
    """NC.inp with ISOLVER 4 (Main Parameters I token 8): the drop-in runs the
    direct solver and prints no CGS line, as the reference does."""
    numcalc = build.build_numcalc()
    c = gc.load("sphere320_adm_velo")
    p = project.Project(root=str(tmp_path / "p"), nodes=c.nodes, elems=c.elems, eval_points=c.pts,
                        eval_elems=meshes.grid_triangles(c.pts), freqs=list(c.freqs), solver=4,
                        boundary=["ELEM 0 TO 319 ADMI 0.5 -1 0.2 -1", "ELEM 10 TO 12 VELO 0.1 -1 0.0 -1"])
    wd = project.write_project(p)
    env = dict(os.environ, NUMCALC_GB300_PRECISION=precision)
    r = subprocess.run([numcalc], cwd=wd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    out = pathlib.Path(os.path.join(wd, "NC.out")).read_text()
    assert "methodSolver_  = 4: Gaussean elimination (direct) solver" in out
    assert "CGS solver:" not in out and "End time:" in out
    for s in range(1, len(c.freqs) + 1):
        for fname in ("pBoundary", "pEvalGrid"):
            ids, vals = project.read_result(os.path.join(wd, "be.out", "be.%d" % s, fname))
            assert gc.rel_err(vals, c["s%d_%s" % (s, fname)]) < tol
