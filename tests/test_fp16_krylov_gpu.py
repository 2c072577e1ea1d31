"""The fp16 Krylov copy of the mixed-precision solver (bem_solver_params.
complex64_krylov = 0, the default): Krylov products read A in row-scaled
fp16, the refinement residuals the complex64 matrix.  The converged solution
must meet the same residual target with the complex64 system as the
complex64-only solver, so the two agree to about the target times the
condition number (bar: 1e-6 relative), and both stay within the metric's
1e-4 of the reference's FP64 solution.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sphere1280_1k", "sphere320_adm_velo", "quad96_soft_plane"])
def test_fp16_krylov_matches_complex64_krylov(name):
    c = gc.load(name)
    st = c.step(1)
    f = capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                       admittance=st["admittance"], point_sources=st["point_sources"],
                       point_amps=st["point_amps"], plane_dirs=st["plane_dirs"], plane_amps=st["plane_amps"])
    m = capi.Mesh(c.nodes, c.elems)
    res = {}
    for c64 in (False, True):
        s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=c64)
        x, pot, grad = s.solve_frequency(f, c.pts)
        assert s.info.rel_residual <= 1e-9
        assert gc.rel_err(x, c["s1_x_dense"]) < 1e-4
        res[c64] = (x, pot, s.info.as_dict())
    assert gc.rel_err(res[False][0], res[True][0]) < 1e-6
    assert gc.rel_err(res[False][1], res[True][1]) < 1e-6


def test_fp16_krylov_on_the_head_mesh():
    """5120-triangle head-like mesh, source 1 mm off a bump, 0.5-16 kHz: the
    fp16-copy solver converges to the target at every frequency and agrees
    with the complex64-only solver."""
    v, f, info = meshes.head_like(16)
    m = capi.Mesh(v, f)
    for fh in (500.0, 4000.0, 16000.0):
        fr = workloads.frequency(capi, len(f), fh, info["source"])
        out = []
        for c64 in (False, True):
            s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=c64)
            s.assemble(fr)
            s.solve()
            assert s.info.rel_residual <= 1e-9
            out.append(s.solution())
        assert gc.rel_err(out[0], out[1]) < 1e-6


def test_footprint_counts_the_fp16_copy():
    n = 20480
    mixed = capi.footprint_bytes(n, capi.PREC_MIXED)
    lda = (n + 31) // 32 * 32
    # the fp16 copy adds 4 bytes per matrix entry and a row scale per row
    assert mixed > n * lda * 12
