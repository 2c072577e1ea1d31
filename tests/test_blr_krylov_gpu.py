"""The block low-rank Krylov copy of the mixed-precision solver
(bem_solver_params.complex64_krylov = 2, capi.KRYLOV_BLR): the off-diagonal
256 x 256 blocks of A compressed by adaptive cross approximation (bem_blr.cu),
read by the Krylov products (k_mv_blr); the refinement residuals read the
complex64 matrix.  The converged solution meets the same residual target
with the complex64 system as the complex64-only solver, so the two agree to
about the target times the condition number (bar: 1e-6 relative), and both
stay within the metric's 1e-4 of the reference's FP64 solution.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["pspw2412_4k", "sphere1280_1k", "sphere320_adm_velo", "quad96_soft_plane"])
def test_blr_krylov_matches_complex64_krylov(name):
    """Golden cases of the reference: 2412, 1280, 320 and 96 unknowns (ten,
    five, two and one block rows, the last ones ragged; plane and point
    sources, admittance and velocity boundary conditions, quadrilaterals)."""
    c = gc.load(name)
    st = c.step(1)
    f = capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                       admittance=st["admittance"], point_sources=st["point_sources"],
                       point_amps=st["point_amps"], plane_dirs=st["plane_dirs"], plane_amps=st["plane_amps"])
    m = capi.Mesh(c.nodes, c.elems)
    res = {}
    for mode in (True, capi.KRYLOV_BLR):
        s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=mode)
        x, pot, grad = s.solve_frequency(f, c.pts)
        assert s.info.rel_residual <= 1e-9
        assert gc.rel_err(x, c["s1_x_dense"]) < 1e-4
        res[mode] = (x, pot)
        if mode == capi.KRYLOV_BLR:
            info = s.krylov_copy_info()
            nb = (c.n + 255) // 256
            assert info["blocks_per_row"] == nb and info["dense_blocks"] >= nb
        s.close()
    m.close()
    assert gc.rel_err(res[True][0], res[capi.KRYLOV_BLR][0]) < 1e-6
    assert gc.rel_err(res[True][1], res[capi.KRYLOV_BLR][1]) < 1e-6


def test_blr_krylov_on_the_head_mesh():
    """5120-triangle head-like mesh (20 block rows), source 1 mm off a bump,
    0.5-16 kHz: converges to the target at every frequency, agrees with the
    complex64-only solver, compresses (below the fp16 copy's 4 bytes per
    entry up to 4 kHz) and is deterministic run to run."""
    v, f, info = meshes.head_like(16)
    m = capi.Mesh(v, f)
    for fh in (500.0, 4000.0, 16000.0):
        fr = workloads.frequency(capi, len(f), fh, info["source"])
        out, its = [], []
        for mode in (True, capi.KRYLOV_BLR, capi.KRYLOV_BLR):
            s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=mode)
            s.assemble(fr)
            s.solve()
            assert s.info.rel_residual <= 1e-9
            out.append(s.solution())
            its.append(s.info.iterations)
            if mode == capi.KRYLOV_BLR:
                ci = s.krylov_copy_info()
            s.close()
        assert gc.rel_err(out[0], out[1]) < 1e-6
        assert np.array_equal(out[1], out[2])
        assert ci["blocks_per_row"] == 20 and 0 < ci["mean_rank"] <= 48
        if fh <= 4000.0:   # the copy pays: under the fp16 copy's 4 bytes per entry
            assert ci["bytes_per_product"] < 4.0 * len(f) ** 2
        print("head5120 %.0f Hz: iterations complex64 %d, block low-rank %d; copy %s" % (fh, its[0], its[1], ci))
    m.close()


def test_blr_krylov_in_a_batch_equals_alone():
    """A batch that mixes a block low-rank solver with an fp16-copy one: each
    result equals the same solver's result alone, bit for bit."""
    v, f = meshes.perturbed_ellipsoid(12, 91)   # 2880 triangles: ragged block rows and chunks
    n = len(f)
    m = capi.Mesh(v, f)
    pts = meshes.random_sphere_points(32, 1.2, 3)
    F = [workloads.frequency(capi, n, fr, [0.3, 0.1, 0.05]) for fr in (3000.0, 7000.0)]
    modes = (capi.KRYLOV_BLR, False)
    alone = []
    for mode, fr in zip(modes, F):
        s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=mode)
        alone.append(s.solve_frequency(fr, pts))
        s.close()
    ss = [capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, complex64_krylov=mode) for mode in modes]
    both = capi.solve_batch(ss, F, [pts, pts])
    for a, b in zip(alone, both):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for s in ss:
        s.close()
    m.close()


def test_copy_info_needs_the_copy():
    v, f = meshes.icosphere(80, 0.1)
    m = capi.Mesh(v, f)
    s = capi.Solver(m, precision=capi.PREC_MIXED)
    with pytest.raises(capi.BemError):
        s.krylov_copy_info()
    s.close()
    m.close()


def test_krylov_copy_mode_out_of_range_is_rejected():
    v, f = meshes.icosphere(80, 0.1)
    m = capi.Mesh(v, f)
    p = capi.SolverParams(capi.PREC_MIXED, 0, 0, 0.0, 0.0, 0, 0, 3)
    h = capi.C.c_void_p()
    assert capi.load().bem_solver_create(m.handle, capi.C.byref(p), capi.C.byref(h)) == capi.BEM_ERR_INVALID
    m.close()
