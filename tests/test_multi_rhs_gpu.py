"""Several right-hand sides on one matrix (bem_solve_multi).

Right-hand side r must give what bem_solve_frequency gives for its sources
alone.  FP64: bit for bit (each right-hand side iterates as its own system
with the same products).  Mixed: the right-hand sides share each read of A
in one product (full-row accumulation instead of 1024-column partials), so
the rounding differs; both solutions meet the 1e-9 residual on the same
complex64 matrix and agree to 1e-7.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_multi_rhs_equals_single(prec):
    v, f = meshes.perturbed_ellipsoid(9, 77)   # 1620 triangles
    m = capi.Mesh(v, f)
    pts = meshes.random_sphere_points(80, 1.2, 4)
    srcs = [meshes.surface_point_with_normal(v, f, 100 + r) for r in range(5)]
    fh = 7000.0
    freqs = [workloads.frequency(capi, len(f), fh, s) for s in srcs]
    s = capi.Solver(m, precision=prec, tol=1e-9, n_rhs=8)
    xs, pots, grads, infos = s.solve_multi(freqs, pts)
    one = capi.Solver(m, precision=prec, tol=1e-9)
    for r in range(len(srcs)):
        x0, p0, g0 = one.solve_frequency(freqs[r], pts)
        assert infos[r]["rel_residual"] <= 1e-9
        if prec == capi.PREC_FP64:
            assert infos[r]["iterations"] == one.info.iterations
            assert np.array_equal(xs[r], x0)
            assert np.array_equal(pots[r], p0)
            assert np.array_equal(grads[r], g0)
        else:
            # the shared products differ from the single solve's (TF32 operands
            # on the tcgen05 path): at most one more refinement cycle's steps
            assert -2 <= infos[r]["iterations"] - one.info.iterations <= 8
            assert np.linalg.norm(xs[r] - x0) <= 1e-7 * np.linalg.norm(x0)
            assert np.linalg.norm(pots[r] - p0) <= 1e-7 * np.linalg.norm(p0)
    # the right-hand sides really differ
    assert np.linalg.norm(xs[0] - xs[1]) > 1e-3 * np.linalg.norm(xs[0])


def test_multi_rhs_footprint_and_limit():
    fp1 = capi.load().bem_footprint_multi(4000, capi.PREC_MIXED, 0, 1)
    fp8 = capi.load().bem_footprint_multi(4000, capi.PREC_MIXED, 0, 8)
    # the complex64 matrix is shared (a single right-hand side also keeps its
    # fp16 Krylov copy, several share the complex64 product)
    assert fp8 > 4000 * 4000 * 8 and fp8 < 2 * fp1
    v, f = meshes.icosphere(320, 0.1)
    m = capi.Mesh(v, f)
    s = capi.Solver(m, precision=capi.PREC_MIXED, n_rhs=2)
    fr = [workloads.frequency(capi, len(f), 1000.0, [1.0, 0, 0])] * 3
    with pytest.raises(capi.BemError):
        s.solve_multi(fr, np.zeros((0, 3)))


def test_multi_rhs_projection_shares_kernel_evaluations():
    """Mixed precision projects all right-hand sides in one pass that
    evaluates each far flat-triangle kernel once (k_project_pts_multi); pairs
    with velocity terms (a vibrating patch in one right-hand side) and
    subdivided near pairs (points 1 mm off the surface) take the per-right-
    hand-side path.  Each field equals the single-right-hand-side solve's to
    the solutions' own agreement (1e-7 relative, 1e-6 for near points)."""
    v, f = meshes.perturbed_ellipsoid(6, 78)   # 720 triangles
    n = len(f)
    m = capi.Mesh(v, f)
    far = meshes.random_sphere_points(48, 1.2, 5)
    near = np.array([meshes.surface_point_with_normal(v, f, 300 + q) for q in range(6)])
    pts = np.vstack([far, near])
    k = 2 * np.pi * 5000.0 / workloads.C0
    amp = 0.1 / (1j * workloads.RHO * 2 * np.pi * 5000.0)
    srcs = [meshes.surface_point_with_normal(v, f, 200 + r) * 1.5 for r in range(3)]
    bcv = np.zeros((n, 4), np.complex128)
    bcv[:12, :3] = 1e-4 + 2e-5j
    freqs = [capi.Frequency(k, n, point_sources=srcs[0], point_amps=[amp]),
             capi.Frequency(k, n, bc_value=bcv, point_sources=srcs[1], point_amps=[amp]),
             capi.Frequency(k, n, plane_dirs=[0.0, 0.6, 0.8], plane_amps=[amp])]
    s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-10, n_rhs=3)
    xs, pots, grads, infos = s.solve_multi(freqs, pts)
    one = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-10)
    for r in range(3):
        x0, p0, g0 = one.solve_frequency(freqs[r], pts)
        assert np.linalg.norm(xs[r] - x0) <= 1e-7 * np.linalg.norm(x0)
        nf = len(far)
        assert np.linalg.norm(pots[r][:nf] - p0[:nf]) <= 1e-7 * np.linalg.norm(p0[:nf])
        assert np.linalg.norm(grads[r][:nf] - g0[:nf]) <= 1e-7 * np.linalg.norm(g0[:nf])
        assert np.linalg.norm(pots[r][nf:] - p0[nf:]) <= 1e-6 * np.linalg.norm(p0[nf:])
        assert np.linalg.norm(grads[r][nf:] - g0[nf:]) <= 1e-6 * np.linalg.norm(g0[nf:])
    s.close()
    one.close()
    m.close()


def test_grouped_product_tensor_core_paths_agree(monkeypatch):
    """The right-hand sides' shared Krylov product on the 5th-generation
    tensor cores (tcgen05, TF32 operands, k_mv_grp_umma; the default) and on
    the warp-level ones (mma.sync 3xTF32, k_mv_grp_tc;
    BEM_GB300_GROUP_PRODUCT=mma)
    reach the same solutions: both refine to a 1e-9 residual of the same
    complex64 system with FP32-accurate residual products."""
    v, f = meshes.perturbed_ellipsoid(14, 79)   # 3920 triangles: several 128-row strips, a ragged last one
    n = len(f)
    m = capi.Mesh(v, f)
    pts = meshes.random_sphere_points(40, 1.2, 6)
    srcs = [meshes.surface_point_with_normal(v, f, 400 + r) for r in range(8)]
    freqs = [workloads.frequency(capi, n, 9000.0, s) for s in srcs]
    out = {}
    for mode in ("mma", "tcgen05"):
        monkeypatch.setenv("BEM_GB300_GROUP_PRODUCT", mode)
        s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, n_rhs=8)
        xs, pots, grads, infos = s.solve_multi(freqs, pts)
        assert all(i["rel_residual"] <= 1e-9 for i in infos)
        out[mode] = (xs, pots, [i["iterations"] for i in infos])
        s.close()
    for r in range(8):
        xa, xb = out["mma"][0][r], out["tcgen05"][0][r]
        assert np.linalg.norm(xa - xb) <= 1e-7 * np.linalg.norm(xa), r
        pa, pb = out["mma"][1][r], out["tcgen05"][1][r]
        assert np.linalg.norm(pa - pb) <= 1e-7 * np.linalg.norm(pa), r
    # TF32 inner products: a few more Krylov steps at most
    assert max(out["tcgen05"][2]) <= 2 * max(out["mma"][2]) + 10
    m.close()
