"""Batched solves (bem_solve_batch): several (mesh, frequency) instances of
different sizes and precisions assembled, iterated and projected together.

Each instance's result must be the one it gets alone (bem_solve_frequency).
The engine's per-instance arithmetic does not depend on the other instances,
so the stated tolerance is 0 (bit-identical); the test also bounds the mixed
instances against the FP64 oracle at the metric's 1e-4.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes
from oracle import oracle_py as op

pytestmark = pytest.mark.gpu

C, RHO = 343.0, 1.21


def _freq(n, f_hz, src):
    k = 2 * np.pi * f_hz / C
    amp = 0.1 / (1j * RHO * 2 * np.pi * f_hz)
    return capi.Frequency(k, n, point_sources=src, point_amps=[amp])


def _cases():
    out = []
    for n_tri, f_hz, src in [(320, 1500.0, [1.0, 0.0, 0.0]), (1280, 3000.0, [0.0, 0.9, 0.2]),
                             (720, 800.0, [0.3, 0.3, 1.1]), (2000, 6000.0, [-1.0, 0.2, 0.1])]:
        v, f = meshes.icosphere(n_tri, 0.1)
        out.append((v, f, f_hz, src))
    return out


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_batch_equals_alone(prec):
    pts = meshes.random_sphere_points(200, 1.2, 7)
    cases = _cases()
    meshes_ = [capi.Mesh(v, f) for v, f, _, _ in cases]
    alone = []
    for m, (v, f, fh, src) in zip(meshes_, cases):
        s = capi.Solver(m, precision=prec, tol=1e-9)
        x, pot, grad = s.solve_frequency(_freq(len(f), fh, src), pts)
        alone.append((x, pot, grad, s.info.as_dict()))
        s.close()
    solvers = [capi.Solver(m, precision=prec, tol=1e-9) for m in meshes_]
    freqs = [_freq(len(f), fh, src) for (v, f, fh, src) in cases]
    res = capi.solve_batch(solvers, freqs, [pts] * len(cases))
    for (x0, p0, g0, i0), (x1, p1, g1, i1, st) in zip(alone, res):
        assert st == capi.BEM_OK
        assert i1["iterations"] == i0["iterations"]
        assert np.array_equal(x1, x0)
        assert np.array_equal(p1, p0)
        assert np.array_equal(g1, g0)


def test_batch_mixed_vs_oracle():
    """Mixed instances of a batch against the FP64 oracle's dense solve."""
    pts = meshes.random_sphere_points(100, 1.2, 11)
    cases = _cases()[:2]
    ms = [capi.Mesh(v, f) for v, f, _, _ in cases]
    solvers = [capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9) for m in ms]
    freqs = [_freq(len(f), fh, src) for (v, f, fh, src) in cases]
    res = capi.solve_batch(solvers, freqs, [pts] * len(cases))
    for (v, f, fh, src), (x, pot, grad, info, st) in zip(cases, res):
        om = op.OracleMesh(v, f)
        k = 2 * np.pi * fh / C
        amp = 0.1 / (1j * RHO * 2 * np.pi * fh)
        of = op.OracleFreq(k, point_sources=src, ps_amp=[amp])
        A, b = op.assemble(om, of)
        xr = op.solve_dense(A, b)
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-4


def test_batch_same_mesh_many_frequencies():
    """Eight frequencies on one mesh (eight solvers sharing the mesh)."""
    v, f = meshes.icosphere(1280, 0.1)
    m = capi.Mesh(v, f)
    pts = meshes.random_sphere_points(50, 1.2, 3)
    fhz = [200.0, 700.0, 1300.0, 2100.0, 3400.0, 5000.0, 6500.0, 8000.0]
    solvers = [capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9) for _ in fhz]
    freqs = [_freq(len(f), fh, [1.0, 0.0, 0.0]) for fh in fhz]
    res = capi.solve_batch(solvers, freqs, [pts] * len(fhz))
    for fh, (x, pot, grad, info, st) in zip(fhz, res):
        s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
        x0, p0, _ = s.solve_frequency(_freq(len(f), fh, [1.0, 0.0, 0.0]), pts)
        assert st == capi.BEM_OK
        assert np.array_equal(x, x0) and np.array_equal(pot, p0)
        assert info["rel_residual"] <= 1e-9


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_large_batch_equals_alone(prec):
    """A batch of 20 instances of one mesh (the engine's launch tables and
    plans hold them all at once): the same bits as alone."""
    pts = meshes.random_sphere_points(64, 1.2, 9)
    v, f = meshes.icosphere(320, 0.1)
    m = capi.Mesh(v, f)
    freqs = [_freq(len(f), 300.0 + 350.0 * i, [1.0, 0.05 * i, 0.0]) for i in range(20)]
    s = capi.Solver(m, precision=prec, tol=1e-9)
    alone = [s.solve_frequency(fr, pts)[:2] for fr in freqs[:3]]
    s.close()
    solvers = [capi.Solver(m, precision=prec, tol=1e-9) for _ in freqs]
    res = capi.solve_batch(solvers, freqs, [pts] * len(freqs))
    for (x0, p0), r in zip(alone, res):
        assert np.array_equal(r[0], x0) and np.array_equal(r[1], p0)
    for sv in solvers:
        sv.close()
    m.close()
