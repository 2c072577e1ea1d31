"""The configurations beyond the head-like bench as GPU parity cases.

- Rigid sphere, 1280 triangles, 1 kHz, point source at 1 m, GMRES tolerance
  1e-8, 1000 seeded points at 1.2 m: FP64 and mixed against the analytic
  series (the discretisation floor of this mesh is ~3e-4; bound 1e-3) and
  mixed against FP64 (1e-4).
- Batched uneven instances (perturbed ellipsoids): a reduced set (16
  instances, 500-4000 triangles) checked mixed vs FP64 at 1e-4 and batch vs
  solo bit for bit; the full set (64 instances, 2k-30k triangles, about 85 GB
  of complex64 matrices in one batch) checked for convergence.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads
from oracle import analytic

pytestmark = pytest.mark.gpu


def test_sphere_1280_vs_analytic():
    v, f = meshes.icosphere(1280, 0.1)
    pts = meshes.random_sphere_points(1000, 1.2, 20261203)
    m = capi.Mesh(v, f)
    k = 2 * np.pi * 1000.0 / 343.0
    F = workloads.frequency(capi, len(f), 1000.0, [1.0, 0.0, 0.0])
    # analytic total pressure for source strength Q = 1 (p = i rho w phi)
    pa = analytic.point_source_sphere(pts, [1.0, 0.0, 0.0], 0.1, k, Q=1.0)
    res = {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        s = capi.Solver(m, precision=prec, tol=1e-8)
        x, pot, _ = s.solve_frequency(F, pts)
        assert s.info.rel_residual <= 1e-8
        p = 1j * 1.21 * 2 * np.pi * 1000.0 * pot
        err = np.linalg.norm(p / 0.1 - pa) / np.linalg.norm(pa)
        assert err < 1e-3, (prec, err)
        res[prec] = x
    assert np.linalg.norm(res[capi.PREC_MIXED] - res[capi.PREC_FP64]) / np.linalg.norm(res[capi.PREC_FP64]) < 1e-4


def _solvers(insts, prec):
    ms = [capi.Mesh(i["nodes"], i["elems"]) for i in insts]
    ss = [capi.Solver(m, precision=prec, tol=1e-9, max_iter=3000) for m in ms]
    fs = [workloads.frequency(capi, len(i["elems"]), i["freq"], i["source"]) for i in insts]
    return ms, ss, fs


def test_batched_uneven_reduced():
    insts = workloads.batched_instances(count=16, n_min=500, n_max=4000)
    pts = meshes.random_sphere_points(64, 1.2, 9)
    ms, smx, fs = _solvers(insts, capi.PREC_MIXED)
    rmx = capi.solve_batch(smx, fs, [pts] * len(insts))
    s64 = [capi.Solver(m, precision=capi.PREC_FP64, tol=1e-9, max_iter=3000) for m in ms]
    r64 = capi.solve_batch(s64, fs, [pts] * len(insts))
    for a, b in zip(rmx, r64):
        assert a[4] == capi.BEM_OK and b[4] == capi.BEM_OK
        assert np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0]) < 1e-4
    # solo solves of three instances: bit-identical to their batched results
    for q in (0, 7, 15):
        s = capi.Solver(ms[q], precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000)
        x, pot, grad = s.solve_frequency(fs[q], pts)
        assert np.array_equal(x, rmx[q][0]) and np.array_equal(pot, rmx[q][1])


def test_batched_uneven_full_size():
    insts = workloads.batched_instances(count=64)
    ms, ss, fs = _solvers(insts, capi.PREC_MIXED)
    res = capi.solve_batch(ss, fs, None)
    for r in res:
        assert r[4] == capi.BEM_OK
        assert r[3]["rel_residual"] <= 1e-9
