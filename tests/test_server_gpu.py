"""Served requests (bem_server_*): continuous batching with HBM admission.

Each request's result must equal the one it gets alone (bem_solve_frequency):
the per-request arithmetic does not depend on the other requests iterating
with it, so the stated tolerance is 0 (bit-identical).  The requests arrive
in two waves while earlier ones are iterating; the budget and the slot limit
are small enough that admission has to wait for memory and slots to free up.
"""
import time

import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes

pytestmark = pytest.mark.gpu

C, RHO = 343.0, 1.21


def _freq(n, f_hz, src):
    k = 2 * np.pi * f_hz / C
    amp = 0.1 / (1j * RHO * 2 * np.pi * f_hz)
    return capi.Frequency(k, n, point_sources=src, point_amps=[amp])


CASES = [(320, 1500.0, [1.0, 0.0, 0.0]), (1280, 3000.0, [0.0, 0.9, 0.2]), (720, 800.0, [0.3, 0.3, 1.1]),
         (2000, 6000.0, [-1.0, 0.2, 0.1]), (1280, 9000.0, [0.2, -1.0, 0.3]), (500, 2500.0, [0.0, 0.0, -1.2]),
         (1620, 4000.0, [0.7, 0.7, 0.0]), (320, 12000.0, [-0.5, 0.9, 0.0])]


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_served_equals_alone(prec):
    pts = meshes.random_sphere_points(150, 1.2, 5)
    ms = {}
    for n_tri, _, _ in CASES:
        if n_tri not in ms:
            v, f = meshes.icosphere(n_tri, 0.1)
            ms[n_tri] = capi.Mesh(v, f)
    # alone
    alone = []
    for n_tri, fh, src in CASES:
        s = capi.Solver(ms[n_tri], precision=prec, tol=1e-9)
        alone.append(s.solve_frequency(_freq(n_tri, fh, src), pts))
        s.close()
    # served: budget for about three of the larger requests, four slots
    biggest = max(capi.footprint_bytes(n, prec) for n, _, _ in CASES)
    srv = capi.Server(precision=prec, hbm_budget=3.2 * biggest, max_active=4, tol=1e-9)
    tickets = [srv.submit(ms[n], _freq(n, fh, src), pts) for n, fh, src in CASES[:5]]
    time.sleep(0.01)   # the second wave arrives while the first iterates
    tickets += [srv.submit(ms[n], _freq(n, fh, src), pts) for n, fh, src in CASES[5:]]
    infos = []
    for t, (x0, p0, g0) in zip(tickets, alone):
        r = srv.wait(t, timeout=120.0)
        assert r is not None, "request did not finish within 120 s"
        x, pot, grad, info, st = r
        assert st == capi.BEM_OK
        assert np.array_equal(x, x0)
        assert np.array_equal(pot, p0)
        assert np.array_equal(grad, g0)
        assert info["rel_residual"] <= 1e-9
        infos.append(info)
    srv.close()
    assert all(i["latency_ms"] >= i["queued_ms"] for i in infos)


def test_server_rejects_oversized_and_reports_pending():
    v, f = meshes.icosphere(1280, 0.1)
    m = capi.Mesh(v, f)
    fp = capi.footprint_bytes(1280, capi.PREC_MIXED)
    srv = capi.Server(precision=capi.PREC_MIXED, hbm_budget=0.5 * fp + 1e6)
    with pytest.raises(capi.BemError) as e:
        srv.submit(m, _freq(1280, 1000.0, [1.0, 0.0, 0.0]), np.zeros((4, 3)) + 1.2)
    assert e.value.status == capi.BEM_ERR_OUT_OF_HBM
    srv.close()
    srv = capi.Server(precision=capi.PREC_MIXED, hbm_budget=2.5 * fp)
    t = srv.submit(m, _freq(1280, 1000.0, [1.0, 0.0, 0.0]), meshes.random_sphere_points(10, 1.2, 1))
    r = srv.wait(t, timeout=0.0)
    if r is None:   # still running: wait for it
        r = srv.wait(t, timeout=120.0)
    assert r is not None
    assert r[4] == capi.BEM_OK
    srv.close()
