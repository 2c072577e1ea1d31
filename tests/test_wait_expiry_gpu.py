"""A bounded device wait that runs out, and the context afterwards.

The Krylov product k_mv_tma streams A through shared memory with bulk copies
and mbarrier waits, each bounded (about 2 s by default).  The environment
variable BEM_GB300_TEST_WAIT_CYCLES lowers the bound of the consumers' and
the producer's waits (not of the drain that lets in-flight copies land
before a block exits) to a few hundred cycles, polled without suspension:
the consumers' first wait of every launch then gives up before the first
stage can arrive from HBM.  Nothing faults and nothing hangs: the kernel
sets the table's error word, drains its copies and returns; the solve
returns BEM_ERR_DEVICE_TIMEOUT, and a fresh solver afterwards solves the
same system to the same bits as before.
"""
import os

import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes

pytestmark = pytest.mark.gpu


def _case():
    v, f = meshes.icosphere(1280, 0.1)
    k = 2 * np.pi * 3000.0 / 343.0
    fr = capi.Frequency(k, len(f), point_sources=[0.4, 0.1, 0.0], point_amps=[1e-3 + 0j])
    return v, f, fr


def test_product_wait_runs_out_and_context_survives(monkeypatch):
    v, f, fr = _case()
    m = capi.Mesh(v, f)
    s0 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
    s0.assemble(fr)
    s0.solve()
    x_ref = s0.solution()
    s0.close()

    monkeypatch.setenv("BEM_GB300_TEST_WAIT_CYCLES", "200")
    s1 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
    s1.assemble(fr)
    with pytest.raises(capi.BemError) as e:
        s1.solve()
    assert e.value.status == capi.BEM_ERR_DEVICE_TIMEOUT
    assert "bounded device wait" in str(e.value)
    s1.close()

    monkeypatch.delenv("BEM_GB300_TEST_WAIT_CYCLES")
    s2 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
    s2.assemble(fr)
    info = s2.solve()
    assert info["rel_residual"] <= 1e-9
    assert np.array_equal(s2.solution(), x_ref)
    s2.close()
    m.close()
    assert "BEM_GB300_TEST_WAIT_CYCLES" not in os.environ


def test_grouped_tensor_core_product_wait_runs_out(monkeypatch):
    """The same for the tcgen05 product of several right-hand sides sharing
    one matrix (k_mv_grp_umma).  BEM_GB300_TEST_WAIT_KINDS=1 shortens only
    the Krylov products' waits, so the first iteration body's residual
    products finish and the tensor-core product of the next body gives up:
    its producer drains the copies in flight, its MMA warp waits for the MMAs
    it issued, and the block releases its tensor memory before it exits.  A
    later grouped solve allocates tensor memory again and reproduces the
    earlier solutions bit for bit."""
    v, f, fr = _case()
    n = len(f)
    m = capi.Mesh(v, f)
    pts = meshes.random_sphere_points(8, 1.2, 2)
    k = fr.desc.wave_number
    freqs = [capi.Frequency(k, n, point_sources=[0.4, 0.05 * r, 0.0], point_amps=[1e-3 + 0j]) for r in range(4)]
    monkeypatch.delenv("BEM_GB300_GROUP_PRODUCT", raising=False)
    s0 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, n_rhs=4)
    xs0, _, _, _ = s0.solve_multi(freqs, pts)
    s0.close()

    monkeypatch.setenv("BEM_GB300_TEST_WAIT_CYCLES", "200")
    monkeypatch.setenv("BEM_GB300_TEST_WAIT_KINDS", "1")
    s1 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, n_rhs=4)
    with pytest.raises(capi.BemError) as e:
        s1.solve_multi(freqs, pts)
    assert e.value.status == capi.BEM_ERR_DEVICE_TIMEOUT
    s1.close()

    monkeypatch.delenv("BEM_GB300_TEST_WAIT_CYCLES")
    monkeypatch.delenv("BEM_GB300_TEST_WAIT_KINDS")
    s2 = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9, n_rhs=4)
    xs2, _, _, infos = s2.solve_multi(freqs, pts)
    assert all(i["rel_residual"] <= 1e-9 for i in infos)
    for a, b in zip(xs0, xs2):
        assert np.array_equal(a, b)
    s2.close()
    m.close()
