"""The benchmarked configuration itself, pinned against the FP64 oracle.

Workload: the head-like scatterer of the benchmark (20480 triangles graded
toward bump 1, source 1 mm off bump 1, 1730-point grid at 1.2 m) at 100 Hz,
10 kHz and 20 kHz (3 elements per wavelength at the coarse end of the
grading).  The oracle (the FP64 C restatement of NC_ComputeEntriesForTBEM,
NC_EquationSystem.cpp:210-302, with NumCalc's subdivision and quadrature)
assembles 32 rows: the 8 collocation points nearest to the source, where the
grading is finest and the near-field integrals dominate, and 24 seeded ones.

Bars (stated per check):
  FP64 matrix rows      max |A_gpu - A_oracle| <= 1e-12 * max |A_oracle row|
  FP64 right-hand side  same bar on the sampled rows
  mixed matrix rows     max |A_gpu - A_oracle| <= 2e-6 * max |A_oracle row|
                        (complex64 storage and FP32 quadrature; measured on
                        GB300: 1.9e-7 at 100 Hz, 3.0e-7 at 10 kHz, 4.5e-7 at
                        20 kHz)
  FP64 solution         the residual of the oracle's rows, scaled to the
                        whole system (sqrt(N / 32) * ||r_sampled||), is at
                        most 1e-9 * ||b||
  mixed vs FP64         boundary pressure and grid field within 1e-4
                        relative L2, with the fp16 Krylov copy and with the
                        block low-rank copy the bench's batches use
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, workloads
from oracle import oracle_py as op

pytestmark = pytest.mark.gpu

FREQS = (100.0, 10000.0, 20000.0)


@pytest.fixture(scope="module")
def head():
    v, f, src, pts, _ = workloads.head_workload()
    m = capi.Mesh(v, f)
    om = op.OracleMesh(v, f)
    d = np.linalg.norm(om.centers - np.asarray(src)[None, :], axis=1)
    near = np.argsort(d)[:8]
    rng = np.random.default_rng(20261204)
    rest = rng.choice(np.setdiff1d(np.arange(len(f)), near), 24, replace=False)
    rows = np.sort(np.concatenate([near, rest]))
    yield {"v": v, "f": f, "src": src, "pts": pts, "mesh": m, "om": om, "rows": rows}
    m.close()


def _oracle_rows(h, fr):
    k = 2 * np.pi * fr / workloads.C0
    amp = 0.1 / (1j * workloads.RHO * 2 * np.pi * fr)
    of = op.OracleFreq(k, h["src"], [amp])
    A = np.zeros((len(h["rows"]), len(h["f"])), np.complex128)
    b = np.zeros(len(h["rows"]), np.complex128)
    for i, r in enumerate(h["rows"]):
        Ar, br = op.assemble(h["om"], of, rows=(int(r), int(r) + 1), nthreads=16)
        A[i], b[i] = Ar[0], br[0]
    return A, b


def _gpu_rows(s, rows):
    A = np.zeros((len(rows), s.n), np.complex128)
    b = None
    for i, r in enumerate(rows):
        Ar, b = s.system(rows=(int(r), int(r) + 1))
        A[i] = Ar[0]
    return A, b


@pytest.mark.parametrize("fr", FREQS)
def test_head20480_against_oracle(head, fr):
    n = len(head["f"])
    F = workloads.frequency(capi, n, fr, head["src"])
    Ao, bo = _oracle_rows(head, fr)
    scale = np.abs(Ao).max(axis=1)

    # FP64: matrix rows, right-hand side, and the solution's residual on the
    # oracle's rows
    s64 = capi.Solver(head["mesh"], precision=capi.PREC_FP64, tol=1e-11, max_iter=3000)
    s64.assemble(F)
    A64, b64 = _gpu_rows(s64, head["rows"])
    e_a64 = (np.abs(A64 - Ao).max(axis=1) / scale).max()
    assert e_a64 <= 1e-12, "FP64 rows: %.3e of the row scale" % e_a64
    e_b = np.abs(b64[head["rows"]] - bo).max() / np.abs(bo).max()
    assert e_b <= 1e-12, "FP64 b: %.3e" % e_b
    s64.solve()
    x64 = s64.solution()
    p64, _ = s64.project(head["pts"], with_grad=False)
    r = bo - Ao @ x64
    res = np.sqrt(n / len(r)) * np.linalg.norm(r) / np.linalg.norm(b64)
    assert res <= 1e-9, "FP64 residual on the oracle's rows: %.3e" % res
    s64.close()

    # mixed: matrix rows within the complex64/FP32 bound, solution and field
    # within the metric's 1e-4 of the FP64 results
    smx = capi.Solver(head["mesh"], precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000)
    smx.assemble(F)
    Amx, _ = _gpu_rows(smx, head["rows"])
    e_amx = (np.abs(Amx - Ao).max(axis=1) / scale).max()
    assert e_amx <= 2e-6, "mixed rows: %.3e of the row scale" % e_amx
    smx.solve()
    xmx = smx.solution()
    pmx, _ = smx.project(head["pts"], with_grad=False)
    smx.close()
    ex = np.linalg.norm(xmx - x64) / np.linalg.norm(x64)
    ep = np.linalg.norm(pmx - p64) / np.linalg.norm(p64)
    assert ex <= 1e-4 and ep <= 1e-4, "mixed vs FP64: boundary %.3e, field %.3e" % (ex, ep)

    # mixed with the block low-rank Krylov copy
    sbl = capi.Solver(head["mesh"], precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000,
                      complex64_krylov=capi.KRYLOV_BLR)
    sbl.assemble(F)
    sbl.solve()
    xbl = sbl.solution()
    pbl, _ = sbl.project(head["pts"], with_grad=False)
    sbl.close()
    exb = np.linalg.norm(xbl - x64) / np.linalg.norm(x64)
    epb = np.linalg.norm(pbl - p64) / np.linalg.norm(p64)
    assert exb <= 1e-4 and epb <= 1e-4, "block low-rank vs FP64: boundary %.3e, field %.3e" % (exb, epb)
    print("head20480 %.0f Hz: FP64 rows %.2e, b %.2e, residual %.2e; mixed rows %.2e, boundary %.2e, field %.2e; "
          "block low-rank boundary %.2e, field %.2e" % (fr, e_a64, e_b, res, e_amx, ex, ep, exb, epb))
