"""The drop-in NumCalc end to end on the GPU: same files and numbers as the
reference NumCalc on the same project (reference results from
tests/golden/sphere80.npz, printed there with 17 digits, here with NumCalc's
7-digit format)."""
import os
import pathlib
import subprocess

import numpy as np
import pytest

from mesh2hrtf_gb300 import build, capi, meshes, output_report, project, sofa
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def numcalc():
    build.build_all()
    return build.NUMCALC_BIN


def _project(tmp_path, name="sphere80", precond=0):
    c = gc.load(name)
    if name == "sphere80":
        ps = c["point_sources"]
        sh = [c.pts[:24], c.pts[24:]]
        p = project.Project(root=str(tmp_path / "p"), nodes=c.nodes, elems=c.elems, eval_points=c.pts,
                            eval_elems=meshes.shells_triangles(sh), freqs=list(c.freqs),
                            point_sources=[tuple(ps[0])], boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"],
                            precond=precond)
    else:   # sphere320_adm_velo: admittance everywhere, velocity source on 3 elements
        p = project.Project(root=str(tmp_path / "p"), nodes=c.nodes, elems=c.elems, eval_points=c.pts,
                            eval_elems=meshes.grid_triangles(c.pts), freqs=list(c.freqs),
                            boundary=["ELEM 0 TO 319 ADMI 0.5 -1 0.2 -1", "ELEM 10 TO 12 VELO 0.1 -1 0.0 -1"])
    return c, project.write_project(p)


@pytest.mark.parametrize("name", ["sphere80", "sphere320_adm_velo"])
@pytest.mark.parametrize("precision,tol", [("fp64", 2e-6), ("mixed", 1e-5)])
def test_be_out_matches_reference(numcalc, tmp_path, precision, tol, name):
    c, wd = _project(tmp_path, name)
    env = dict(os.environ, NUMCALC_GB300_PRECISION=precision)
    r = subprocess.run([numcalc], cwd=wd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    out = pathlib.Path(os.path.join(wd, "NC.out")).read_text()
    assert out.count(">> S T E P   N U M B E R   A N D   F R E Q U E N C Y <<") == len(c.freqs)
    assert "CGS solver: number of iterations = " in out and "End time:" in out
    assert "Assembling the equation system         : " in out
    for s in range(1, len(c.freqs) + 1):
        for f in ("pBoundary", "vBoundary", "pEvalGrid", "vEvalGrid"):
            ids, vals = project.read_result(os.path.join(wd, "be.out", "be.%d" % s, f))
            assert np.array_equal(ids, c["s%d_%s_ids" % (s, f)])
            ref = c["s%d_%s" % (s, f)]
            if np.abs(ref).max() == 0:
                assert np.abs(vals).max() == 0
            else:
                assert gc.rel_err(vals, ref) < tol, (s, f, gc.rel_err(vals, ref))


@pytest.mark.parametrize("precond", [1, 2])
def test_scaling_and_no_preconditioner(numcalc, tmp_path, precond):
    """NC.inp's scaling preconditioner (1) and none (2): the same results as
    the reference's (ILU) run within the mixed path's bar."""
    c, wd = _project(tmp_path, "sphere80", precond)
    r = subprocess.run([numcalc], cwd=wd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    out = pathlib.Path(os.path.join(wd, "NC.out")).read_text()
    assert ("with the scaling preconditioner above" if precond == 1 else "without a preconditioner") in out
    for s in range(1, len(c.freqs) + 1):
        for f in ("pBoundary", "pEvalGrid"):
            ids, vals = project.read_result(os.path.join(wd, "be.out", "be.%d" % s, f))
            assert gc.rel_err(vals, c["s%d_%s" % (s, f)]) < 1e-5, (s, f)


@pytest.mark.parametrize("nitermax", [0, 1, 2])
def test_nitermax_reports_limit(numcalc, tmp_path, nitermax):
    # 320 unknowns: more than one preconditioner block, so a few iterations
    # are needed (with 80 unknowns the block-Jacobi inverse is exact)
    c, wd = _project(tmp_path, "sphere320_adm_velo")
    r = subprocess.run([numcalc, "-nitermax", str(nitermax)], cwd=wd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    out = pathlib.Path(os.path.join(wd, "NC.out")).read_text()
    assert "CGS solver: number of iterations = %d" % nitermax in out
    assert "Warning: Maximum number of iterations is reached!" in out
    # then, as NumCalc (NC_CommonFunctions.cpp:1181-1191), the direct solver
    assert "Iteration method CGS failed, direct method is used!" in out
    # the step still ends with the system's solution
    ids, vals = project.read_result(os.path.join(wd, "be.out", "be.1", "pEvalGrid"))
    assert gc.rel_err(vals, c["s1_pEvalGrid"]) < 1e-5


def test_istart_iend_keeps_other_steps(numcalc, tmp_path):
    c, wd = _project(tmp_path)
    assert subprocess.run([numcalc, "-istart", "2", "-iend", "2"], cwd=wd, capture_output=True).returncode == 0
    assert os.path.exists(os.path.join(wd, "NC2-2.out"))
    assert os.path.exists(os.path.join(wd, "be.out", "be.2", "pEvalGrid"))
    assert not os.path.exists(os.path.join(wd, "be.out", "be.1"))
    assert subprocess.run([numcalc, "-istart", "1", "-iend", "1"], cwd=wd, capture_output=True).returncode == 0
    assert os.path.exists(os.path.join(wd, "be.out", "be.2", "pEvalGrid"))
    out = pathlib.Path(os.path.join(wd, "NC1-1.out")).read_text()
    assert "Step 1," in out and "Step 2," not in out


def test_manage_numcalc_runs_every_step_on_the_gpu(numcalc, tmp_path):
    """The GPU-aware scheduler on a two-source project: both sources' steps
    run as drop-in processes under device-memory admission, and every step's
    be.out equals the reference's (source 1 is the sphere80 fixture)."""
    from mesh2hrtf_gb300 import manage_numcalc as mn
    c = gc.load("sphere80")
    ps = c["point_sources"]
    sh = [c.pts[:24], c.pts[24:]]
    p = project.Project(root=str(tmp_path / "p"), nodes=c.nodes, elems=c.elems, eval_points=c.pts,
                        eval_elems=meshes.shells_triangles(sh), freqs=list(c.freqs),
                        point_sources=[tuple(ps[0])], boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"])
    project.write_project(p, "source_1")
    p.point_sources = [(-0.4, 0.2, 0.1, 1.0, 0.0)]
    wd2 = project.write_project(p, "source_2")
    pathlib.Path(os.path.join(str(tmp_path / "p"), "parameters.json")).write_text("{}")
    mn.manage_numcalc(str(tmp_path / "p"), numcalc, max_hbm_load=20.0, steps_per_instance=1, wait_time=0.05)
    wd1 = os.path.join(str(tmp_path / "p"), "NumCalc", "source_1")
    for s in range(1, len(c.freqs) + 1):
        assert "End time:" in pathlib.Path(os.path.join(wd1, "NC%d-%d.out" % (s, s))).read_text()
        ids, vals = project.read_result(os.path.join(wd1, "be.out", "be.%d" % s, "pEvalGrid"))
        assert gc.rel_err(vals, c["s%d_pEvalGrid" % s]) < 1e-5
        assert os.path.isfile(os.path.join(wd2, "be.out", "be.%d" % s, "pEvalGrid"))
    assert os.path.isfile(os.path.join(wd1, "MemoryGPU.txt"))


def test_full_precision_results_and_hrtfs(numcalc, tmp_path):
    """NUMCALC_GB300_NPY=1: every result file also as .npy (the printed
    values at full precision); the project report parses the run's NC.out;
    Output2HRTF's referencing reads the results and equals the same HRTFs
    made from the solver's in-memory results (mesh2hrtf_gb300/output2hrtf.py,
    output_report.py)."""
    import json

    from mesh2hrtf_gb300 import output2hrtf as o2h
    c, wd = _project(tmp_path)
    env = dict(os.environ, NUMCALC_GB300_PRECISION="fp64", NUMCALC_GB300_NPY="1")
    r = subprocess.run([numcalc], cwd=wd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    for s in range(1, len(c.freqs) + 1):
        d = os.path.join(wd, "be.out", "be.%d" % s)
        for f in ("pBoundary", "vBoundary", "pEvalGrid", "vEvalGrid"):
            ids, txt = project.read_result(os.path.join(d, f))
            full = np.load(os.path.join(d, f + ".npy"))
            assert full.shape == np.asarray(txt).shape
            assert gc.rel_err(full, txt) < 1e-6                     # 7 printed digits
            assert gc.rel_err(full, c["s%d_%s" % (s, f)]) < 2e-6     # the reference, 17 digits
    root = str(tmp_path / "p")
    pathlib.Path(os.path.join(root, "parameters.json")).write_text(json.dumps({
        "Mesh2HRTF_Version": "1.0.0", "speedOfSound": 343.0, "densityOfMedium": 1.21,
        "evaluationGrids": ["Grid"], "sourceType": "Point source", "numSources": 1,
        "sourceCenter": [[0.5, 0.1, 0.0]], "sourceArea": [], "reference": True, "computeHRIRs": False,
        "numFrequencies": len(c.freqs), "frequencies": [float(v) for v in c.freqs]}))
    # the drop-in's NC.out through the project report: every step found,
    # converged, with its iterations and timings (no -1 anywhere)
    issues, text = output_report.write_output_report(root)
    assert not issues, text
    rows = pathlib.Path(os.path.join(root, "Output2HRTF", "report_source_1.csv")).read_text().splitlines()[1:]
    assert len(rows) == len(c.freqs)
    for r, f in zip(rows, c.freqs):
        v = [x.strip() for x in r.split(",")]
        assert v[2] == "NC.out" and float(v[1]) == float("%g" % f) and int(v[5]) > 0 and 0 <= float(v[6]) <= 1e-9
    h = sofa.read(o2h.output2hrtf(root)[0])
    hrtf = h["Data_Real"] + 1j * h["Data_Imag"]
    assert hrtf.shape == (len(c.pts), 1, len(c.freqs)) and np.all(np.isfinite(hrtf))
    assert h["GLOBAL_SOFAConventions"] == "GeneralTF"
    # the same HRTFs straight from the solver's results (no result file)
    with open(os.path.join(root, "parameters.json")) as fh:
        params = json.load(fh)
    m = capi.Mesh(c.nodes, c.elems)
    sv = capi.Solver(m, precision=capi.PREC_FP64, tol=1e-9)   # the drop-in's tolerance
    pres = []
    for s in range(1, len(c.freqs) + 1):
        st = c.step(s)
        fr = capi.Frequency(st["k"], c.n, bc_type=st["bc_type"], bc_value=st["bc_value"],
                            admittance=st["admittance"], point_sources=st["point_sources"],
                            point_amps=st["point_amps"], plane_dirs=st["plane_dirs"], plane_amps=st["plane_amps"])
        _, pot, _ = sv.solve_frequency(fr, c.pts, with_grad=False)
        pres.append(1j * st["rpfact"] * pot)   # pressure = i rho omega potential
    sv.close()
    m.close()
    mem, _ = o2h.hrtf_sofa(np.stack(pres, axis=-1)[:, None, :], c.pts, params)
    assert gc.rel_err(mem["Data_Real"] + 1j * mem["Data_Imag"], hrtf) < 1e-6
