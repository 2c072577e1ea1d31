"""NC.inp's preconditioner choice (Main Parameters II, token 4; NC_Input.cpp
:292-323) in the drop-in: NumCalc's echo line for the choice, and the GPU
solver's line beside it (nc_project.cpp), which names what runs: the
block-Jacobi preconditioner with its window correction for the incomplete
LU (0 and the scanning degrees -1..-3), NumCalc's scaling preconditioner for
1, none for 2.  On the CPU: the executable stops after parsing
(NUMCALC_GB300_DUMP_TABLES), after NC.out's header is written; the solver
option itself (bem_solver_params.no_precond) is covered on the GPU by
tests/test_precond_gpu.py.
"""
import os
import pathlib
import subprocess

import pytest

from mesh2hrtf_gb300 import build, meshes, project


@pytest.fixture(scope="module")
def numcalc():
    build.build_all()
    return build.NUMCALC_BIN


def _nc_out(exe, tmp_path, precond):
    v, f = meshes.icosphere(80, 0.1)
    pts = meshes.random_sphere_points(12, 0.5, 3)
    p = project.Project(root=str(tmp_path / ("p%d" % precond)), nodes=v, elems=f, eval_points=pts,
                        eval_elems=meshes.grid_triangles(pts), freqs=[1000.0],
                        point_sources=[(0.5, 0.0, 0.0, 0.1, 0.0)], boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"],
                        precond=precond)
    wd = project.write_project(p)
    env = dict(os.environ, NUMCALC_GB300_DUMP_TABLES=str(tmp_path / ("tables%d.bin" % precond)))
    r = subprocess.run([exe], cwd=wd, capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    return pathlib.Path(os.path.join(wd, "NC.out")).read_text()


@pytest.mark.parametrize("precond,echo,gpu", [
    (0, "methodPreconditioner_ = 0: incomplete LU-decomposition preconditioner", "with a block-Jacobi preconditioner"),
    (-2, "methodPreconditioner_ = 0: incomplete LU-decomposition preconditioner", "with a block-Jacobi preconditioner"),
    (1, "methodPreconditioner_ = 1: scaling preconditioner", "with the scaling preconditioner above"),
    (2, "methodPreconditioner_ = 2: no preconditioner", "without a preconditioner"),
])
def test_preconditioner_choice_is_echoed_and_named(numcalc, tmp_path, precond, echo, gpu):
    out = _nc_out(numcalc, tmp_path, precond)
    assert echo in out
    line = [ln for ln in out.splitlines() if ln.startswith("GPU solver:")]
    assert len(line) == 1 and gpu in line[0]
