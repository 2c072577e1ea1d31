"""-check_normals (NC_checkedges, NC_Input.cpp:741-789, called from
NC_ReadMesh, NC_Input.cpp:512-518): the drop-in's half-edge test of the
element orientation, on the CPU (it stops before any device work).

Expected output recorded from the reference NumCalc (built by oracle/Makefile)
on the same project, the 80-triangle sphere with element 5's nodes 15 and 16
swapped: exit code 1, one "Problem with element containing the node <id>"
line on stderr per unbalanced node (12, 15, 16), and the message below as the
last line of stdout and of NC.out.  Where the reference build is present the
test also runs it live and compares.
"""
import os
import pathlib
import subprocess

import pytest

from mesh2hrtf_gb300 import build, meshes, project
from oracle import refdump

MESSAGE = "There seems to be at least one element that is differently ordered to the rest"
REF_STDERR = ["Problem with element containing the node 12", "Problem with element containing the node 15",
              "Problem with element containing the node 16"]


@pytest.fixture(scope="module")
def numcalc():
    build.build_all()
    return build.NUMCALC_BIN


def _project(tmp_path, flip):
    v, f = meshes.icosphere(80, 0.1)
    f = f.copy()
    if flip:
        f[5] = f[5][[0, 2, 1]]
    pts = meshes.random_sphere_points(12, 0.5, 3)
    p = project.Project(root=str(tmp_path / "p"), nodes=v, elems=f, eval_points=pts,
                        eval_elems=meshes.grid_triangles(pts), freqs=[1000.0],
                        point_sources=[(0.5, 0.0, 0.0, 0.1, 0.0)], boundary=["ELEM 0 TO 79 VELO 0.0 -1 0.0 -1"])
    return project.write_project(p)


def _run(exe, wd, env=None):
    r = subprocess.run([exe, "-check_normals"], cwd=wd, capture_output=True, text=True, env=env, timeout=120)
    return r.returncode, r.stdout.strip().split("\n")[-1], [ln for ln in r.stderr.split("\n") if ln.strip()]


def test_flipped_element_is_reported_as_the_reference_does(numcalc, tmp_path):
    wd = _project(tmp_path, flip=True)
    rc, last, err = _run(numcalc, wd)
    assert rc == 1 and last == MESSAGE and err == REF_STDERR
    assert pathlib.Path(os.path.join(wd, "NC.out")).read_text().strip().split("\n")[-1] == MESSAGE
    if refdump.available():
        wd2 = _project(tmp_path / "ref", flip=True)
        assert _run(refdump.REF_NUMCALC, wd2) == (rc, last, err)


def test_consistent_mesh_passes_the_check(numcalc, tmp_path):
    wd = _project(tmp_path, flip=False)
    env = dict(os.environ, NUMCALC_GB300_DUMP_TABLES=str(tmp_path / "tables.bin"))
    rc, last, err = _run(numcalc, wd, env)
    assert rc == 0 and err == []
