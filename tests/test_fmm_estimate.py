"""-estimate_ram on SL-/ML-FMM projects (mesh2hrtf_gb300/numcalc/src/
nc_fmm_plan.cpp): the drop-in writes the reference NumCalc's Memory.txt byte
for byte, and prints the same matrix counts, on the reference's SHTF test
project (the file its test_numcalc_commandline_estimate_ram compares) and
on projects that exercise traditional-BEM steps, single- and multilevel
FMM, the fall-back between them, frequencies in falling order,
quadrilaterals, several element groups, the minimum expansion order, a
prescribed cluster edge length and one to three symmetry planes (the
clusters' images) (tests/fmm_estimate_cases.py; golden files
from the reference built here, tests/golden/make_fmm_estimate_golden.py).
No GPU: -estimate_ram makes no device call."""
import json
import os
import pathlib
import subprocess

import numpy as np
import pytest

from mesh2hrtf_gb300 import build
from tests import fmm_estimate_cases as fc

GOLDEN = json.loads(str(np.load(os.path.join(os.path.dirname(__file__), "golden", "fmm_estimate.npz"))["doc"]))


@pytest.fixture(scope="module")
def numcalc():
    return build.build_numcalc()


def _estimate(numcalc, wd):
    r = subprocess.run([numcalc, "-estimate_ram"], cwd=wd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    return fc.memory_txt(wd), fc.count_lines(r.stdout)


@pytest.mark.parametrize("name", fc.CASES)
def test_memory_txt_matches_the_reference(numcalc, tmp_path, name):
    wd = fc.write(name, tmp_path / "p")
    mem, counts = _estimate(numcalc, wd)
    assert mem == GOLDEN[name]["memory"]
    assert counts == GOLDEN[name]["counts"]


def test_shtf_memory_txt(numcalc, tmp_path):
    case = GOLDEN["SHTF"]
    for f, text in case["files"].items():
        (tmp_path / f).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / f).write_text(text)
    wd = tmp_path / "NumCalc" / "source_1"
    mem, counts = _estimate(numcalc, str(wd))
    assert mem == case["memory"]
    assert counts == case["counts"]
    # the device-memory estimate for this build's own scheduler is written too
    assert len(pathlib.Path(wd / "MemoryGPU.txt").read_text().splitlines()) == len(mem.splitlines())
