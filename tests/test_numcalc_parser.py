"""Drop-in NumCalc without a GPU: NC.inp / mesh parsing parity with the
reference (table digests from tests/golden/parser/digests.json), error exits,
command line, output naming and -estimate_ram for traditional-BEM projects."""
import json
import os
import pathlib
import shutil
import subprocess
import sys

import numpy as np
import pytest

from mesh2hrtf_gb300 import build
from oracle import refdump

HERE = os.path.dirname(os.path.abspath(__file__))
PARSER = os.path.join(HERE, "golden", "parser")
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_parser_cases as mpc  # noqa: E402

REF = json.loads(pathlib.Path(os.path.join(PARSER, "digests.json")).read_text())


@pytest.fixture(scope="module")
def numcalc():
    build.build_all()
    return build.NUMCALC_BIN


def _copy(case, tmp_path):
    dst = tmp_path / case
    shutil.copytree(os.path.join(PARSER, case), dst)
    return str(dst / "NumCalc" / "source_1")


@pytest.mark.parametrize("case", sorted(REF))
def test_parsed_tables_match_reference(case, numcalc, tmp_path):
    wd = _copy(case, tmp_path)
    env = dict(os.environ, NUMCALC_GB300_DUMP_TABLES=str(tmp_path / "tables.bin"))
    r = subprocess.run([numcalc, "-nitermax", "1"], cwd=wd, env=env, capture_output=True, text=True)
    ref = REF[case]
    assert r.returncode == ref["returncode"], r.stdout[-500:]
    if ref["returncode"] != 0:
        assert r.stdout.strip().split("\n")[-1] == ref["stdout_tail"]
        return
    got = mpc.table_digests(refdump.read_dump(str(tmp_path / "tables.bin")))
    assert got == ref["digests"]


@pytest.mark.parametrize("case", [c for c in sorted(REF) if "memory_txt" in REF[c]])
def test_estimate_ram_matches_reference(case, numcalc, tmp_path):
    wd = _copy(case, tmp_path)
    r = subprocess.run([numcalc, "-estimate_ram"], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-500:]
    assert pathlib.Path(os.path.join(wd, "Memory.txt")).read_text() == REF[case]["memory_txt"]
    assert not os.path.exists(os.path.join(wd, "be.out", "be.1"))


def test_unknown_flag(numcalc, tmp_path):
    r = subprocess.run([numcalc, "-invalid_parameter"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0
    assert "NumCalc was called with an unknown parameter or flag." in r.stderr


def test_help(numcalc, tmp_path):
    r = subprocess.run([numcalc, "-h"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0 and "-nitermax int" in r.stdout


def test_missing_input(numcalc, tmp_path):
    r = subprocess.run([numcalc], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "No input file found!" in r.stdout
    assert os.path.exists(tmp_path / "NC.out")


@pytest.mark.parametrize("args,name", [([], "NC.out"), (["-istart", "2"], "NCfrom2.out"),
                                       (["-iend", "2"], "NCuntil2.out"), (["-istart", "2", "-iend", "3"], "NC2-3.out")])
def test_output_naming_estimate_mode(args, name, numcalc, tmp_path):
    wd = _copy("plain", tmp_path)
    r = subprocess.run([numcalc, "-estimate_ram", *args], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 0
    assert os.path.exists(os.path.join(wd, name))
    mem = pathlib.Path(os.path.join(wd, "Memory.txt")).read_text().strip().split("\n")
    first = int(args[args.index("-istart") + 1]) if "-istart" in args else 1
    last = int(args[args.index("-iend") + 1]) if "-iend" in args else 3
    assert [int(l.split()[0]) for l in mem] == list(range(first, last + 1))


@pytest.mark.skipif(not (refdump.available() or refdump.default_refsrc()), reason="reference build and sources not present")
@pytest.mark.parametrize("case", sorted(REF))
def test_live_reference_agrees(case, numcalc, tmp_path):
    """Where the reference builds (this container), compare directly."""
    if not refdump.available():
        refdump.build()
    wd = _copy(case, tmp_path)
    live = mpc.reference_result(wd)
    assert live["returncode"] == REF[case]["returncode"]
    assert live.get("digests") == REF[case].get("digests")
