"""The project report (mesh2hrtf_gb300/output_report.py) against the
reference's write_output_report run on the reference's own NC*.out fixtures
(tests/golden/output_report.npz, made by make_output_report_golden.py):
report_source_*.csv, the issue flag and report_issues.txt, character for
character.  Cases: a clean run (case_0), a step recomputed by a second file
(case_4), missing steps (case_1), steps that did not converge (case_2), bad
input and missing steps (case_3), one clean and one broken source, and the
SHTF project (three NC*.out files per source, named two ways)."""
import json
import os

import numpy as np
import pytest

from mesh2hrtf_gb300 import output_report as orep

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "output_report.npz")
DOC = json.loads(str(np.load(GOLDEN)["doc"]))


def _project(root, case):
    (root / "parameters.json").write_text(json.dumps(case["parameters"]))
    for s, files in enumerate(case["files"]):
        d = root / "NumCalc" / ("source_%d" % (s + 1))
        d.mkdir(parents=True)
        for name, text in files.items():
            (d / name).write_text(text)


@pytest.mark.parametrize("name", sorted(DOC))
def test_report_matches_the_reference(tmp_path, name):
    case = DOC[name]
    _project(tmp_path, case)
    issues, report = orep.write_output_report(str(tmp_path))
    assert issues is case["issues"]
    assert (report or "") == case["report"]
    for s, ref in enumerate(case["csv"]):
        assert (tmp_path / "Output2HRTF" / ("report_source_%d.csv" % (s + 1))).read_text() == ref
    txt = tmp_path / "Output2HRTF" / "report_issues.txt"
    if case["issues_txt"] is None:
        assert not txt.exists()
    else:
        assert txt.read_text() == case["issues_txt"]


def test_sections_and_files(tmp_path):
    assert orep.parse_sections("no step marker here") is None
    sec = ("x\n" + orep.STEP_MARK + "\nStep 3, Frequency = 250.5 Hz\nCGS solver: number of iterations = 17, "
           "relative error = 2.5e-10\n" + "Total".ljust(39) + ": 4\n")
    got = orep.parse_sections(sec)
    assert got == {3: {1: 250.5, 3: 1, 4: 1, 5: 17, 6: 2.5e-10, 7: 4.0}}
    bad = orep.parse_sections(orep.STEP_MARK + "Step 2, Frequency = 10 Hz\n" + orep.NOT_CONVERGED + "\n"
                              + orep.BAD_INPUT)
    assert bad[2][3] == 0 and bad[2][4] == 0
    for n in ("NC2-2.out", "NC.out", "NC1-1.out", "other.out"):
        (tmp_path / n).write_text("")
    assert orep.nc_out_files(str(tmp_path)) == ["NC.out", "NC1-1.out", "NC2-2.out"]


def test_no_result_files_is_an_issue(tmp_path):
    (tmp_path / "parameters.json").write_text(json.dumps({"numFrequencies": 2}))
    (tmp_path / "NumCalc" / "source_1").mkdir(parents=True)
    issues, report = orep.write_output_report(str(tmp_path))
    assert issues and "Frequency steps that were not calculated:\n1, 2" in report
    csv = (tmp_path / "Output2HRTF" / "report_source_1.csv").read_text().splitlines()
    assert csv[1] == "1, -1.0, ,-1, -1, -1, -1.0, -1, -1, -1, -1"
