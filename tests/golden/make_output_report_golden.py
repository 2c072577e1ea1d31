"""Golden vectors for the project report (write_output_report): the
reference's NC*.out fixtures (mesh2hrtf tests/resources/nc.out/case_0..4 and
the SHTF project's NC1-20/21-40/41-60.out of both sources) and what the
reference's own write_output_report makes of them (report_source_*.csv, the
issue flag and report_issues.txt).

    python tests/golden/make_output_report_golden.py

with MESH2HRTF_REFERENCE set to the root of a Mesh2HRTF checkout.

The reference module is loaded from its file (it needs only numpy; the
mesh2hrtf package itself imports sofar, which is not installed) and run on
a scratch copy of each project.  Writes tests/golden/output_report.npz: one
JSON document with, per case, the NC*.out texts of every source, the
parameters.json, and the reference's outputs.
"""
from __future__ import annotations

import importlib.util
import json
import os
import pathlib
import shutil
import sys
import tempfile

import numpy as np

CASES = {
    "case_0": ["case_0"], "case_4": ["case_4"], "case_1": ["case_1"], "case_2": ["case_2"],
    "case_3": ["case_3"], "case_0+case_1": ["case_0", "case_1"],
}


def main(ref_root):
    spec = importlib.util.spec_from_file_location(
        "ref_write_output_report", os.path.join(ref_root, "mesh2hrtf", "Output2HRTF", "write_output_report.py"))
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    res = os.path.join(ref_root, "tests", "resources")
    projects = {}
    for name, folders in CASES.items():
        srcs = [os.path.join(res, "nc.out", f) for f in folders]
        projects[name] = (os.path.join(res, "nc.out", "parameters.json"), srcs)
    shtf = os.path.join(res, "SHTF")
    projects["SHTF"] = (os.path.join(shtf, "parameters.json"),
                        [os.path.join(shtf, "NumCalc", "source_%d" % s) for s in (1, 2)])
    out = {}
    for name, (params, srcs) in projects.items():
        tmp = tempfile.mkdtemp()
        try:
            os.makedirs(os.path.join(tmp, "NumCalc"))
            os.makedirs(os.path.join(tmp, "Output2HRTF"))
            shutil.copyfile(params, os.path.join(tmp, "parameters.json"))
            files = []
            for s, src in enumerate(srcs):
                dst = os.path.join(tmp, "NumCalc", "source_%d" % (s + 1))
                os.makedirs(dst)
                texts = {}
                for f in sorted(os.listdir(src)):
                    if f.startswith("NC") and f.endswith(".out"):
                        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
                        texts[f] = pathlib.Path(os.path.join(src, f)).read_text()
                files.append(texts)
            issues, report = ref.write_output_report(tmp)
            csv = [pathlib.Path(os.path.join(tmp, "Output2HRTF", "report_source_%d.csv" % (s + 1))).read_text()
                   for s in range(len(srcs))]
            issues_txt = os.path.join(tmp, "Output2HRTF", "report_issues.txt")
            out[name] = {"parameters": json.loads(pathlib.Path(params).read_text()), "files": files, "issues": bool(issues),
                         "report": report or "", "csv": csv,
                         "issues_txt": pathlib.Path(issues_txt).read_text() if os.path.isfile(issues_txt) else None}
        finally:
            shutil.rmtree(tmp)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "output_report.npz")
    np.savez_compressed(dst, doc=np.array(json.dumps(out)))
    print("wrote %s: %s" % (dst, ", ".join("%s (issues %s)" % (k, v["issues"]) for k, v in out.items())))


if __name__ == "__main__":
    root = os.environ.get("MESH2HRTF_REFERENCE", "")
    if not os.path.isdir(root):
        sys.exit("set MESH2HRTF_REFERENCE to the root of a Mesh2HRTF checkout")
    main(root)
