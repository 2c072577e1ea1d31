"""Golden vectors for -estimate_ram on FMM projects: the reference NumCalc
(oracle/_ref/NumCalc, built by oracle/Makefile from the reference's sources)
run with -estimate_ram on the projects of tests/fmm_estimate_cases.py, and
on the reference's own SHTF test project (mesh2hrtf tests/resources/SHTF,
whose Memory.txt the reference's test_numcalc_commandline_estimate_ram
checks).

    python tests/golden/make_fmm_estimate_golden.py

with MESH2HRTF_REFERENCE set to the root of a Mesh2HRTF checkout (for the
SHTF files) and oracle/_ref built.  Writes tests/golden/fmm_estimate.npz:
per case the reference's Memory.txt and the count lines it printed, and the
SHTF project's input files.
"""
from __future__ import annotations

import json
import os
import pathlib
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refdump  # noqa: E402
from tests import fmm_estimate_cases as fc  # noqa: E402

SHTF_FILES = ("NumCalc/source_1/NC.inp", "ObjectMeshes/Reference/Nodes.txt", "ObjectMeshes/Reference/Elements.txt",
              "EvaluationGrids/FourPointHorPlane_r100cm/Nodes.txt",
              "EvaluationGrids/FourPointHorPlane_r100cm/Elements.txt")


def run_reference(wd):
    r = subprocess.run([refdump.REF_NUMCALC, "-estimate_ram"], cwd=wd, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError("reference NumCalc failed in %s: %s" % (wd, r.stdout[-2000:]))
    return fc.memory_txt(wd), fc.count_lines(r.stdout)


def main(ref_root):
    out = {}
    tmp = tempfile.mkdtemp()
    try:
        for name in fc.CASES:
            wd = fc.write(name, os.path.join(tmp, name))
            mem, counts = run_reference(wd)
            out[name] = {"memory": mem, "counts": counts}
            print("%-22s %3d steps, %s" % (name, len(mem.splitlines()),
                                           sorted(set(c.split(":")[0].split(" ")[0] for c in counts
                                                      if c.startswith(("TBEM", "SLFMM", "MLFMM"))))))
        shtf = os.path.join(ref_root, "tests", "resources", "SHTF")
        files = {f: pathlib.Path(os.path.join(shtf, f)).read_text() for f in SHTF_FILES}
        root = os.path.join(tmp, "SHTF")
        for f, text in files.items():
            os.makedirs(os.path.dirname(os.path.join(root, f)), exist_ok=True)
            pathlib.Path(os.path.join(root, f)).write_text(text)
        mem, counts = run_reference(os.path.join(root, "NumCalc", "source_1"))
        committed = pathlib.Path(os.path.join(shtf, "NumCalc", "source_1", "Memory.txt")).read_text()
        if mem != committed:
            raise RuntimeError("the reference NumCalc built here does not reproduce the SHTF Memory.txt")
        out["SHTF"] = {"memory": mem, "counts": counts, "files": files}
        print("SHTF: the reference built here reproduces the committed Memory.txt")
    finally:
        shutil.rmtree(tmp)
    dst = os.path.join(HERE, "fmm_estimate.npz")
    np.savez_compressed(dst, doc=np.array(json.dumps(out)))
    print("wrote", dst)


if __name__ == "__main__":
    root = os.environ.get("MESH2HRTF_REFERENCE", "")
    if not os.path.isdir(root):
        sys.exit("set MESH2HRTF_REFERENCE to the root of a Mesh2HRTF checkout")
    main(root)
