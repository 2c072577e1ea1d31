"""Test infrastructure (oracle only): run the reference NumCalc built in
oracle/_ref and read what its dump harness (oracle/ref_dump.cpp) wrote.

Only tests, fixture scripts and the bench's CPU-baseline leg use this file.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_NUMCALC = os.path.join(REF_DIR, "NumCalc")
REF_NUMCALC_DUMP = os.path.join(REF_DIR, "NumCalc_dump")
# Root of a Mesh2HRTF checkout holding the reference sources, from the
# environment; unset means the reference is absent and build() skips.
REFERENCE_ENV = "MESH2HRTF_REFERENCE"


def reference_root():
    root = os.environ.get(REFERENCE_ENV, "")
    return root if root and os.path.isdir(root) else None


def default_refsrc():
    root = reference_root()
    return os.path.join(root, "mesh2hrtf", "NumCalc", "src") if root else None

_DT = {"f8": (np.float64, 8), "i4": (np.int32, 4), "c16": (np.complex128, 16)}


def available() -> bool:
    return os.path.isfile(REF_NUMCALC_DUMP) and os.access(REF_NUMCALC_DUMP, os.X_OK)


def build(refsrc: str | None = None) -> bool:
    """Build oracle/_ref when the reference sources are present."""
    refsrc = refsrc or default_refsrc()
    if not refsrc or not os.path.isfile(os.path.join(refsrc, "NC_Main.cpp")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "-j8", "REFSRC=" + refsrc], check=True)
    return available()


def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as fh:
        while True:
            head = fh.read(40)
            if len(head) < 40:
                break
            name = head[:24].split(b"\0")[0].decode()
            dt = head[24:32].split(b"\0")[0].decode()
            cnt = int(np.frombuffer(head[32:40], dtype=np.int64)[0])
            typ, sz = _DT[dt]
            out[name] = np.frombuffer(fh.read(cnt * sz), dtype=typ).copy()
    return out


def run(workdir: str, args=(), dump_dir: str | None = None, binary: str | None = None,
        timeout: float = 3600.0):
    """Run the reference NumCalc in ``workdir`` (the NumCalc/source_k folder)."""
    exe = binary or (REF_NUMCALC_DUMP if dump_dir else REF_NUMCALC)
    env = dict(os.environ)
    if dump_dir:
        os.makedirs(dump_dir, exist_ok=True)
        env["NC_DUMP_DIR"] = dump_dir
    return subprocess.run([exe, *args], cwd=workdir, env=env, capture_output=True,
                          text=True, timeout=timeout)
