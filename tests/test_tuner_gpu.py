"""The launch-shape tuner (bem_tune.cu, bem_tune_info).

Only shapes that leave every result bit unchanged are tuned: the assembly's
persistent grids and the complex64 product's strip height.  So a solve with
the tuner on equals the solve with the defaults (BEM_GB300_TUNE=0) bit for
bit, and a choice made in one process is read back from the cache file by
the next.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes, workloads

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _solve(m, f, n, fr=6000.0):
    s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
    x, pot, grad = s.solve_frequency(workloads.frequency(capi, n, fr, [0.3, 0.1, 0.05]),
                                     meshes.random_sphere_points(32, 1.2, 3))
    s.close()
    return x, pot


def test_tuned_shapes_change_no_result_bit(monkeypatch):
    v, f = meshes.perturbed_ellipsoid(12, 91)   # 2880 triangles
    n = len(f)
    m = capi.Mesh(v, f)
    monkeypatch.setenv("BEM_GB300_TUNE", "0")
    x0, p0 = _solve(m, f, n)
    assert capi.tune_info(n)["enabled"] is False
    monkeypatch.delenv("BEM_GB300_TUNE")
    x1, p1 = _solve(m, f, n)
    x2, p2 = _solve(m, f, n)
    info = capi.tune_info(n)
    assert info["assembly"]["tuned"] and info["product"]["tuned"]
    assert info["product"]["strip_rows"] in (16, 32, 64, 128)
    assert 1 <= info["assembly"]["far_blocks_per_sm"] <= 3
    assert np.array_equal(x0, x1) and np.array_equal(x1, x2)
    assert np.array_equal(p0, p1) and np.array_equal(p1, p2)
    m.close()


PROG = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
from mesh2hrtf_gb300 import capi, meshes, workloads
v, f = meshes.perturbed_ellipsoid(10, 92)
n = len(f)
if sys.argv[2] == "solve":
    m = capi.Mesh(v, f)
    s = capi.Solver(m, precision=capi.PREC_MIXED, tol=1e-9)
    s.solve_frequency(workloads.frequency(capi, n, 3000.0, [0.3, 0.0, 0.0]), meshes.random_sphere_points(8, 1.2, 1))
print(json.dumps(capi.tune_info(n)))
"""


def test_choices_persist_in_the_cache_file(tmp_path):
    cache = tmp_path / "tune.txt"
    env = dict(os.environ, BEM_GB300_TUNE_CACHE=str(cache))
    env.pop("BEM_GB300_TUNE", None)
    a = subprocess.run([sys.executable, "-c", PROG, ROOT, "solve"], env=env, capture_output=True, text=True,
                       timeout=600)
    assert a.returncode == 0, a.stderr[-2000:]
    first = json.loads(a.stdout.strip().splitlines()[-1])
    assert first["assembly"]["tuned"] and first["product"]["tuned"]
    lines = cache.read_text().splitlines()
    assert any(" asm " in ln for ln in lines) and any(" mv " in ln for ln in lines)
    # a new process reads the choice back without solving
    b = subprocess.run([sys.executable, "-c", PROG, ROOT, "info"], env=env, capture_output=True, text=True,
                       timeout=600)
    assert b.returncode == 0, b.stderr[-2000:]
    second = json.loads(b.stdout.strip().splitlines()[-1])
    for part, keys in (("assembly", ("far_blocks_per_sm", "near_blocks_per_sm", "tuned")),
                       ("product", ("strip_rows", "tuned"))):
        for k in keys:
            assert second[part][k] == first[part][k], (part, k)
