"""The GPU arm of bench.py: one JSON line with the measurement contract's
keys (value, e2e with its copied bytes, roofline with the achieved rate, the
measured peak and the per-stage fractions, cpu_baseline, gpu_launches,
clocks), on the 1280-triangle version of the head mesh (--mesh-n 8) in
batches of 4 so that it ends in seconds, with the block low-rank Krylov copy
(the default) and with the fp16 copy."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("copy", ["blr", "fp16"])
def test_gpu_arm_prints_the_contract_line(copy):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "2", "--warmup", "3",
                          "--mesh-n", "8", "--batch", "4", "--no-serving", "--krylov-copy", copy],
                         cwd=ROOT, capture_output=True, text=True, timeout=1200)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline",
                "gpu_launches", "clocks", "latency_ms", "fp64_gpu"):
        assert key in d, key
    assert d["unit"] == "solves/s" and d["value"] > 0 and d["gpu_launches"] > 0 and d["steps"] == 2
    assert d["config"]["n_elements"] == 1280 and d["config"]["batch_per_step"] == 4
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["achieved"] > 0 and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    assert len(r["stages"]) == 4 and all(s["actual_ms"] > 0 for s in r["stages"])
    assert r["bytes_per_krylov_product"] > 0
    if copy == "fp16":
        n = 1280
        assert r["bytes_per_krylov_product"] == n * n * 4.0 + 2 * n * 16.0
    assert d["cpu_baseline"]["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert d["fp64_gpu"]["mixed_rel_l2_boundary_err_max"] < 1e-4
