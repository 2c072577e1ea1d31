"""The reference arm of bench.py on the CPU: the FP64 C restatement of
NumCalc's path (assembly, NumCalc's CGS with threshold ILU, projection),
complete solves timed on the host cores, prints one JSON line with the keys
the measurement contract names, on the same metric as the GPU arm.  The test
runs it on the 1280-triangle version of the head mesh (--mesh-n 8) so that
it ends in seconds; the bench's default is the 20480-triangle workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3", "--mesh-n", "8"], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and 1 <= d["steps"] <= d["steps_requested"] == 2 and d["warmup"] >= 3
    assert d["config"]["n_elements"] == 1280 and d["config"]["n_eval_points"] == 1730
    # one step is one complete solve: the step time and the value agree
    assert abs(d["ms_per_step"] * d["value"] / 1000.0 - d["solves_per_step"]) < 1e-9
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert len(cb["solves"]) == d["steps"]
    for s in cb["solves"]:
        assert s["cgs_rel_err"] < 1e-9 and not s["direct_fallback"] and s["cgs_iterations"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
