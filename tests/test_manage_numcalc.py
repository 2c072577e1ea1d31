"""GPU-aware NumCalc scheduling (mesh2hrtf_gb300/manage_numcalc.py) on the
CPU, with a stand-in NumCalc that records when it ran, on which device and
with which footprint: device-memory admission, ranges of steps per process,
completion and error rules of the reference's manage_numcalc
(mesh2hrtf/NumCalc/manage_numcalc.py)."""
import json
import os
import stat
import sys

import numpy as np
import pytest

from mesh2hrtf_gb300 import manage_numcalc as mn

FAKE = r'''#!{python}
import json, os, sys, time
args = sys.argv[1:]
cfg = json.load(open("fake.json"))
steps = {{int(s): (f, gb) for s, f, gb in cfg["steps"]}}
if "-estimate_ram" in args:
    with open("MemoryGPU.txt", "w") as fh:
        for s in sorted(steps):
            fh.write("%d %g %g\n" % (s, steps[s][0], steps[s][1]))
    with open("Memory.txt", "w") as fh:
        for s in sorted(steps):
            fh.write("%d %g %g\n" % (s, steps[s][0], 2 * steps[s][1]))
    sys.exit(0)
a = int(args[args.index("-istart") + 1]); b = int(args[args.index("-iend") + 1])
dev = int(os.environ.get("NUMCALC_GB300_DEVICE", "0"))
gb = max(steps[k][1] for k in range(a, b + 1))
log = os.environ["FAKE_NUMCALC_LOG"]
t0 = time.time()
out = open("NC%d-%d.out" % (a, b), "w")
out.write("Start time\n")
for k in range(a, b + 1):
    if k in cfg.get("fail", []):
        sys.exit(3)
    time.sleep(cfg.get("sleep", 0.05))
    d = os.path.join("be.out", "be.%d" % k)
    os.makedirs(d, exist_ok=True)
    open(os.path.join(d, "pEvalGrid"), "w").write("x\n")
out.write("End time: now\n")
out.close()
with open(log, "a") as fh:
    fh.write(json.dumps([os.getcwd(), a, b, dev, gb, t0, time.time()]) + "\n")
'''


def _project(root, name, sources):
    p = root / name
    (p / "ObjectMeshes" / "Reference").mkdir(parents=True)
    for sid, steps in sources.items():
        d = p / "NumCalc" / ("source_%d" % sid)
        d.mkdir(parents=True)
        (d / "fake.json").write_text(json.dumps(steps))
    return p


@pytest.fixture
def fake(tmp_path, monkeypatch):
    exe = tmp_path / "bin" / "NumCalc"
    exe.parent.mkdir()
    exe.write_text(FAKE.format(python=sys.executable))
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    log = tmp_path / "runs.jsonl"
    monkeypatch.setenv("FAKE_NUMCALC_LOG", str(log))
    return str(exe), log


def _runs(log):
    return [json.loads(line) for line in log.read_text().splitlines()] if os.path.exists(log) else []


def _max_concurrent_gb(runs, dev):
    ev = []
    for _, a, b, d, gb, t0, t1 in runs:
        if d == dev:
            ev += [(t0, gb), (t1, -gb)]
    cur = best = 0.0
    for _, g in sorted(ev, key=lambda e: (e[0], e[1])):
        cur += g
        best = max(best, cur)
    return best


def test_admission_keeps_each_device_within_budget(tmp_path, fake):
    exe, log = fake
    steps = {"steps": [[k, 100.0 * k, 3.0] for k in range(1, 9)], "sleep": 0.15}
    root = tmp_path / "projects"
    root.mkdir()
    _project(root, "a", {1: steps, 2: steps})
    _project(root, "b", {1: {"steps": [[k, 50.0 * k, 5.0] for k in range(1, 5)], "sleep": 0.15}})
    mn.manage_numcalc(str(root), exe, max_hbm_load=10.0, hbm_safety_factor=1.0, devices=[0, 1],
                      max_instances=8, steps_per_instance=3, wait_time=0.02)
    runs = _runs(log)
    # every step ran exactly once, in ranges of at most 3 consecutive steps
    done = {}
    for cwd, a, b, d, gb, t0, t1 in runs:
        assert 1 <= b - a + 1 <= 3
        for k in range(a, b + 1):
            done[(cwd, k)] = done.get((cwd, k), 0) + 1
    assert len(done) == 8 + 8 + 4 and set(done.values()) == {1}
    # both devices used, neither above its 10 GB budget at any time
    assert {r[3] for r in runs} == {0, 1}
    for dev in (0, 1):
        assert _max_concurrent_gb(runs, dev) <= 10.0 + 1e-9
    assert max(_max_concurrent_gb(runs, d) for d in (0, 1)) > 5.0   # instances did overlap


def test_finished_steps_are_skipped(tmp_path, fake):
    exe, log = fake
    p = _project(tmp_path, "p", {1: {"steps": [[k, 100.0 * k, 1.0] for k in range(1, 7)]}})
    src = p / "NumCalc" / "source_1"
    for k in (1, 2, 5):
        (src / "be.out" / ("be.%d" % k)).mkdir(parents=True)
        (src / "be.out" / ("be.%d" % k) / "pEvalGrid").write_text("x\n")
    (src / "NC5-5.out").write_text("Start\n")   # step 5 did not end: run again
    mn.manage_numcalc(str(tmp_path), exe, max_hbm_load=4.0, steps_per_instance=10, wait_time=0.02)
    ranges = sorted((a, b) for _, a, b, *_ in _runs(log))
    assert ranges == [(3, 6)]
    all_steps, to_run = mn.check_project(str(p), exe)
    assert len(all_steps) == 6 and len(to_run) == 0


def test_step_larger_than_every_device_stops(tmp_path, fake):
    exe, log = fake
    _project(tmp_path, "p", {1: {"steps": [[1, 100.0, 2.0], [2, 200.0, 30.0]]}})
    with pytest.raises(ValueError, match="not sufficient device memory"):
        mn.manage_numcalc(str(tmp_path), exe, max_hbm_load=20.0, wait_time=0.02)
    assert _runs(log) == []


def test_unfinished_instances_are_reported(tmp_path, fake):
    exe, log = fake
    _project(tmp_path, "p", {1: {"steps": [[k, 100.0 * k, 1.0] for k in range(1, 5)], "fail": [3]}})
    with pytest.raises(ValueError, match="source 1 step 3"):
        mn.manage_numcalc(str(tmp_path), exe, max_hbm_load=4.0, steps_per_instance=1, wait_time=0.02)
    # the other steps finished
    src = tmp_path / "p" / "NumCalc" / "source_1"
    assert all(mn.step_finished(str(src), k) for k in (1, 2, 4))


def test_instances_and_estimates_fallback(tmp_path):
    rows = np.array([[1, 1, 100, 1.0], [1, 2, 200, 2.0], [1, 4, 400, 1.5], [2, 1, 100, 0.5],
                     [1, 5, 500, 1.0], [1, 6, 600, 1.0]], float)
    inst = mn.make_instances(rows, 2)
    assert inst.tolist() == [[1, 1, 2, 2.0], [1, 4, 5, 1.5], [1, 6, 6, 1.0], [2, 1, 1, 0.5]]
    # host-RAM estimates when MemoryGPU.txt is absent (the reference NumCalc)
    src = tmp_path / "p" / "NumCalc" / "source_1"
    src.mkdir(parents=True)
    (src / "Memory.txt").write_text("1 100 2.5\n2 200 2.5\n")
    exe = tmp_path / "true_numcalc"
    exe.write_text("#!/bin/sh\nexit 0\n")
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    all_steps, to_run = mn.check_project(str(tmp_path / "p"), str(exe))
    assert np.allclose(all_steps[:, 3], 2.5 + mn.CONTEXT_GB) and len(to_run) == 2
