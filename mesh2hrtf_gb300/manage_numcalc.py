"""Run NumCalc on Mesh2HRTF project folders with GPU-memory admission.

The reference's scheduler (``mesh2hrtf/NumCalc/manage_numcalc.py:10-398``)
starts one NumCalc process per frequency step whenever enough *host RAM*
(estimated by ``NumCalc -estimate_ram`` into ``Memory.txt``) and CPU are
free.  With the GPU build every step's matrix lives in device memory, so the
scarce resource is HBM, and a process per step would spend more time
creating its CUDA context and uploading the mesh than solving (a 20k-element
step solves in ~40 ms).  This scheduler keeps the reference's interface,
project discovery, log file and completion rule, and changes what it gates
on and what an instance is:

* The drop-in's ``-estimate_ram`` also writes ``MemoryGPU.txt`` (same
  ``"step frequency GB"`` lines) with its device footprint per process:
  solver (matrix, Krylov basis, preconditioner), mesh tables, evaluation
  points and a CUDA context.  Without that file (the reference NumCalc) the
  host-RAM estimate of ``Memory.txt`` stands in.
* An instance is a run of consecutive unfinished steps of one source
  (``NumCalc -istart a -iend b``, at most ``steps_per_instance`` steps); its
  footprint is the largest of its steps'.
* Instances start while the footprints of the running ones on a device,
  times ``hbm_safety_factor``, stay within that device's budget
  (``max_hbm_load`` GB, by default 90 % of its memory); several GPUs take
  instances on the device with the most room (``NUMCALC_GB300_DEVICE``).
  The drop-in itself also waits for device memory (``NUMCALC_GB300_WAIT_S``),
  so processes started outside this scheduler do not make it fail.

A step is finished when ``be.out/be.<step>/pEvalGrid`` exists and the newest
``NC<a>-<b>.out`` covering the step, if any, says ``End time:`` (the
reference checks ``NC<k>-<k>.out``, ``manage_numcalc.py:545-573``).

    python -m mesh2hrtf_gb300.manage_numcalc --project_path <dir> [--max_hbm_load GB]
"""
from __future__ import annotations

import argparse
import glob
import os
import re
import shutil
import subprocess
import sys
import time

import numpy as np

CONTEXT_GB = 0.6   # device memory of one process's CUDA context


# ------------------------------------------------------------------ logging
class _Log:
    def __init__(self, path):
        self.path = path

    def __call__(self, message):
        print(message)
        with open(self.path, "a", encoding="utf8", newline="\n") as fh:
            fh.write(message + "\n")

    def error(self, message, confirm_errors=False):
        with open(self.path, "a", encoding="utf8", newline="\n") as fh:
            fh.write("\n\n" + message + "\n")
        if confirm_errors:
            print(message)
            input("Press Enter to exit manage_numcalc")
            raise Exception("manage_numcalc was stopped due to an error")
        raise ValueError(message)


# ------------------------------------------------------------- projects
def find_projects(project_path):
    """One project (a folder with parameters.json) or every subfolder that
    holds ObjectMeshes/Reference (``manage_numcalc.py:133-152``)."""
    if os.path.isfile(os.path.join(project_path, "parameters.json")):
        return [project_path]
    out = []
    for sub in sorted(os.listdir(project_path)):
        if os.path.isdir(os.path.join(project_path, sub, "ObjectMeshes", "Reference")):
            out.append(os.path.join(project_path, sub))
    return out


def read_estimates(path):
    """Rows (step, frequency, GB) of a Memory.txt-style file."""
    rows = []
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if len(tok) >= 3:
                rows.append([float(tok[0]), float(tok[1]), float(tok[2])])
    return np.asarray(rows, float).reshape(-1, 3)


_NC_RANGE = re.compile(r"^NC(\d+)-(\d+)\.out$")


def _nc_outputs(source_dir):
    """(first step, last step, finished, mtime) of every NC<a>-<b>.out."""
    out = []
    for name in os.listdir(source_dir):
        m = _NC_RANGE.match(name)
        if m:
            path = os.path.join(source_dir, name)
            with open(path, encoding="utf8", errors="replace") as fh:
                done = "End time:" in fh.read()
            out.append((int(m.group(1)), int(m.group(2)), done, os.path.getmtime(path)))
    return out


def step_finished(source_dir, step, nc_outputs=None):
    """pEvalGrid written and, if a NC<a>-<b>.out covers the step, the newest
    such file ends with "End time:" (the reference's rule for NC<k>-<k>.out,
    manage_numcalc.py:558-573, extended to the ranges this scheduler runs)."""
    if not os.path.isfile(os.path.join(source_dir, "be.out", "be.%d" % step, "pEvalGrid")):
        return False
    cover = [(t, done) for a, b, done, t in (nc_outputs if nc_outputs is not None else _nc_outputs(source_dir))
             if a <= step <= b]
    return not cover or max(cover)[1]


def check_project(project, numcalc, log=None):
    """All steps and the unfinished ones of a project.

    Returns (all_steps, to_run): arrays of rows (source, step, frequency,
    device GB); runs ``numcalc -estimate_ram`` where the estimates are
    missing (``manage_numcalc.py:507-541``)."""
    sources = sorted(glob.glob(os.path.join(project, "NumCalc", "source_*")),
                     key=lambda p: int(p.rsplit("_", 1)[1]))
    all_rows, run_rows = [], []
    for src in sources:
        sid = int(src.rsplit("_", 1)[1])
        gpu_est = os.path.join(src, "MemoryGPU.txt")
        if not os.path.isfile(gpu_est):
            if log:
                log("Obtaining memory estimates for %s" % src)
            subprocess.run([numcalc, "-estimate_ram"], cwd=src, stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL, check=True)
        if os.path.isfile(gpu_est):
            est = read_estimates(gpu_est)
        else:   # host-RAM estimate of the dense FP64 system, plus a context
            est = read_estimates(os.path.join(src, "Memory.txt"))
            est[:, 2] += CONTEXT_GB
        ncs = _nc_outputs(src)
        for step, freq, gb in est:
            row = [sid, int(step), freq, gb]
            all_rows.append(row)
            if not step_finished(src, int(step), ncs):
                run_rows.append(row)
    return np.asarray(all_rows, float).reshape(-1, 4), np.asarray(run_rows, float).reshape(-1, 4)


def make_instances(to_run, steps_per_instance):
    """Runs of consecutive unfinished steps per source, cut into instances
    of at most steps_per_instance steps: rows (source, first, last, GB)."""
    out = []
    for sid in np.unique(to_run[:, 0]).astype(int):
        rows = to_run[to_run[:, 0] == sid]
        rows = rows[np.argsort(rows[:, 1])]
        start = 0
        for k in range(1, len(rows) + 1):
            if k == len(rows) or rows[k, 1] != rows[k - 1, 1] + 1 or k - start == steps_per_instance:
                chunk = rows[start:k]
                out.append([sid, int(chunk[0, 1]), int(chunk[-1, 1]), float(chunk[:, 3].max())])
                start = k
    return np.asarray(out, float).reshape(-1, 4)


# ------------------------------------------------------------- devices
def device_budgets(devices=None, max_hbm_load=None):
    """{device: GB the scheduler may fill}.  max_hbm_load (GB per device)
    wins; otherwise 90 % of each device's memory from nvidia-smi, or from
    the library (in a child process, so that no context stays open here)."""
    if max_hbm_load is not None:
        return {d: float(max_hbm_load) for d in (devices if devices is not None else [0])}
    totals = {}
    smi = shutil.which("nvidia-smi")
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if smi:
        r = subprocess.run([smi, "--query-gpu=index,memory.total", "--format=csv,noheader,nounits"],
                           capture_output=True, text=True)
        if r.returncode == 0:
            phys = {}
            for line in r.stdout.strip().splitlines():
                i, mib = [t.strip() for t in line.split(",")]
                phys[int(i)] = float(mib) * 1048576 / 1e9
            if vis and all(t.strip().isdigit() for t in vis.split(",")):
                order = [int(t) for t in vis.split(",")]
                totals = {k: phys[p] for k, p in enumerate(order) if p in phys}
            else:
                totals = phys
    if not totals:
        code = ("from mesh2hrtf_gb300 import capi; f, t = capi.device_memory(0); print(t)")
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                           cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        if r.returncode != 0:
            raise RuntimeError("no device found; pass max_hbm_load")
        totals = {0: float(r.stdout.split()[-1]) / 1e9}
    if devices is not None:
        totals = {d: totals[d] for d in devices}
    return {d: 0.9 * gb for d, gb in totals.items()}


def default_numcalc():
    from . import build
    return build.NUMCALC_BIN if os.path.isfile(build.NUMCALC_BIN) else "NumCalc"


# ------------------------------------------------------------- scheduler
def manage_numcalc(project_path=None, numcalc_path=None, max_hbm_load=None, hbm_safety_factor=1.05,
                   max_instances=None, devices=None, steps_per_instance=20, wait_time=0.5,
                   starting_order="alternate", confirm_errors=False):
    """Run every unfinished frequency step of the projects under project_path.

    Parameters follow the reference's manage_numcalc; max_hbm_load (GB per
    device) and hbm_safety_factor replace max_ram_load and
    ram_safety_factor, max_cpu_load has no counterpart, max_instances caps
    the processes over all devices (default two per device), devices lists
    the CUDA devices to use, steps_per_instance bounds the steps one
    process solves, wait_time is the polling interval in seconds."""
    project_path = os.path.abspath(project_path or os.getcwd())
    stamp = time.strftime("%Y_%m_%d_%H-%M-%S", time.localtime())
    log = _Log(os.path.join(project_path, "manage_numcalc_%s.txt" % stamp))
    numcalc = numcalc_path or default_numcalc()
    if starting_order not in ("alternate", "high", "low"):
        log.error("starting_order must be 'alternate', 'high' or 'low'", confirm_errors)
    projects = find_projects(project_path)
    if not projects:
        log.error("manage_numcalc could not detect any Mesh2HRTF projects at project_path=%s" % project_path,
                  confirm_errors)
    budgets = device_budgets(devices, max_hbm_load)
    devs = sorted(budgets)
    if max_instances is None:
        max_instances = 2 * len(devs)
    log("\nStarting manage_numcalc with the following arguments [%s]\n" % time.strftime("%b %d %Y, %H:%M:%S")
        + "-" * 60 + "\n"
        + "project_path: %s\nnumcalc_path: %s\n" % (project_path, numcalc)
        + "devices: %s (budget %s GB)\n" % (devs, ", ".join("%.2f" % budgets[d] for d in devs))
        + "hbm_safety_factor: %s\nmax_instances: %d\nsteps_per_instance: %d\nstarting_order: %s\n"
        % (hbm_safety_factor, max_instances, steps_per_instance, starting_order))

    running = []   # (Popen, device, GB, label, log handle)

    def reap():
        keep = []
        for proc, dev, gb, label, fh in running:
            rc = proc.poll()
            if rc is None:
                keep.append((proc, dev, gb, label, fh))
                continue
            fh.close()
            if rc != 0:
                log("%s exited with code %d" % (label, rc))
        running[:] = keep

    for pi, project in enumerate(projects):
        all_steps, to_run = check_project(project, numcalc, log)
        name = os.path.basename(project)
        if not len(to_run):
            log("'%s' is already complete" % name)
            continue
        inst = make_instances(to_run, max(1, int(steps_per_instance)))
        inst = inst[np.argsort(inst[:, 3], kind="stable")]
        log("\nStarted '%s' project (%d/%d): %d/%d unfinished steps in %d instances"
            % (name, pi + 1, len(projects), len(to_run), len(all_steps), len(inst)))
        if inst[-1, 3] * hbm_safety_factor > max(budgets.values()):
            log.error("Stop - not sufficient device memory for this project: source %d steps %d-%d need "
                      "%.2f GB, the largest device budget is %.2f GB"
                      % (inst[-1, 0], inst[-1, 1], inst[-1, 2], inst[-1, 3] * hbm_safety_factor,
                         max(budgets.values())), confirm_errors)
        if starting_order != "low":
            inst = inst[::-1]
        total = len(inst)
        while len(inst):
            reap()
            used = {d: sum(gb for _, dv, gb, _, _ in running if dv == d) for d in devs}
            placed = None
            if len(running) < max_instances:
                for idx in range(len(inst)):
                    need = inst[idx, 3] * hbm_safety_factor
                    fits = [d for d in devs if used[d] + need <= budgets[d]]
                    if fits:
                        placed = (idx, max(fits, key=lambda d: budgets[d] - used[d]), need)
                        break
            if placed is None:
                time.sleep(wait_time)
                continue
            idx, dev, need = placed
            sid, a, b = int(inst[idx, 0]), int(inst[idx, 1]), int(inst[idx, 2])
            cwd = os.path.join(project, "NumCalc", "source_%d" % sid)
            label = "source %d steps %d-%d" % (sid, a, b)
            log("%d/%d starting instance from '%s' (%s): %s on device %d, %.2f GB of %.2f GB free"
                % (total - len(inst) + 1, total, name, time.strftime("%H:%M:%S"), label, dev, need,
                   budgets[dev] - used[dev]))
            env = dict(os.environ, NUMCALC_GB300_DEVICE=str(dev))
            fh = open(os.path.join(cwd, "NC%d-%d_log.txt" % (a, b)), "w")
            proc = subprocess.Popen([numcalc, "-istart", str(a), "-iend", str(b)], cwd=cwd, env=env,
                                    stdout=fh, stderr=subprocess.STDOUT)
            running.append((proc, dev, need, label, fh))
            inst = np.delete(inst, idx, 0)
            if starting_order == "alternate":
                inst = inst[::-1]
    log("\n... waiting for the last NumCalc instances to finish (%s)" % time.strftime("%H:%M:%S"))
    while running:
        reap()
        if running:
            time.sleep(wait_time)
    unfinished = []
    for project in projects:
        _, to_run = check_project(project, numcalc)
        for sid, step, _, _ in to_run:
            unfinished.append("'%s': source %d step %d" % (os.path.basename(project), sid, step))
    if unfinished:
        log.error("\nThe following instances did not finish\n" + "-" * 38 + "\n" + "\n".join(unfinished),
                  confirm_errors)
    log("\nAll NumCalc projects finished at %s" % time.strftime("%b %d %Y, %H:%M:%S"))
    return log.path


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0],
                                 formatter_class=argparse.ArgumentDefaultsHelpFormatter)
    ap.add_argument("--project_path", default=None)
    ap.add_argument("--numcalc_path", default=None)
    ap.add_argument("--max_hbm_load", default=None, type=float, help="GB per device")
    ap.add_argument("--hbm_safety_factor", default=1.05, type=float)
    ap.add_argument("--max_instances", default=None, type=int)
    ap.add_argument("--devices", default=None, help="comma-separated CUDA device indices")
    ap.add_argument("--steps_per_instance", default=20, type=int)
    ap.add_argument("--wait_time", default=0.5, type=float)
    ap.add_argument("--starting_order", default="alternate", choices=["alternate", "high", "low"])
    ap.add_argument("--confirm_errors", action="store_true")
    a = ap.parse_args(argv)
    devs = None if a.devices is None else [int(t) for t in a.devices.split(",")]
    manage_numcalc(a.project_path, a.numcalc_path, a.max_hbm_load, a.hbm_safety_factor, a.max_instances,
                   devs, a.steps_per_instance, a.wait_time, a.starting_order, a.confirm_errors)


if __name__ == "__main__":
    main()
