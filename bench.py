"""Benchmark: frequency solves/s of the GPU BEM on the head-like workload.

Workload (one GPU): head-like scatterer (ellipsoid 0.09/0.075/0.11 m + two
seeded Gaussian bumps, 20480 triangles graded toward bump 1), reciprocal point
source 1 mm off bump 1, evaluation grid of 1730 points on a 1.2 m sphere,
frequencies 100 Hz .. 20 kHz in 100 Hz steps (200 solves).  One solve =
assemble A(k) and b, GMRES to a relative residual of 1e-9, project onto the
1730 points.  A step is one batch of --batch frequencies (default 16) taken
from a seeded permutation of the 200, so K steps sample the whole band.

value     mixed-precision solves/s with the mesh resident on the device; a
          step is one bem_solve_batch call over its frequencies (one solver
          per frequency on the shared mesh).
latency   p50/p99 of the same frequencies solved one at a time
          (bem_solve_frequency).
e2e       the same as value through the C ABI with host buffers: every step
          uploads the mesh and evaluation points, creates the solvers, runs
          bem_solve_batch and copies unknowns and fields back.
fp64      the plain FP64 GPU path on one batch of the same frequencies (also
          batched), with the mixed path's relative L2 boundary-pressure error
          against it.
roofline  the dominant kernel (the matrix-vector products of the solve:
          Krylov products from the fp16 copy of A, algorithmic bytes
          N^2*4 + 2*N*16 per product and system; refinement residuals from
          the complex64 matrix, N^2*8 + 2*N*16) over the CUDA-event time of
          the product launches, against the measured HBM copy bandwidth.
cpu_baseline  the FP64 C restatement of the reference path (oracle/, the
          "port") on the host cores, on a bounded sample: 2048 rows of the
          assembly, the dense matrix-vector product of those rows and 256
          evaluation points at 10 kHz, scaled to one full solve.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RHO, C0 = 1.21, 343.0
N_TRI = 20480
SEED = 20261204
METRIC = "freq solves/s at <=1e-4 rel err, mixed vs plain FP64 GPU BEM; p50/p99 latency"
# DRAM bytes (read + write) of one Krylov product from the fp16 copy at
# N = 20480, measured by ncu on this workload (k_mv_tma launch list)
MV_TRAFFIC = 1.6863e9


def workload():
    from mesh2hrtf_gb300 import workloads

    return workloads.head_workload(SEED)


def freq_desc(capi, n, fr, src):
    k = 2 * np.pi * fr / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * fr)    # NC.inp amplitude 0.1, as mesh2input writes it
    return capi.Frequency(k, n, point_sources=src, point_amps=[amp])


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        return False

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            p = [x.strip() for x in ln.split(",")]
            try:
                sm.append(float(p[0]))
                smax = max(smax, float(p[1]))
            except (ValueError, IndexError):
                continue
            for nm, val in zip(names, p[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- cpu port
def cpu_port_solve_seconds(v, f, src, pts, fr, iters, threads, rows=2048, n_pts=256):
    """Seconds for one full solve of the FP64 C restatement, from a sample."""
    from oracle import oracle_py as op

    om = op.OracleMesh(v, f)
    k = 2 * np.pi * fr / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * fr)
    of = op.OracleFreq(k, src, [amp])
    n = len(f)
    r0 = 0
    t0 = time.perf_counter()
    A, b = op.assemble(om, of, rows=(r0, r0 + rows), nthreads=threads)
    t_asm = (time.perf_counter() - t0) * n / rows
    x = np.ones(n, np.complex128)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        A @ x
    t_mv = (time.perf_counter() - t0) / reps * n / rows
    phi, vel = op.boundary_fields(om, np.ones(n, np.complex128) * 1e-3)
    sel = pts[:: max(len(pts) // n_pts, 1)][:n_pts]
    t0 = time.perf_counter()
    op.project(om, of, phi, vel, sel, nthreads=threads)
    t_proj = (time.perf_counter() - t0) * len(pts) / len(sel)
    total = t_asm + iters * t_mv + t_proj
    return total, {"assemble_s": t_asm, "matvec_s": t_mv, "iterations": iters, "project_s": t_proj}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    v, f, src, pts, freqs = workload()
    n = len(f)
    cfg = {"workload": "head-like ellipsoid with 2 bumps, %d triangles, 1730-point 1.2 m grid, "
                       "point source 1 mm off bump 1, 100 Hz-20 kHz step 100 Hz" % n,
           "n_elements": n, "n_eval_points": len(pts), "frequencies": 200, "batch_per_step": args.batch,
           "gmres_tol": 1e-9, "restart": 60, "l2": "inputs larger than L2 (3.4 GB matrix per solve)",
           "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        threads = cpu_threads()
        vals, details = [], None
        for s in range(args.warmup + args.steps):
            fr = float(freqs[s % len(freqs)])
            t, det = cpu_port_solve_seconds(v, f, src, pts, fr, iters=100, threads=threads, rows=512, n_pts=64)
            if s >= args.warmup:
                vals.append(1.0 / t)
                details = det
        val = float(np.mean(vals))
        line = {"metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 / val, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg, "impl": "reference",
                "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": "port",
                                 "sample": "FP64 C restatement of NumCalc's TBEM path (oracle/bem_oracle.c); "
                                           "per step 512 assembly rows + dense matvec of those rows + 64 "
                                           "evaluation points at one frequency, scaled to the full "
                                           "20480-unknown solve with 100 Krylov iterations",
                                 "breakdown": details},
                "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    from mesh2hrtf_gb300 import capi

    dev = local if torch.cuda.device_count() > 1 else 0
    torch.cuda.set_device(dev)
    lib = capi.load()
    mesh = capi.Mesh(v, f, device=dev)
    B = args.batch
    # one solver per frequency of a step, all on the resident mesh; a step is
    # one bem_solve_batch call (assembly, lockstep GMRES and projection of the
    # B frequencies together)
    solvers = [capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000) for _ in range(B)]

    # each rank takes its own slice of the permuted frequency list
    def batch_freqs(step):
        base = (step * world + rank) * B
        return [float(freqs[(base + b) % len(freqs)]) for b in range(B)]

    infos, batch_ms = [], []

    def run_step(step, record):
        Fs = [freq_desc(capi, n, fr, src) for fr in batch_freqs(step)]
        res = capi.solve_batch(solvers, Fs, [pts] * B)
        if record:
            infos.append([r[3] for r in res])

    for s in range(args.warmup):
        run_step(s, False)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.bem_kernel_launches()
    with ClockSampler(dev) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        t0 = time.perf_counter()
        for s in range(args.warmup, args.warmup + args.steps):
            run_step(s, True)
        ev1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = lib.bem_kernel_launches() - launches0
    elapsed = ev0.elapsed_time(ev1) / 1000.0
    if dist:
        t = torch.tensor([elapsed], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t[0])
    total_solves = args.steps * B * world
    value = total_solves / elapsed

    # roofline of the dominant kernel: the matrix-vector products.  Each
    # launch of the batched product covers every system still iterating; its
    # bytes are counted per system and product (Krylov products read the fp16
    # copy, N^2*4 + 2*N*16; refinement residuals the complex64 matrix,
    # N^2*8 + 2*N*16), its time is the CUDA-event time of the launches inside
    # the iteration bodies.
    bytes_krylov = n * n * 4.0 + 2 * n * 16.0
    bytes_resid = n * n * 8.0 + 2 * n * 16.0
    mv_ms = sum(step[0]["matvec_ms"] for step in infos)
    n_mv = sum(i["n_matvec"] for step in infos for i in step)
    n_kry = sum(i["iterations"] for step in infos for i in step)
    mv_bytes = bytes_krylov * n_kry + bytes_resid * (n_mv - n_kry)
    achieved = mv_bytes / (mv_ms / 1000.0) / 1e9 if mv_ms > 0 else None
    asm_ms = sum(step[0]["assemble_ms"] for step in infos)
    solve_ms = sum(step[0]["solve_ms"] for step in infos)
    proj_ms = sum(step[0]["project_ms"] for step in infos)
    n_solves = len(infos) * B
    iters = [i["iterations"] for step in infos for i in step]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    for sv in solvers:
        sv.close()

    # latency: the same frequencies solved one at a time (bem_solve_frequency)
    lat = []
    single = capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000)
    for s in range(args.warmup, args.warmup + args.steps):
        for fr in batch_freqs(s):
            F = freq_desc(capi, n, fr, src)
            t1 = time.perf_counter()
            single.solve_frequency(F, pts)
            lat.append(time.perf_counter() - t1)
    single.close()

    # end to end through the C ABI with host buffers: per step the mesh and
    # the evaluation points go up, B solvers are created, bem_solve_batch
    # runs, unknowns and fields come back
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 2))
    for s in range(args.warmup, args.warmup + e2e_steps):
        m2 = capi.Mesh(v, f, device=dev)
        s2 = [capi.Solver(m2, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000) for _ in range(B)]
        capi.solve_batch(s2, [freq_desc(capi, n, fr, src) for fr in batch_freqs(s)], [pts] * B)
        for sv in s2:
            sv.close()
        m2.close()
    torch.cuda.synchronize()
    e2e_val = e2e_steps * B / (time.perf_counter() - t0)
    # bem_mesh_create uploads 20 FP64 + 30 FP32/int rows per element; every
    # solve uploads the evaluation points and the frequency data, and returns
    # the unknowns (complex128), potentials and gradients (4 x complex128)
    h2d = n * (20 * 8 + 30 * 4) + B * (pts.nbytes + 16 + 24)
    d2h = B * (n * 16 + len(pts) * 16 * 4)

    # FP64 GPU path on one batch (also batched), and the mixed path's error
    # against it
    frs = batch_freqs(args.warmup)
    Fs = [freq_desc(capi, n, fr, src) for fr in frs]
    s64 = [capi.Solver(mesh, precision=capi.PREC_FP64, tol=1e-9, max_iter=3000) for _ in range(B)]
    capi.solve_batch(s64[:1], Fs[:1], [pts])   # warm-up of the FP64 engine
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    r64 = capi.solve_batch(s64, Fs, [pts] * B)
    t64 = time.perf_counter() - t1
    for sv in s64:
        sv.close()
    smx = [capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000) for _ in range(B)]
    rmx = capi.solve_batch(smx, Fs, [pts] * B)
    for sv in smx:
        sv.close()
    errs = [float(np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0])) for a, b in zip(rmx, r64)]
    fp64_val = B / t64

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1000.0, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (fp16 Krylov copy of A, complex64 residual matrix, FP64-accurate refinement residuals)",
        "data": "synthetic", "config": cfg,
        "latency_ms": {"p50": float(np.percentile(lat, 50) * 1000), "p99": float(np.percentile(lat, 99) * 1000),
                       "mode": "one solve at a time (bem_solve_frequency), same frequencies"},
        "fp64_gpu": {"value": fp64_val, "unit": "solves/s", "frequencies": frs, "mode": "bem_solve_batch of %d" % B,
                     "speedup_mixed_over_fp64": value / fp64_val,
                     "mixed_rel_l2_boundary_err_max": max(errs)},
        "stage_ms_per_solve": {"assemble": asm_ms / n_solves, "solve": solve_ms / n_solves,
                               "project": proj_ms / n_solves, "matvec": mv_ms / n_solves,
                               "iterations": float(np.mean(iters))},
        "roofline": {"bound": "hbm", "kernel": "k_mv_tma (batched A x: fp16 Krylov copy, complex64 residuals)",
                     "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if achieved else None,
                     "traffic": MV_TRAFFIC if n == N_TRI else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per Krylov k_mv_tma<0> "
                                       "launch from the fp16 copy, same N (profiles/k_mv_tma_fp16_head20480.md)",
                     "bytes_per_krylov_product": bytes_krylov, "bytes_per_residual_product": bytes_resid,
                     "krylov_products": n_kry, "residual_products": n_mv - n_kry,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "wall_s": wall,
    }
    if rank == 0:
        threads = cpu_threads()
        it_mean = int(round(np.mean(iters)))
        t_cpu, det = cpu_port_solve_seconds(v, f, src, pts, 10000.0, it_mean, threads)
        line["cpu_baseline"] = {
            "value": 1.0 / t_cpu, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": "FP64 C restatement of NumCalc's TBEM path (oracle/bem_oracle.c) at 10 kHz: 2048 "
                      "assembly rows, the dense complex128 matvec of those rows and 256 of the 1730 "
                      "evaluation points, scaled to one 20480-unknown solve with the GPU run's mean "
                      "iteration count (%d)" % it_mean,
            "breakdown": det}
        print(json.dumps(line))
    mesh.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
