"""Benchmark: frequency solves/s of the GPU BEM on the head-like workload.

Workload (one GPU): head-like scatterer (ellipsoid 0.09/0.075/0.11 m + two
seeded Gaussian bumps, 20480 triangles graded toward bump 1), reciprocal point
source 1 mm off bump 1, evaluation grid of 1730 points on a 1.2 m sphere,
frequencies 100 Hz .. 20 kHz in 100 Hz steps (200 solves).  One solve =
assemble A(k) and b, solve to a relative residual of 1e-9, project onto the
1730 points.  A GPU step is one batch of --batch frequencies (default 16)
taken from a seeded permutation of the 200, so K steps sample the band.

value     mixed-precision solves/s with the mesh resident on the device; a
          step is one bem_solve_batch call over its frequencies (one solver
          per frequency on the shared mesh).  The Krylov products read the
          block low-rank copy of A by default (--krylov-copy blr; fp16 and
          complex64 select the other copies).
e2e       the same K steps through the C ABI with host buffers: every step
          uploads the mesh and evaluation points, creates the solvers, runs
          bem_solve_batch and copies unknowns and fields back.
latency   p50/p99 of the same frequencies solved one at a time
          (bem_solve_frequency) with the library's default fp16 Krylov copy,
          the faster one for a single solve.
fp64_gpu  the plain FP64 GPU path on the first timed batch (the same 16
          frequencies, also one bem_solve_batch), against the mixed time of
          that batch, and the mixed path's relative L2 error against it.
roofline  the dominant kernel (the matrix-vector products of the solve) over
          the CUDA-event time of the product launches, against the measured
          HBM copy bandwidth; roofline.stages gives every stage of a solve a
          roofline time from its algorithmic work and the measured peaks
          (HBM copy, and the FP32 FMA / special-function / FP64 FMA issue
          rates from bem_measure_issue_peaks) and the end-to-end fraction.
serving   a seeded Poisson stream of solve requests (perturbed ellipsoids of
          2k-40k triangles, 0.1-20 kHz, 1730 points) through bem_server_*:
          first all at once (capacity), then at 85 % of that rate; FP64 on
          the first requests of the same stream.
cpu_baseline  the FP64 C restatement of NumCalc's path (oracle/, the
          "port": assembly, NumCalc's CGS with threshold ILU to 1e-9,
          projection) on all host cores, one complete solve of the first
          timed frequency.

--impl reference times the same port, complete solves only (one frequency
per step, every row, every point), with as many steps as fit a time budget.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RHO, C0 = 1.21, 343.0
N_TRI = 20480
SEED = 20261204
METRIC = "freq solves/s at <=1e-4 rel err, mixed vs plain FP64 GPU BEM; p50/p99 latency"
# DRAM bytes (read + write) of one Krylov product at N = 20480 measured by
# ncu on this workload, the algorithmic bytes of the same launch, and the
# capture it comes from, per Krylov copy
MV_TRAFFIC = {
    "fp16": (1.6863e9, 1.6784e9, "ncu dram__bytes_read.sum + dram__bytes_write.sum per Krylov k_mv_tma<0> launch "
                                 "from the fp16 copy, 5 kHz (profiles/k_mv_tma_fp16_head20480.md)"),
    "blr": (4.0315e9, 4.1127e9, "ncu dram__bytes_read.sum + dram__bytes_write.sum per busy k_mv_blr launch of the "
                                "bench's first batch of 16, against that batch's algorithmic bytes per launch "
                                "(bem_krylov_copy_info bytes x Krylov steps / 48 launches; "
                                "profiles/k_mv_blr_head20480.md)"),
    "complex64": (None, None, "not captured"),
}
COPY_DESC = {"blr": "a block low-rank Krylov copy (fp16 factors and fp16 dense blocks)",
             "fp16": "an fp16 Krylov copy", "complex64": "no Krylov copy"}
ROOF_KERNEL = {"blr": "k_mv_blr (Krylov products from the block low-rank copy) + k_mv_tma (complex64 residuals)",
               "fp16": "k_mv_tma (batched A x: fp16 Krylov copy, complex64 residuals)",
               "complex64": "k_mv_tma (batched A x from the complex64 matrix)"}
# Fixed work accounting of one kernel evaluation (one quadrature point of one
# (collocation point, element) pair, NC_RegularIntegration,
# NC_EquationSystem.cpp:1600-1728): r, 1/r and the phase (sin, cos, rsqrt:
# 3 special-function operations) and 48 FP32 operations for G, dG/dn_y and
# the hypersingular kernel E combined in Burton-Miller form; a projection
# point (NC_IntegrationTBEM, NC_PostProcessing.cpp:1217-1322) with potential
# and gradient takes 3 special-function and 64 FP32 operations.
ASM_FP32_PER_EVAL, ASM_SFU_PER_EVAL = 48, 3
PROJ_FP32_PER_EVAL, PROJ_SFU_PER_EVAL = 64, 3
# Points of the cheapest rule NumCalc applies to a triangle pair (order 2,
# NC_ComputeGausseanPoints, NC_3dFunctions.cpp:455-530): a lower bound of
# the quadrature work of every pair
MIN_POINTS = 4


def workload(mesh_n=32):
    from mesh2hrtf_gb300 import workloads

    return workloads.head_workload(SEED, mesh_n)


def freq_desc(capi, n, fr, src):
    k = 2 * np.pi * fr / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * fr)    # NC.inp amplitude 0.1, as mesh2input writes it
    return capi.Frequency(k, n, point_sources=src, point_amps=[amp])


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks, throttle reasons and utilisation sampled during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

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
        sm, smax, util, reasons = [], 0.0, [], set()
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
            try:
                util.append(float(p[8]))
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm),
                "util_mean_pct": float(np.mean(util)) if util else None}


# ------------------------------------------------------------- cpu port
def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_port_solve(om, src, pts, fr, threads):
    """One complete solve with the FP64 restatement of NumCalc's path:
    assembly of every row, NumCalc's CGS with threshold ILU (scanning degree
    0) to 1e-9, projection onto every point.  Returns (seconds, breakdown)."""
    from oracle import oracle_py as op

    k = 2 * np.pi * fr / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * fr)
    of = op.OracleFreq(k, src, [amp])
    t0 = time.perf_counter()
    A, b = op.assemble(om, of, nthreads=threads)
    t1 = time.perf_counter()
    x, it, err, direct, stg = op.solve_cgs(A, b, precond=0, scan=0, niter_max=250, tol=1e-9,
                                            nthreads=threads, overwrite=True)
    del A
    t2 = time.perf_counter()
    phi, vel = op.boundary_fields(om, x)
    op.project(om, of, phi, vel, pts, nthreads=threads)
    t3 = time.perf_counter()
    return t3 - t0, {"freq_hz": fr, "assemble_s": t1 - t0, "ilu_s": float(stg[0]), "cgs_s": float(stg[1]),
                     "cgs_iterations": it, "cgs_rel_err": err, "direct_fallback": bool(direct),
                     "project_s": t3 - t2, "total_s": t3 - t0}


def cpu_warmup(om, src, pts, threads):
    """A bounded sample (64 rows, 16 points) that pages the port in."""
    from oracle import oracle_py as op

    of = op.OracleFreq(2 * np.pi * 1000.0 / C0, src, [1e-3 + 0j])
    op.assemble(om, of, rows=(0, 64), nthreads=threads)
    n = om.n
    phi, vel = op.boundary_fields(om, np.full(n, 1e-3, np.complex128))
    op.project(om, of, phi, vel, pts[:16], nthreads=threads)


PORT_SAMPLE = ("FP64 C restatement of NumCalc's TBEM path (oracle/bem_oracle.c): assembly of all %d rows, "
               "NumCalc's CGS with threshold ILU (scanning degree 0, NC_CommonFunctions.cpp:1066-1721; "
               "bit-identical to the reference's CGS on its fixtures) to 1e-9, projection onto all %d points; "
               "complete solves, no scaling. Single-threaded it runs at 0.46x the reference NumCalc's wall "
               "time on the 5120-triangle head (oracle/port_vs_reference.py)")


# ------------------------------------------------------------- rooflines
def stage_rooflines(n, m_pts, peaks, hbm, info_steps, value, copy="fp16"):
    """Roofline time per solve of every stage from its algorithmic work and
    the measured peaks, against the measured stage times (ms per solve)."""
    fp32, sfu = peaks["fp32_fma_per_s"], peaks["sfu_per_s"]
    solves = sum(len(s) for s in info_steps)
    it = np.mean([i["iterations"] for s in info_steps for i in s])
    nmv = np.mean([i["n_matvec"] for s in info_steps for i in s])
    cyc = np.mean([i["restarts"] for s in info_steps for i in s])
    act = {k: sum(s[0][k] for s in info_steps) / solves for k in ("assemble_ms", "solve_ms", "project_ms", "matvec_ms")}
    act["nonproduct_ms"] = act["solve_ms"] - act["matvec_ms"]
    ev_asm = MIN_POINTS * float(n) * n
    t_asm = max(ev_asm * ASM_FP32_PER_EVAL / fp32, ev_asm * ASM_SFU_PER_EVAL / sfu, n * n * 8.0 / (hbm * 1e9))
    by_res = n * n * 8.0 + 2 * n * 16.0
    kry = sum(i["krylov_bytes"] * i["iterations"] for s in info_steps for i in s) / solves
    t_mv = (kry + (nmv - it) * by_res) / (hbm * 1e9)
    # non-product solve work: the fp16 copy (read 8, write 4 bytes per entry),
    # block inverses (N/128 blocks, 8*128^3 FP32 operations each), per
    # preconditioner application the 1024-wide windows (fp16) and X twice,
    # and the Arnoldi passes (two Gram-Schmidt passes over the basis: reads
    # of (k+1) complex64 vectors for the dots and for the update)
    papp = it + cyc
    # the copies: fp16 split 12 B per entry; the block low-rank copy adds one
    # full read of A by the probe check (8 B per entry)
    copy_b = {"fp16": 12.0, "blr": 20.0, "complex64": 0.0}[copy]
    by_np = n * n * copy_b + papp * (n * 1024 * 4.0 + 2 * n * 128 * 8.0)
    steps_per_cycle = it / max(cyc, 1.0)
    by_np += cyc * sum(4.0 * (k + 1) * n * 8.0 for k in range(int(round(steps_per_cycle))))
    t_np = by_np / (hbm * 1e9) + (n / 128.0) * 8 * 128.0 ** 3 / fp32
    ev_proj = MIN_POINTS * float(m_pts) * n
    t_proj = max(ev_proj * PROJ_FP32_PER_EVAL / fp32, ev_proj * PROJ_SFU_PER_EVAL / sfu)
    stages = [
        {"stage": "assembly (k_far, k_near, k_rhs)", "bound": "fp32 issue",
         "roof_ms": t_asm * 1e3, "actual_ms": act["assemble_ms"],
         "work": "%d-point rule on every pair (lower bound): %.3g evaluations x (%d FP32 + %d SFU); N^2*8 B written"
                 % (MIN_POINTS, ev_asm, ASM_FP32_PER_EVAL, ASM_SFU_PER_EVAL)},
        {"stage": "products (%s)" % ROOF_KERNEL[copy], "bound": "hbm", "roof_ms": t_mv * 1e3,
         "actual_ms": act["matvec_ms"],
         "work": "%.1f Krylov products (%.3g B each, mean) + %.1f complex64 residual products (N^2*8 B)"
                 % (it, kry / max(it, 1e-9), nmv - it)},
        {"stage": "other solve work (Krylov copy, block inverses, preconditioner, Arnoldi, cycle ends)",
         "bound": "hbm", "roof_ms": t_np * 1e3, "actual_ms": act["nonproduct_ms"],
         "work": "N^2*%g B Krylov copy + %.1f preconditioner applications x (N*1024*4 + 2*N*128*8) B + "
                 "Gram-Schmidt passes + N/128 x 8*128^3 FP32 operations%s"
                 % (copy_b, papp, "; the cross approximation's row and column reads are not counted"
                    if copy == "blr" else "")},
        {"stage": "projection (k_fields, k_project_pts, k_project_sum)", "bound": "fp32 issue",
         "roof_ms": t_proj * 1e3, "actual_ms": act["project_ms"],
         "work": "%.3g evaluations x (%d FP32 + %d SFU)" % (ev_proj, PROJ_FP32_PER_EVAL, PROJ_SFU_PER_EVAL)},
    ]
    for s in stages:
        s["frac"] = s["roof_ms"] / s["actual_ms"] if s["actual_ms"] > 0 else None
    roof = sum(s["roof_ms"] for s in stages)
    actual = 1000.0 / value
    return stages, {"roof_ms_per_solve": roof, "actual_ms_per_solve": actual, "frac": roof / actual,
                    "note": "actual = 1000 / value: batched wall time per solve, host gaps included"}


# ---------------------------------------------------------------- serving
def serving_leg(dev, n_requests=200, n_fp64=12):
    from mesh2hrtf_gb300 import capi, meshes, stream, workloads

    reqs = workloads.serving_stream(n_requests, 1.0, n_min=2000, n_max=40000)
    pts = meshes.equal_angle_grid(1.2, 5.0, 24)
    handles = [capi.Mesh(r["nodes"], r["elems"], device=dev) for r in reqs]
    budget = 160e9
    # capacity: every request at t = 0
    for r in reqs:
        r["arrival"] = 0.0
    _, cap = stream.serve(reqs, handles, pts, capi.PREC_MIXED, budget, 0)
    rate = 0.85 * cap["throughput_per_s"]
    arr = np.cumsum(np.random.default_rng(workloads.SEED_STREAM).exponential(1.0 / rate, size=n_requests))
    for r, t in zip(reqs, arr - arr[0]):
        r["arrival"] = float(t)
    with ClockSampler(dev) as clk:
        out_mx, mx = stream.serve(reqs, handles, pts, capi.PREC_MIXED, budget, 0)
    util = clk.summary().get("util_mean_pct")
    out_64, d64 = stream.serve(reqs[:n_fp64], handles[:n_fp64], pts, capi.PREC_FP64, budget, 0)
    errs = [float(np.linalg.norm(a["x"] - b["x"]) / np.linalg.norm(b["x"])) for a, b in zip(out_mx, out_64)]
    for h in handles:
        h.close()
    ns = np.array([len(r["elems"]) for r in reqs])
    return {
        "workload": "seeded Poisson stream of %d requests: perturbed ellipsoids %d-%d triangles (log-uniform, "
                    "mean %.0f), 0.1-20 kHz, 1730-point 1.2 m grid, 160 GB admission budget"
                    % (n_requests, ns.min(), ns.max(), ns.mean()),
        "capacity_per_s": cap["throughput_per_s"], "rate_per_s": rate,
        "mixed": mx, "gpu_busy": {"nvidia_smi_util_mean_pct": util,
                                  "offered_load": rate / cap["throughput_per_s"]},
        "fp64": dict(d64, note="the first %d requests of the same stream (same arrival times)" % n_fp64),
        "mixed_rel_l2_err_vs_fp64_max": max(errs),
    }


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="reference arm: complete solves are timed while their total stays within this")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--krylov-copy", default="blr", choices=["blr", "fp16", "complex64"],
                    help="the copy of A the Krylov products of the batched solves read (complex64_krylov)")
    ap.add_argument("--mesh-n", type=int, default=32,
                    help="head mesh of 20 n^2 triangles (32: the 20480-triangle workload; smaller for tests)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1 and args.impl == "gb300":
        import torch.distributed as dist
        dist.init_process_group("gloo")

    v, f, src, pts, freqs = workload(args.mesh_n)
    n = len(f)
    cfg = {"workload": "head-like ellipsoid with 2 bumps, %d triangles, 1730-point 1.2 m grid, "
                       "point source 1 mm off bump 1, 100 Hz-20 kHz step 100 Hz" % n,
           "n_elements": n, "n_eval_points": len(pts), "frequencies": 200, "batch_per_step": args.batch,
           "gmres_tol": 1e-9, "restart": 60, "l2": "inputs larger than L2 (3.4 GB matrix per solve)",
           "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle_py as op

        threads = cpu_threads()
        om = op.OracleMesh(v, f)
        for _ in range(args.warmup):
            cpu_warmup(om, src, pts, threads)
        times, details = [], []
        t_start = time.perf_counter()
        for s in range(args.steps):
            t, det = cpu_port_solve(om, src, pts, float(freqs[s % len(freqs)]), threads)
            times.append(t)
            details.append(det)
            mean = float(np.mean(times))
            if time.perf_counter() - t_start + mean > args.ref_budget_s:
                break
        total = float(np.sum(times))
        val = len(times) / total
        line = {"metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus, "steps": len(times),
                "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": total / len(times) * 1000.0,
                "solves_per_step": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
                "step": "one complete solve of one frequency (the GPU arm's step is a batch of %d); steps "
                        "lowered to what fits %.0f s of complete solves; warm-up steps are bounded samples "
                        "(64 rows, 16 points)" % (args.batch, args.ref_budget_s),
                "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": "port",
                                 "sample": PORT_SAMPLE % (n, len(pts)), "solves": details},
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
    kcopy = {"blr": capi.KRYLOV_BLR, "fp16": False, "complex64": True}[args.krylov_copy]
    solvers = [capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000, complex64_krylov=kcopy)
               for _ in range(B)]

    # each rank takes its own slice of the permuted frequency list
    def batch_freqs(step):
        base = (step * world + rank) * B
        return [float(freqs[(base + b) % len(freqs)]) for b in range(B)]

    infos, step_s, first_res = [], [], None
    # bytes one Krylov product reads, per system: the block low-rank copy's
    # own count (bem_krylov_copy_info, a 25 KB read-back per system and step,
    # inside the timed region), else the fp16 or complex64 matrix
    by_fp16, by_c64 = n * n * 4.0 + 2 * n * 16.0, n * n * 8.0 + 2 * n * 16.0

    def run_step(step, record):
        nonlocal first_res
        Fs = [freq_desc(capi, n, fr, src) for fr in batch_freqs(step)]
        t1 = time.perf_counter()
        res = capi.solve_batch(solvers, Fs, [pts] * B)
        if record:
            step_s.append(time.perf_counter() - t1)
            inf = [dict(r[3]) for r in res]
            for i, sv in zip(inf, solvers):
                i["krylov_bytes"] = (sv.krylov_copy_info()["bytes_per_product"] if args.krylov_copy == "blr"
                                     else by_fp16 if args.krylov_copy == "fp16" else by_c64)
            infos.append(inf)
            if first_res is None:
                first_res = res

    for s in range(args.warmup):
        run_step(s, False)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.bem_kernel_launches()
    # for profilers: the library's kernel launches before the timed region
    print("kernel launches before the timed region: %d" % launches0, file=sys.stderr)
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
    # the iteration bodies (events on the engine's stream).
    bytes_resid = by_c64
    mv_ms = sum(step[0]["matvec_ms"] for step in infos)
    n_mv = sum(i["n_matvec"] for step in infos for i in step)
    n_kry = sum(i["iterations"] for step in infos for i in step)
    kry_bytes = sum(i["krylov_bytes"] * i["iterations"] for step in infos for i in step)
    bytes_krylov = kry_bytes / max(n_kry, 1)   # mean over the timed products
    mv_bytes = kry_bytes + bytes_resid * (n_mv - n_kry)
    achieved = mv_bytes / (mv_ms / 1000.0) / 1e9 if mv_ms > 0 else None
    asm_ms = sum(step[0]["assemble_ms"] for step in infos)
    solve_ms = sum(step[0]["solve_ms"] for step in infos)
    proj_ms = sum(step[0]["project_ms"] for step in infos)
    n_solves = len(infos) * B
    iters = [i["iterations"] for step in infos for i in step]
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    for sv in solvers:
        sv.close()

    # end to end through the C ABI with host buffers, over the same K steps:
    # per step the mesh and the evaluation points go up, B solvers are
    # created, bem_solve_batch runs, unknowns and fields come back
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        m2 = capi.Mesh(v, f, device=dev)
        s2 = [capi.Solver(m2, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000, complex64_krylov=kcopy)
              for _ in range(B)]
        capi.solve_batch(s2, [freq_desc(capi, n, fr, src) for fr in batch_freqs(s)], [pts] * B)
        for sv in s2:
            sv.close()
        m2.close()
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_t], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t[0])
    e2e_val = args.steps * B * world / e2e_t
    # bem_mesh_create uploads 20 FP64 + 30 FP32/int rows per element; every
    # solve uploads the evaluation points and the frequency data, and returns
    # the unknowns (complex128), potentials and gradients (4 x complex128)
    h2d = n * (20 * 8 + 30 * 4) + B * (pts.nbytes + 16 + 24)
    d2h = B * (n * 16 + len(pts) * 16 * 4)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1000.0, "solves_per_step": B,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 (FP32 assembly, complex64 matrix with %s; refinement residuals from "
                 "the complex64 matrix, about twice-FP32 accurate; FP64 solution, Hessenberg and Givens)"
                 % COPY_DESC[args.krylov_copy],
        "data": "synthetic", "config": cfg,
        "stage_ms_per_solve": {"assemble": asm_ms / n_solves, "solve": solve_ms / n_solves,
                               "project": proj_ms / n_solves, "matvec": mv_ms / n_solves,
                               "iterations": float(np.mean(iters))},
        "roofline": {"bound": "hbm", "kernel": ROOF_KERNEL[args.krylov_copy],
                     "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if achieved else None,
                     "traffic": MV_TRAFFIC[args.krylov_copy][0] if n == N_TRI else None,
                     "traffic_algorithmic_bytes_same_launch": MV_TRAFFIC[args.krylov_copy][1] if n == N_TRI else None,
                     "traffic_source": MV_TRAFFIC[args.krylov_copy][2],
                     "bytes_per_krylov_product": bytes_krylov, "bytes_per_residual_product": bytes_resid,
                     "krylov_products": n_kry, "residual_products": n_mv - n_kry,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": args.steps, "frequencies": "the same K batches as value"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "wall_s": wall,
        "tuned": capi.tune_info(n, capi.PREC_MIXED, 1),
    }

    if rank == 0:
        # measured issue peaks and every stage's roofline
        ip = capi.issue_peaks(dev)
        stages, e2e_roof = stage_rooflines(n, len(pts), ip, hbm, infos, value, args.krylov_copy)
        line["roofline"]["stages"] = stages
        line["roofline"]["end_to_end"] = e2e_roof
        line["roofline"]["issue_peaks"] = dict(ip, source="bem_measure_issue_peaks (micro-kernels, CUDA events)")

        # latency: the same frequencies solved one at a time
        lat = []
        single = capi.Solver(mesh, precision=capi.PREC_MIXED, tol=1e-9, max_iter=3000)
        for s in range(args.warmup, args.warmup + args.steps):
            for fr in batch_freqs(s):
                F = freq_desc(capi, n, fr, src)
                t1 = time.perf_counter()
                single.solve_frequency(F, pts)
                lat.append(time.perf_counter() - t1)
        single.close()
        line["latency_ms"] = {"p50": float(np.percentile(lat, 50) * 1000),
                              "p99": float(np.percentile(lat, 99) * 1000),
                              "mode": "one solve at a time (bem_solve_frequency), the same %d frequencies" % len(lat)}

        # FP64 GPU path on the first timed batch, against the mixed time of
        # the same batch
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
        errs = [float(np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0])) for a, b in zip(first_res, r64)]
        ferrs = [float(np.linalg.norm(a[1] - b[1]) / np.linalg.norm(b[1])) for a, b in zip(first_res, r64)]
        line["fp64_gpu"] = {"value": B / t64, "unit": "solves/s", "frequencies": frs,
                            "mode": "bem_solve_batch of %d, the first timed batch" % B,
                            "mixed_same_batch_solves_per_s": B / step_s[0],
                            "speedup_mixed_over_fp64": t64 / step_s[0],
                            "mixed_rel_l2_boundary_err_max": max(errs),
                            "mixed_rel_l2_field_err_max": max(ferrs),
                            "hardest_frequency": {"freq_hz": max(frs), "boundary_err":
                                                  errs[int(np.argmax(frs))]}}
        if not args.no_serving:
            mesh.close()
            mesh = None
            capi.load().bem_release_cached_memory()
            line["serving"] = serving_leg(dev)

        from oracle import oracle_py as op

        threads = cpu_threads()
        om = op.OracleMesh(v, f)
        cpu_warmup(om, src, pts, threads)
        t_cpu, det = cpu_port_solve(om, src, pts, frs[0], threads)
        line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "solves/s", "cores": threads, "kind": "port",
                                "sample": (PORT_SAMPLE % (n, len(pts))) + "; one solve at %.0f Hz, the first "
                                          "frequency of the first timed batch" % frs[0],
                                "breakdown": det}
        print(json.dumps(line))
    if mesh is not None:
        mesh.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
