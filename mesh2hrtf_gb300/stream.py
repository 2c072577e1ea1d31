"""Serve a seeded Poisson stream of solve requests (bem_server_*) and report
throughput and latency, mixed precision and plain FP64 on the same stream.

    python -m mesh2hrtf_gb300.stream [--requests 48] [--rate 30] [--budget 160e9]
        [--precision both|mixed|fp64] [--n-min 2000] [--n-max 40000]

Requests: perturbed ellipsoids with element counts log-uniform in
[n-min, n-max], frequencies uniform in 0.1-20 kHz, a point source 1 mm off
the surface, the 1730-point 1.2 m grid (workloads.serving_stream).  Each
request is submitted at its arrival time; latency runs from submission to
results ready, throughput is requests over the time from the first arrival
to the last completion.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi, meshes, workloads


def serve(reqs, mesh_handles, pts, precision, budget, max_active):
    srv = capi.Server(precision=precision, hbm_budget=budget, max_active=max_active, tol=1e-9, max_iter=3000)
    freqs = [workloads.frequency(capi, len(r["elems"]), r["freq"], r["source"]) for r in reqs]
    t0 = time.perf_counter()
    tickets = []
    for r, m, F in zip(reqs, mesh_handles, freqs):
        dt = r["arrival"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append((time.perf_counter() - t0, srv.submit(m, F, pts)))
    out = []
    for (ts, t) in tickets:
        x, pot, grad, info, st = srv.wait(t, timeout=3600.0, allow_not_converged=True)
        out.append({"submit_s": ts, "x": x, "info": info, "status": st})
    srv.close()
    lat = np.array([o["info"]["latency_ms"] for o in out])
    done = max(o["submit_s"] + o["info"]["latency_ms"] / 1000.0 for o in out)
    return out, {
        "requests": len(out), "throughput_per_s": len(out) / done, "makespan_s": done,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "mean": float(lat.mean())},
        "queued_ms_mean": float(np.mean([o["info"]["queued_ms"] for o in out])),
        "iterations_mean": float(np.mean([o["info"]["iterations"] for o in out])),
        "converged": int(sum(o["status"] == capi.BEM_OK for o in out)),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--rate", type=float, default=30.0)
    ap.add_argument("--budget", type=float, default=160e9)
    ap.add_argument("--max-active", type=int, default=0)
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"])
    ap.add_argument("--n-min", type=int, default=2000)
    ap.add_argument("--n-max", type=int, default=40000)
    a = ap.parse_args()
    reqs = workloads.serving_stream(a.requests, a.rate, n_min=a.n_min, n_max=a.n_max)
    pts = meshes.equal_angle_grid()
    handles = [capi.Mesh(r["nodes"], r["elems"]) for r in reqs]
    n = np.array([len(r["elems"]) for r in reqs])
    rep = {"workload": "Poisson stream, %d requests at %.1f/s, perturbed ellipsoids %d-%d triangles "
                       "(log-uniform), 0.1-20 kHz, 1730-point 1.2 m grid" % (a.requests, a.rate, a.n_min, a.n_max),
           "n_elements": {"min": int(n.min()), "max": int(n.max()), "mean": float(n.mean())},
           "budget_bytes": a.budget}
    res = {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        if a.precision not in ("both", name):
            continue
        out, summ = serve(reqs, handles, pts, prec, a.budget, a.max_active)
        res[name] = out
        rep[name] = summ
    if "mixed" in res and "fp64" in res:
        errs = [float(np.linalg.norm(m["x"] - d["x"]) / np.linalg.norm(d["x"]))
                for m, d in zip(res["mixed"], res["fp64"])]
        rep["mixed_rel_l2_err_max"] = max(errs)
        rep["throughput_mixed_over_fp64"] = rep["mixed"]["throughput_per_s"] / rep["fp64"]["throughput_per_s"]
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
