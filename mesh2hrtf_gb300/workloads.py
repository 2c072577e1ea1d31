"""Seeded synthetic workloads of the batched and served configurations.

head_workload       the head-like scatterer of the benchmark: ellipsoid
                    0.09/0.075/0.11 m with two seeded Gaussian bumps, 20480
                    triangles graded toward bump 1, source 1 mm off bump 1,
                    1730-point equal-angle grid on a 1.2 m sphere, 200
                    frequencies 100 Hz .. 20 kHz in a seeded order.
batched_instances   (mesh, frequency) pairs: perturbed ellipsoids
                    (0.09/0.075/0.11 m, smooth radial noise of 3 mm standard
                    deviation), element counts drawn log-uniform and rounded
                    to the nearest geodesic count 20 n^2, frequencies uniform,
                    a point source 1 mm off a seeded surface point.
serving_stream      the same kind of requests with Poisson arrival times.

No public data set is involved; the sizes, distributions and seeds stand in
for the reference's HRTF projects.
"""
from __future__ import annotations

import math

import numpy as np

from . import meshes

C0, RHO = 343.0, 1.21
SEED_BATCH = 20261205
SEED_STREAM = 20261206
SEED_HEAD = 20261204


def head_workload(seed=SEED_HEAD, mesh_n=32):
    """(nodes, elems, source, points, frequencies in a seeded order); mesh_n
    = 32 gives the 20480-triangle mesh (20 mesh_n^2 triangles)."""
    v, f, info = meshes.head_like(mesh_n, seed=seed)
    pts = meshes.equal_angle_grid(1.2, 5.0, 24)
    freqs = np.arange(1, 201) * 100.0
    order = np.random.default_rng(seed).permutation(len(freqs))
    return v, f, info["source"], pts, freqs[order]


def _instance(rng, i, seed, n_min, n_max, f_min, f_max):
    t = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
    n = max(2, int(round(math.sqrt(t / 20.0))))
    v, f = meshes.perturbed_ellipsoid(n, seed + 1000 + i)
    src = meshes.surface_point_with_normal(v, f, seed + 2000 + i)
    return {"nodes": v, "elems": f, "freq": float(rng.uniform(f_min, f_max)), "source": src}


def batched_instances(count=64, n_min=2000, n_max=30000, f_min=200.0, f_max=16000.0, seed=SEED_BATCH):
    rng = np.random.default_rng(seed)
    return [_instance(rng, i, seed, n_min, n_max, f_min, f_max) for i in range(count)]


def serving_stream(count, rate_hz, n_min=2000, n_max=40000, f_min=100.0, f_max=20000.0, seed=SEED_STREAM):
    """Requests with arrival times (s) of a Poisson process of rate_hz."""
    rng = np.random.default_rng(seed)
    reqs = [_instance(rng, i, seed, n_min, n_max, f_min, f_max) for i in range(count)]
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=count))
    for r, ti in zip(reqs, t):
        r["arrival"] = float(ti - t[0])
    return reqs


def frequency(capi, n, f_hz, src):
    """bem_frequency_desc of a point source of NC.inp amplitude 0.1 (potential units)."""
    k = 2 * np.pi * f_hz / C0
    amp = 0.1 / (1j * RHO * 2 * np.pi * f_hz)
    return capi.Frequency(k, n, point_sources=src, point_amps=[amp])
