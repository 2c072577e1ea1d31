"""Synthetic boundary meshes and evaluation grids for the BEM workloads.

The reference ships only one small sphere fixture and its remesher
(``mesh2hrtf/Mesh2Input/Meshes/GradingHybrid``) is an empty submodule, so the
workloads are generated here from seeded parameters:

* ``geodesic_sphere(n)``: icosahedron with every face split into ``n**2``
  triangles, vertices projected on the sphere (``20*n**2`` triangles;
  ``n = 2**L`` is the usual L-times subdivided icosphere, n = 8 gives the
  1280-triangle sphere).
* ``head_like(...)``: triaxial ellipsoid (0.09/0.075/0.11 m) with two seeded
  Gaussian bumps standing in for pinnae, vertices graded toward bump 1 by a
  stereographic dilation on the parameter sphere.
* ``perturbed_ellipsoid(...)``: the same ellipsoid with smooth, seeded radial
  noise and an arbitrary ``20*n**2`` triangle count.
* ``sphere_sector(...)``: the part of a cube-projected sphere on the positive
  side of one to three coordinate planes, the input of a problem with
  symmetry planes (NumCalc's SYMMETRY block, ``NC_Input.cpp:459-494``).

All triangles are oriented so that (P0-P2) x (P1-P2) points into the fluid,
the orientation the reference's sphere fixture uses
(``tests/resources/test_numcalc/project_folder_pspw``) and the one NumCalc's
normal computation assumes (``NC_3dFunctions.cpp:132-178``).
"""
from __future__ import annotations

import numpy as np

HEAD_AXES = (0.09, 0.075, 0.11)


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    v /= np.linalg.norm(v, axis=1)[:, None]
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], int)
    return v, f


def geodesic_sphere(n: int, radius: float = 1.0):
    """Unit-sphere geodesic triangulation with ``20*n*n`` triangles.

    Vertices shared between faces are merged exactly (edge points are
    generated from the sorted edge key), so the mesh is closed and every
    interior edge is used by two triangles with opposite orientation.
    """
    if n < 1:
        raise ValueError("n must be >= 1")
    v0, f0 = _icosahedron()
    verts: list[np.ndarray] = [p for p in v0]
    key_to_idx: dict[tuple, int] = {}

    def vid(face_corner_ids, i, j):
        # barycentric lattice point (i, j, n-i-j) on the face spanned by a, b, c
        a, b, c = face_corner_ids
        w = {a: n - i - j, b: i, c: j}
        nz = tuple(sorted((k, wk) for k, wk in w.items() if wk > 0))
        if len(nz) == 1:
            return nz[0][0]
        if nz in key_to_idx:
            return key_to_idx[nz]
        p = sum(v0[k] * wk for k, wk in nz) / n
        verts.append(p / np.linalg.norm(p))
        key_to_idx[nz] = len(verts) - 1
        return key_to_idx[nz]

    tris = []
    for a, b, c in f0:
        ids = (a, b, c)
        grid = [[vid(ids, i, j) for j in range(n + 1 - i)] for i in range(n + 1)]
        for i in range(n):
            for j in range(n - i):
                p = grid[i][j]
                q = grid[i + 1][j]
                r = grid[i][j + 1]
                tris.append((p, q, r))
                if j < n - i - 1:
                    s = grid[i + 1][j + 1]
                    tris.append((q, s, r))
    v = np.asarray(verts) * radius
    f = np.asarray(tris, dtype=np.int64)
    return _orient_outward(v, f)


def _orient_outward(v, f):
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    nrm = np.cross(a - c, b - c)
    cen = (a + b + c) / 3.0
    flip = np.einsum("ij,ij->i", nrm, cen) < 0
    f = f.copy()
    f[flip] = f[flip][:, [1, 0, 2]]
    return v, f


def icosphere(n_triangles: int = 1280, radius: float = 0.1):
    n = int(round((n_triangles / 20) ** 0.5))
    if 20 * n * n != n_triangles:
        raise ValueError("icosphere triangle counts are 20*n^2")
    return geodesic_sphere(n, radius)


def _stereo_grade(u, pole, lam):
    """Move unit vectors toward ``pole``: tan(theta'/2) = lam*tan(theta/2)."""
    cth = np.clip(u @ pole, -1.0, 1.0)
    th = np.arccos(cth)
    th2 = 2.0 * np.arctan(lam * np.tan(0.5 * th))
    perp = u - cth[:, None] * pole[None, :]
    pn = np.linalg.norm(perp, axis=1)
    ok = pn > 1e-14
    e = np.zeros_like(u)
    e[ok] = perp[ok] / pn[ok, None]
    out = np.cos(th2)[:, None] * pole[None, :] + np.sin(th2)[:, None] * e
    out[~ok] = np.where((cth[~ok] > 0)[:, None], pole[None, :], -pole[None, :])
    return out


def _ellipsoid_radius(u, axes):
    a, b, c = axes
    return 1.0 / np.sqrt((u[:, 0] / a) ** 2 + (u[:, 1] / b) ** 2 + (u[:, 2] / c) ** 2)


def head_like(n: int = 32, seed: int = 20261204, lam: float = 0.577,
              axes=HEAD_AXES):
    """Head-like scatterer: ellipsoid + two Gaussian bumps, graded mesh.

    Returns (nodes, triangles, info) where ``info`` holds the bump centres
    (unit directions), the outward surface normal at bump 1 and the point
    1 mm off bump 1 along that normal (the reciprocal source position).
    ``n = 32`` gives 20480 triangles.
    """
    rng = np.random.default_rng(seed)
    u, f = geodesic_sphere(n, 1.0)
    # bump directions: near +y and -y (pinna positions), seeded jitter
    dirs = []
    for side in (+1.0, -1.0):
        d = np.array([rng.normal(0, 0.15), side, rng.normal(0, 0.15)])
        dirs.append(d / np.linalg.norm(d))
    amps = rng.uniform(0.006, 0.010, size=2)     # bump heights in m
    widths = rng.uniform(0.18, 0.26, size=2)     # angular widths in rad
    ug = _stereo_grade(u, dirs[0], lam)

    def surface(dirs_u):
        r = _ellipsoid_radius(dirs_u, axes)
        for d, a, w in zip(dirs, amps, widths):
            ang = np.arccos(np.clip(dirs_u @ d, -1, 1))
            r = r + a * np.exp(-0.5 * (ang / w) ** 2)
        return dirs_u * r[:, None]

    v = surface(ug)
    # outward normal at bump 1 by finite differences on the parameter sphere
    d1 = dirs[0]
    t1 = np.cross(d1, [0.0, 0.0, 1.0])
    t1 /= np.linalg.norm(t1)
    t2 = np.cross(d1, t1)
    h = 1e-5
    p = surface(d1[None, :])[0]
    pa = surface(((d1 + h * t1) / np.linalg.norm(d1 + h * t1))[None, :])[0]
    pb = surface(((d1 + h * t2) / np.linalg.norm(d1 + h * t2))[None, :])[0]
    nrm = np.cross(pa - p, pb - p)
    nrm /= np.linalg.norm(nrm)
    if nrm @ p < 0:
        nrm = -nrm
    info = {"bump_dirs": np.array(dirs), "bump_amps": amps, "bump_widths": widths,
            "bump1_point": p, "bump1_normal": nrm, "source": p + 0.001 * nrm}
    v, f = _orient_outward(v, f)
    return v, f, info


def perturbed_ellipsoid(n: int, seed: int, sigma: float = 0.003, axes=HEAD_AXES):
    """Ellipsoid with smooth seeded radial noise of standard deviation sigma."""
    rng = np.random.default_rng(seed)
    u, f = geodesic_sphere(n, 1.0)
    r = _ellipsoid_radius(u, axes)
    k = rng.normal(size=(24, 3)) * 2.0          # low spatial frequencies
    ph = rng.uniform(0, 2 * np.pi, size=24)
    noise = np.cos(u @ k.T + ph[None, :]).sum(axis=1)
    noise = (noise - noise.mean()) / noise.std() * sigma
    v = u * (r + noise)[:, None]
    return _orient_outward(v, f)


def surface_point_with_normal(v, f, seed):
    """Seeded point 1 mm off the centroid of a random triangle, along its normal."""
    rng = np.random.default_rng(seed)
    t = int(rng.integers(len(f)))
    a, b, c = v[f[t, 0]], v[f[t, 1]], v[f[t, 2]]
    nrm = np.cross(a - c, b - c)
    nrm /= np.linalg.norm(nrm)
    return (a + b + c) / 3.0 + 0.001 * nrm


# ----------------------------------------------------------------- eval grids
def random_sphere_points(m: int, radius: float, seed: int):
    """``m`` points at ``radius`` with directions = normalised N(0, I3) draws."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return d * radius


def equal_angle_grid(radius: float = 1.2, az_step_deg: float = 5.0,
                     n_rings: int = 24):
    """72 azimuths x 24 elevation rings (step 180/25 = 7.2 deg) + 2 poles.

    With the defaults this is the 1730-point grid of the head-like workload.
    """
    az = np.deg2rad(np.arange(0.0, 360.0, az_step_deg))
    step = 180.0 / (n_rings + 1)
    el = np.deg2rad(-90.0 + step * np.arange(1, n_rings + 1))
    pts = [[0.0, 0.0, -radius]]
    for e in el:
        for a in az:
            pts.append([radius * np.cos(e) * np.cos(a), radius * np.cos(e) * np.sin(a),
                        radius * np.sin(e)])
    pts.append([0.0, 0.0, radius])
    return np.asarray(pts)


def fibonacci_sphere(m: int, radius: float):
    """Near-uniform spherical point set (golden-angle spiral).

    11950 points give a mean spacing of sqrt(4 pi / 11950) = 1.86 degrees,
    the "2 degree" grid of the large single-solve workload.
    """
    i = np.arange(m) + 0.5
    z = 1.0 - 2.0 * i / m
    phi = np.pi * (1.0 + 5.0 ** 0.5) * i
    rr = np.sqrt(1.0 - z * z)
    return radius * np.stack([rr * np.cos(phi), rr * np.sin(phi), z], axis=1)


def grid_triangles(points):
    """Triangulate a closed point set on a sphere (convex hull).

    NumCalc needs every evaluation node to belong to an evaluation element
    (``NC_Input.cpp:610-654``); the element shapes are not used otherwise.
    """
    from scipy.spatial import ConvexHull

    hull = ConvexHull(points)
    return np.asarray(hull.simplices, dtype=np.int64)


def shells_triangles(shells):
    """Evaluation elements for several concentric point shells, one hull each."""
    tris, off = [], 0
    for pts in shells:
        tris.append(grid_triangles(np.asarray(pts)) + off)
        off += len(pts)
    return np.vstack(tris)


def cube_sphere(n: int, radius: float):
    """Quadrilateral sphere: every cube face split into n x n quads and
    projected; quads ordered so that NumCalc's quad normal dx/ds x dx/dt
    (``NC_3dFunctions.cpp:132-178``) points outward."""
    pts, quads, idx = [], [], {}

    def vid(p):
        key = tuple(np.round(p, 12))
        if key not in idx:
            idx[key] = len(pts)
            pts.append(p)
        return idx[key]

    g = np.linspace(-1.0, 1.0, n + 1)
    for ax in range(3):
        for sgn in (-1.0, 1.0):
            for a in range(n):
                for b in range(n):
                    cs = []
                    for (u, w) in ((g[a], g[b]), (g[a + 1], g[b]), (g[a + 1], g[b + 1]), (g[a], g[b + 1])):
                        p = np.zeros(3)
                        p[ax] = sgn
                        p[(ax + 1) % 3] = u
                        p[(ax + 2) % 3] = w
                        cs.append(vid(p))
                    quads.append(cs)
    v = np.array(pts)
    v = v / np.linalg.norm(v, axis=1)[:, None] * radius
    q = np.array(quads)
    for e in range(len(q)):
        P = v[q[e]]
        dxs = 0.25 * (P[0] - P[1] - P[2] + P[3])
        dxt = 0.25 * (P[0] + P[1] - P[2] - P[3])
        if np.dot(np.cross(dxs, dxt), P.mean(axis=0)) < 0:
            q[e] = q[e][::-1]
    return v, q


def sphere_sector(n: int, radius: float, axes, center=(0.0, 0.0, 0.0), triangles: bool = False):
    """The quads of ``cube_sphere(n, radius)`` (n even) whose centres lie on
    the positive side of the planes normal to ``axes``, moved by ``center``
    (the planes then pass through ``center``).  ``triangles`` splits every
    quad (P0, P1, P2, P3) into (P0, P1, P2) and (P0, P2, P3), keeping the
    normal.  Nodes on a plane lie on it exactly when ``center`` is zero."""
    if n % 2:
        raise ValueError("n must be even so that grid lines lie on the planes")
    v, q = cube_sphere(n, radius)
    cen = v[q].mean(axis=1)
    keep = np.ones(len(q), bool)
    for ax in axes:
        keep &= cen[:, ax] > 0.0
    q = q[keep]
    used = np.unique(q)
    remap = -np.ones(len(v), np.int64)
    remap[used] = np.arange(len(used))
    v = v[used] + np.asarray(center, float)[None, :]
    q = remap[q]
    if triangles:
        q = np.concatenate([q[:, [0, 1, 2]], q[:, [0, 2, 3]]], axis=0)
    return v, q
