"""Loading helpers for the fixtures in tests/golden (made by make_golden.py)."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = ["sphere80", "quad96_soft_plane", "sphere320_adm_velo", "sphere1280_1k", "pspw2412_4k"]
# projects with symmetry planes (NC.inp SYMMETRY block)
SYM_CASES = ["sym1_half216", "sym2_quarter54", "sym3_octant54"]


class Case:
    def __init__(self, name):
        self.name = name
        self.d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
        d = self.d
        self.nodes = d["nodes"]
        self.elems = d["elems"]
        self.n = len(self.elems)
        self.pts = d["eval_points"]
        self.freqs = d["freqs"]
        self.ibval = d["elem_ibval"].astype(np.int32)
        self.rho = float(d["speed_density"][1])
        # NC.inp symmetry codes per axis (0 none, 1 symmetric, 2 antisymmetric,
        # 3 / 4 reflecting) and the plane positions
        self.sym = tuple(int(v) for v in d.get("sym_planes", np.zeros(3, np.int32)))
        self.sym_coords = tuple(float(v) for v in d.get("sym_coords", np.zeros(3)))

    def step(self, s):
        d = self.d
        f, k, rp = d["s%d_freq_k_rpfact" % s]
        ps = d["point_sources"][:, :3]
        pw = d["plane_waves"][:, :3]
        return dict(k=k, rpfact=rp, freq=f, bc_type=self.ibval, bc_value=d["s%d_zbval0" % s],
                    admittance=d["s%d_zbval1" % s], point_sources=ps, point_amps=d["s%d_zposoc" % s],
                    plane_dirs=pw, plane_amps=d["s%d_zinwav" % s])

    def has(self, key):
        return key in self.d

    def __getitem__(self, key):
        return self.d[key]


def load(name):
    return Case(name)


def rel_err(a, b):
    """Relative L2 difference over the entries where b is finite; NaN entries
    (e.g. an evaluation point on a point source, where the reference also
    prints NaN) must sit at the same places in a, else the result is inf."""
    a = np.ravel(a)
    b = np.ravel(b)
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb):
        return float("inf")
    return float(np.linalg.norm(a[fb] - b[fb]) / max(np.linalg.norm(b[fb]), 1e-300))
