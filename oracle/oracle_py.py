"""Test infrastructure (oracle only): ctypes front end of the FP64 C
restatement in oracle/bem_oracle.c.  Tests, fixture scripts and the bench's
CPU-baseline leg are its only callers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbem_oracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle-lib"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        _lib.or_geometry.argtypes = [C.c_void_p, dp, dp, dp]
        _lib.or_assemble.argtypes = [C.c_void_p, dp, dp, dp, C.c_void_p, C.c_int, C.c_int, dp, dp, C.c_int]
        _lib.or_assemble.restype = C.c_int
        _lib.or_solve_dense.argtypes = [C.c_int, dp, dp, dp]
        _lib.or_project.argtypes = [C.c_void_p, dp, dp, dp, C.c_void_p, dp, dp, C.c_int, dp, dp, dp, C.c_int]
        _lib.or_project.restype = C.c_int
        _lib.or_solve_cgs.argtypes = [C.c_int, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double, dp, ip, dp,
                                      C.c_int, dp]
        _lib.or_solve_cgs.restype = C.c_int
        _lib.or_subelements.argtypes = [C.c_void_p, C.c_int, dp, C.c_double, dp, dp, dp, ip]
        _lib.or_subelements.restype = C.c_int
    return _lib


class _Mesh(C.Structure):
    _fields_ = [("n_elem", C.c_int), ("nodes", C.c_void_p), ("conn", C.c_void_p),
                ("nvert", C.c_void_p), ("bc_type", C.c_void_p), ("bc_val", C.c_void_p),
                ("adm", C.c_void_p), ("sym", C.c_int * 3), ("sym_coord", C.c_double * 3)]


# NC.inp symmetry codes -> the reference's internal codes (NC_Input.cpp:470-491)
SYM_CODES = {0: 0, 1: 1, 2: -1, 3: 2, 4: -2}


class _Freq(C.Structure):
    _fields_ = [("k", C.c_double), ("htf", C.c_double), ("tao", C.c_double),
                ("n_point", C.c_int), ("ps_xyz", C.c_void_p), ("ps_amp", C.c_void_p),
                ("n_plane", C.c_int), ("pw_dir", C.c_void_p), ("pw_amp", C.c_void_p)]


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleMesh:
    """Boundary mesh in the oracle's layout (keeps the numpy buffers alive)."""

    def __init__(self, nodes, elems, bc_type=None, bc_val=None, adm=None, sym=(0, 0, 0),
                 sym_coord=(0.0, 0.0, 0.0)):
        """sym: per axis the NC.inp SYMMETRY code (0 none, 1 symmetric,
        2 antisymmetric, 3 / 4 reflecting, treated as 1 / 2 on this path)."""
        elems = np.asarray(elems)
        n = len(elems)
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.conn = -np.ones((n, 4), dtype=np.int32)
        self.conn[:, : elems.shape[1]] = elems
        self.nvert = np.full(n, elems.shape[1], dtype=np.int32)
        if elems.shape[1] == 4:
            self.nvert[:] = 4
        self.bc_type = np.zeros(n, np.int32) if bc_type is None else np.asarray(bc_type, np.int32)
        self.bc_val = np.zeros((n, 4), np.complex128) if bc_val is None else np.asarray(bc_val, np.complex128)
        self.adm = np.zeros(n, np.complex128) if adm is None else np.asarray(adm, np.complex128)
        self.n = n
        self.sym = tuple(SYM_CODES[int(c)] for c in sym)
        self.sym_coord = tuple(float(c) for c in sym_coord)
        self._s = _Mesh(n, self.nodes.ctypes.data, self.conn.ctypes.data, self.nvert.ctypes.data,
                        self.bc_type.ctypes.data, self.bc_val.ctypes.data, self.adm.ctypes.data,
                        (C.c_int * 3)(*self.sym), (C.c_double * 3)(*self.sym_coord))
        self.centers = np.zeros((n, 3))
        self.normals = np.zeros((n, 15))
        self.areas = np.zeros(n)
        lib().or_geometry(C.byref(self._s), _p(self.centers), _p(self.normals), _p(self.areas))


class OracleFreq:
    def __init__(self, k, point_sources=(), ps_amp=(), plane_dirs=(), pw_amp=(), htf=1.0, tao=1.0):
        self.ps = np.ascontiguousarray(np.reshape(point_sources, (-1, 3)), dtype=np.float64)
        self.psa = np.ascontiguousarray(np.asarray(ps_amp, np.complex128).reshape(-1))
        self.pw = np.ascontiguousarray(np.reshape(plane_dirs, (-1, 3)), dtype=np.float64)
        self.pwa = np.ascontiguousarray(np.asarray(pw_amp, np.complex128).reshape(-1))
        self._s = _Freq(k, htf, tao, len(self.ps), self.ps.ctypes.data, self.psa.ctypes.data,
                        len(self.pw), self.pw.ctypes.data, self.pwa.ctypes.data)


def assemble(mesh: OracleMesh, freq: OracleFreq, rows=None, nthreads=0):
    r0, r1 = (0, mesh.n) if rows is None else rows
    A = np.zeros((r1 - r0, mesh.n), np.complex128)
    b = np.zeros(r1 - r0, np.complex128)
    rc = lib().or_assemble(C.byref(mesh._s), _p(mesh.centers), _p(mesh.normals), _p(mesh.areas),
                           C.byref(freq._s), r0, r1, _p(A), _p(b), nthreads)
    if rc != 0:
        raise RuntimeError("oracle assembly failed (subdivision limit)")
    return A, b


def solve_dense(A, b):
    A = np.array(A, dtype=np.complex128, order="C", copy=True)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros_like(b)
    if lib().or_solve_dense(len(b), _p(A), _p(b), _p(x)) != 0:
        raise RuntimeError("singular matrix")
    return x


def solve_cgs(A, b, precond=0, scan=0, niter_max=250, tol=1e-9, nthreads=0, overwrite=False):
    """NumCalc's CGS with its preconditioners (or_solve_cgs).  A and b are
    copied unless overwrite (then A must be C-contiguous complex128; it is
    row-scaled and, on the direct fallback, factored in place).  Returns x,
    iterations, relative error, whether the direct fallback ran, and the
    stage seconds (set-up, iterations, final step)."""
    if overwrite:
        assert A.dtype == np.complex128 and A.flags.c_contiguous
    else:
        A = np.array(A, dtype=np.complex128, order="C", copy=True)
    b = np.array(b, dtype=np.complex128, copy=True)
    x = np.zeros_like(b)
    it = C.c_int(0)
    err = C.c_double(0.0)
    st = np.zeros(3)
    rc = lib().or_solve_cgs(len(b), _p(A), _p(b), precond, scan, niter_max, tol, _p(x), C.byref(it),
                            C.byref(err), nthreads, _p(st))
    if rc < 0:
        raise RuntimeError("or_solve_cgs: allocation failed")
    return x, it.value, err.value, rc == 1, st


def boundary_fields(mesh: OracleMesh, x, tao=1.0):
    """Element potentials and nodal velocities from the unknowns
    (NC_WriteResultsObjectMesh, NC_PostProcessing.cpp:367-400)."""
    phi = np.where(mesh.bc_type == 1, mesh.bc_val[:, 0], x)
    vel = mesh.bc_val.copy()
    adm = mesh.bc_type == 2
    vel[adm] -= (x[adm] * mesh.adm[adm])[:, None] * tao
    pres = mesh.bc_type == 1
    vel[pres] = x[pres][:, None]
    vel[np.arange(4)[None, :] >= mesh.nvert[:, None]] = 0.0
    return np.ascontiguousarray(phi), np.ascontiguousarray(vel)


def project(mesh: OracleMesh, freq: OracleFreq, phi, vel, pts, nthreads=0):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    pot = np.zeros(len(pts), np.complex128)
    grad = np.zeros((len(pts), 3), np.complex128)
    phi = np.ascontiguousarray(phi, np.complex128)
    vel = np.ascontiguousarray(vel, np.complex128)
    rc = lib().or_project(C.byref(mesh._s), _p(mesh.centers), _p(mesh.normals), _p(mesh.areas),
                          C.byref(freq._s), _p(phi), _p(vel), len(pts), _p(pts), _p(pot), _p(grad),
                          nthreads)
    if rc != 0:
        raise RuntimeError("oracle projection failed (subdivision limit)")
    return pot, grad


def subelements(mesh: OracleMesh, j, x):
    xi = np.zeros(220); eta = np.zeros(220); fac = np.zeros(220)
    order = np.zeros(220, np.int32)
    x = np.ascontiguousarray(x, np.float64)
    n = lib().or_subelements(C.byref(mesh._s), j, _p(x), float(mesh.areas[j]), _p(xi), _p(eta), _p(fac),
                             order.ctypes.data_as(C.POINTER(C.c_int)))
    if n < 0:
        raise RuntimeError("subdivision limit")
    return xi[:n], eta[:n], fac[:n], order[:n]
