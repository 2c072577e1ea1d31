"""ctypes binding of the C ABI in include/bem_gb300.h (libbem_gb300.so).

This is the Python face of the GPU library: tests, the bench and the serving
loop drive the solver through exactly the entry points the drop-in NumCalc
executable uses.  There is no fallback: if the library or a CUDA device is
missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

BEM_OK = 0
BEM_ERR_INVALID = 1
BEM_ERR_OUT_OF_HBM = 2
BEM_ERR_NOT_CONVERGED = 3
BEM_ERR_DEVICE_TIMEOUT = 4
BEM_ERR_CUDA = 5
BEM_ERR_SUBDIVISION = 6
BEM_ERR_PENDING = 7
PREC_FP64 = 0
PREC_MIXED = 1
KRYLOV_BLR = 2   # Solver(complex64_krylov=KRYLOV_BLR): block low-rank Krylov copy

EXPORTED = [
    "bem_last_error", "bem_version", "bem_kernel_launches", "bem_set_device", "bem_footprint_bytes",
    "bem_mesh_create", "bem_mesh_destroy", "bem_solver_create", "bem_solver_destroy", "bem_solver_set_params",
    "bem_assemble", "bem_solve", "bem_get_solution", "bem_get_system", "bem_project",
    "bem_solve_frequency", "bem_project_static", "bem_solve_batch", "bem_solve_multi", "bem_footprint_multi",
    "bem_server_create", "bem_server_submit", "bem_server_wait", "bem_server_destroy",
    "bem_mesh_footprint_bytes", "bem_device_memory", "bem_release_cached_memory", "bem_measure_issue_peaks",
    "bem_solve_direct", "bem_tune_info", "bem_krylov_copy_info",
]
STATIC_MAX_ELEMENTS = 32768


class BemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("bem status %d: %s" % (status, msg))
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [("n_elem", C.c_int32), ("n_nodes", C.c_int32), ("nodes", C.c_void_p),
                ("conn", C.c_void_p), ("nvert", C.c_void_p), ("centers", C.c_void_p),
                ("normals", C.c_void_p), ("areas", C.c_void_p), ("sym_planes", C.c_int32 * 3),
                ("sym_coords", C.c_double * 3)]


class FreqDesc(C.Structure):
    _fields_ = [("wave_number", C.c_double), ("time_factor", C.c_double), ("tao", C.c_double),
                ("bc_type", C.c_void_p), ("bc_value", C.c_void_p), ("admittance", C.c_void_p),
                ("n_point", C.c_int32), ("point_xyz", C.c_void_p), ("point_amp", C.c_void_p),
                ("n_plane", C.c_int32), ("plane_dir", C.c_void_p), ("plane_amp", C.c_void_p)]


class SolverParams(C.Structure):
    _fields_ = [("precision", C.c_int32), ("restart", C.c_int32), ("max_iter", C.c_int32),
                ("tol", C.c_double), ("hbm_budget_bytes", C.c_double), ("no_precond", C.c_int32),
                ("n_rhs", C.c_int32), ("complex64_krylov", C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("restarts", C.c_int32), ("rel_residual", C.c_double),
                ("assemble_ms", C.c_double), ("solve_ms", C.c_double), ("project_ms", C.c_double),
                ("n_near_pairs", C.c_int64), ("matvec_ms", C.c_double), ("n_matvec", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerParams(C.Structure):
    _fields_ = [("precision", C.c_int32), ("hbm_budget_bytes", C.c_double), ("max_active", C.c_int32),
                ("restart", C.c_int32), ("max_iter", C.c_int32), ("tol", C.c_double), ("device", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("queued_ms", C.c_double), ("latency_ms", C.c_double), ("solve", SolveInfo)]

    def as_dict(self):
        d = {"queued_ms": self.queued_ms, "latency_ms": self.latency_ms}
        d.update(self.solve.as_dict())
        return d


_lib = None


def load(build_if_missing: bool = True):
    """Load libbem_gb300.so (building it first when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError("libbem_gb300.so not built: " + LIB_PATH)
        _build.build_library()
    lib = C.CDLL(LIB_PATH)
    vp, i32, dp = C.c_void_p, C.c_int32, C.POINTER(C.c_double)
    lib.bem_last_error.restype = C.c_char_p
    lib.bem_version.restype = C.c_char_p
    lib.bem_kernel_launches.restype = C.c_int64
    lib.bem_set_device.argtypes = [i32]
    lib.bem_footprint_bytes.argtypes = [i32, i32, i32]
    lib.bem_footprint_bytes.restype = C.c_double
    lib.bem_footprint_multi.argtypes = [i32, i32, i32, i32]
    lib.bem_footprint_multi.restype = C.c_double
    lib.bem_mesh_footprint_bytes.argtypes = [i32, i32]
    lib.bem_mesh_footprint_bytes.restype = C.c_double
    lib.bem_device_memory.argtypes = [i32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.bem_solve_multi.argtypes = [vp, i32, vp, i32, vp, vp, vp, vp, vp]
    lib.bem_mesh_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(vp)]
    lib.bem_mesh_destroy.argtypes = [vp]
    lib.bem_solver_create.argtypes = [vp, C.POINTER(SolverParams), C.POINTER(vp)]
    lib.bem_solver_destroy.argtypes = [vp]
    lib.bem_solver_set_params.argtypes = [vp, C.POINTER(SolverParams)]
    lib.bem_assemble.argtypes = [vp, C.POINTER(FreqDesc)]
    lib.bem_solve.argtypes = [vp, C.POINTER(SolveInfo)]
    lib.bem_get_solution.argtypes = [vp, vp]
    lib.bem_get_system.argtypes = [vp, i32, i32, vp, vp]
    lib.bem_project.argtypes = [vp, i32, vp, vp, vp]
    lib.bem_solve_frequency.argtypes = [vp, C.POINTER(FreqDesc), i32, vp, vp, vp, vp, C.POINTER(SolveInfo)]
    lib.bem_project_static.argtypes = [vp, i32, vp, vp, vp, vp]
    lib.bem_solve_batch.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.bem_server_create.argtypes = [C.POINTER(ServerParams), C.POINTER(vp)]
    lib.bem_server_submit.argtypes = [vp, vp, C.POINTER(FreqDesc), i32, vp, C.POINTER(C.c_uint64)]
    lib.bem_server_wait.argtypes = [vp, C.c_uint64, C.c_double, vp, vp, vp, C.POINTER(RequestInfo)]
    lib.bem_server_destroy.argtypes = [vp]
    lib.bem_measure_issue_peaks.argtypes = [i32, dp]
    lib.bem_solve_direct.argtypes = [vp, C.POINTER(SolveInfo)]
    lib.bem_tune_info.argtypes = [i32, i32, i32, C.c_char_p, i32]
    lib.bem_krylov_copy_info.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
    for name in EXPORTED:
        if name not in ("bem_last_error", "bem_version", "bem_footprint_bytes", "bem_footprint_multi",
                        "bem_kernel_launches", "bem_mesh_footprint_bytes"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def _check(rc, allow=()):
    if rc != BEM_OK and rc not in allow:
        raise BemError(rc, load().bem_last_error().decode())
    return rc


def _ptr(a):
    return None if a is None else a.ctypes.data


class Mesh:
    """Device-resident boundary mesh (bem_mesh_create).

    sym_planes / sym_coords: NumCalc's SYMMETRY block, per axis the NC.inp
    code (0 none, 1 symmetric, 2 antisymmetric, 3 / 4 reflecting) and the
    plane position; the mesh is the part on one side of the planes."""

    def __init__(self, nodes, elems, centers=None, normals=None, areas=None, device=0,
                 sym_planes=(0, 0, 0), sym_coords=(0.0, 0.0, 0.0)):
        lib = load()
        _check(lib.bem_set_device(device))
        elems = np.asarray(elems)
        n = len(elems)
        self.n = n
        self.nodes = np.ascontiguousarray(nodes, np.float64)
        self.conn = -np.ones((n, 4), np.int32)
        self.conn[:, : elems.shape[1]] = elems
        self.nvert = np.full(n, elems.shape[1], np.int32)
        if elems.shape[1] == 4:
            self.nvert[elems[:, 3] < 0] = 3
        keep = [self.nodes, self.conn, self.nvert]
        cen = None if centers is None else np.ascontiguousarray(centers, np.float64)
        nor = None if normals is None else np.ascontiguousarray(normals, np.float64)
        ar = None if areas is None else np.ascontiguousarray(areas, np.float64)
        keep += [cen, nor, ar]
        d = MeshDesc(n, len(self.nodes), _ptr(self.nodes), _ptr(self.conn), _ptr(self.nvert),
                     _ptr(cen), _ptr(nor), _ptr(ar), (C.c_int32 * 3)(*[int(c) for c in sym_planes]),
                     (C.c_double * 3)(*[float(c) for c in sym_coords]))
        h = C.c_void_p()
        _check(lib.bem_mesh_create(C.byref(d), C.byref(h)))
        self.handle = h
        self._keep = keep

    def close(self):
        if getattr(self, "handle", None):
            load().bem_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Frequency:
    """Per-frequency data (bem_frequency_desc); arrays are kept alive here."""

    def __init__(self, k, n_elem, bc_type=None, bc_value=None, admittance=None, point_sources=(),
                 point_amps=(), plane_dirs=(), plane_amps=(), time_factor=1.0, tao=1.0):
        self.bct = None if bc_type is None else np.ascontiguousarray(bc_type, np.int32)
        self.bcv = None if bc_value is None else np.ascontiguousarray(
            np.asarray(bc_value, np.complex128).reshape(n_elem, 4))
        self.adm = None if admittance is None else np.ascontiguousarray(admittance, np.complex128)
        self.ps = np.ascontiguousarray(np.reshape(point_sources, (-1, 3)), np.float64)
        self.psa = np.ascontiguousarray(np.asarray(point_amps, np.complex128).reshape(-1))
        self.pw = np.ascontiguousarray(np.reshape(plane_dirs, (-1, 3)), np.float64)
        self.pwa = np.ascontiguousarray(np.asarray(plane_amps, np.complex128).reshape(-1))
        self.desc = FreqDesc(k, time_factor, tao, _ptr(self.bct), _ptr(self.bcv), _ptr(self.adm),
                             len(self.ps), _ptr(self.ps), _ptr(self.psa), len(self.pw), _ptr(self.pw),
                             _ptr(self.pwa))


class Solver:
    """bem_solver_t: matrix + Krylov workspace for one mesh on the device."""

    def __init__(self, mesh: Mesh, precision=PREC_FP64, restart=0, max_iter=0, tol=0.0, hbm_budget=0.0,
                 precond=True, n_rhs=1, complex64_krylov=False):
        """complex64_krylov: the copy of A that the Krylov products of a mixed
        precision solver with one right-hand side read: False (the fp16 copy),
        True (none: they read A) or KRYLOV_BLR (the block low-rank copy).
        precond: True (block-Jacobi with its window correction), "block-jacobi"
        (block-Jacobi alone), "scaling" (NumCalc's diagonal scaling) or False
        (none)."""
        lib = load()
        self.mesh = mesh
        self.n = mesh.n
        if precond == "block-jacobi":
            npc = 2
        elif precond == "scaling":
            npc = 3
        elif precond is True or precond is False:
            npc = 0 if precond else 1
        else:
            raise ValueError("precond must be True, False, 'block-jacobi' or 'scaling', not %r" % (precond,))
        kc = KRYLOV_BLR if complex64_krylov == KRYLOV_BLR else (1 if complex64_krylov else 0)
        p = SolverParams(precision, restart, max_iter, tol, hbm_budget, npc, n_rhs, kc)
        h = C.c_void_p()
        _check(lib.bem_solver_create(mesh.handle, C.byref(p), C.byref(h)))
        self.handle = h
        self.info = SolveInfo()

    def set_params(self, max_iter=0, tol=0.0):
        p = SolverParams(0, 0, max_iter, tol, 0.0, 0, 0, 0)
        _check(load().bem_solver_set_params(self.handle, C.byref(p)))

    def assemble(self, freq: Frequency):
        _check(load().bem_assemble(self.handle, C.byref(freq.desc)))

    def solve(self, allow_not_converged=False):
        allow = (BEM_ERR_NOT_CONVERGED,) if allow_not_converged else ()
        _check(load().bem_solve(self.handle, C.byref(self.info)), allow)
        return self.info.as_dict()

    def solve_direct(self):
        """bem_solve_direct: LU without pivoting in place (the matrix is
        consumed until the next assemble)."""
        _check(load().bem_solve_direct(self.handle, C.byref(self.info)))
        return self.info.as_dict()

    def krylov_copy_info(self):
        """bem_krylov_copy_info: the block low-rank Krylov copy (dict)."""
        nb, nd = C.c_int32(), C.c_int32()
        mr, by = C.c_double(), C.c_double()
        _check(load().bem_krylov_copy_info(self.handle, C.byref(nb), C.byref(nd), C.byref(mr), C.byref(by)))
        return {"blocks_per_row": nb.value, "dense_blocks": nd.value, "mean_rank": mr.value,
                "bytes_per_product": by.value}

    def solution(self):
        x = np.zeros(self.n, np.complex128)
        _check(load().bem_get_solution(self.handle, _ptr(x)))
        return x

    def system(self, rows=None, with_matrix=True):
        r0, r1 = (0, self.n) if rows is None else rows
        A = np.zeros((r1 - r0, self.n), np.complex128) if with_matrix else None
        b = np.zeros(self.n, np.complex128)
        _check(load().bem_get_system(self.handle, r0, r1, _ptr(A), _ptr(b)))
        return A, b

    def project(self, pts, with_grad=True):
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        pot = np.zeros(len(pts), np.complex128)
        grad = np.zeros((len(pts), 3), np.complex128) if with_grad else None
        _check(load().bem_project(self.handle, len(pts), _ptr(pts), _ptr(pot), _ptr(grad)))
        return pot, grad

    def project_static(self, n_pts, pts_dev, pot_dev, grad_dev=None, stream=None):
        """bem_project_static: device pointers in and out, no allocation."""
        return _check(load().bem_project_static(self.handle, n_pts, pts_dev, pot_dev, grad_dev, stream))

    def solve_frequency(self, freq: Frequency, pts, with_grad=True, allow_not_converged=False):
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        x = np.zeros(self.n, np.complex128)
        pot = np.zeros(len(pts), np.complex128)
        grad = np.zeros((len(pts), 3), np.complex128) if with_grad else None
        allow = (BEM_ERR_NOT_CONVERGED,) if allow_not_converged else ()
        _check(load().bem_solve_frequency(self.handle, C.byref(freq.desc), len(pts), _ptr(pts), _ptr(x),
                                          _ptr(pot), _ptr(grad), C.byref(self.info)), allow)
        return x, pot, grad

    def solve_multi(self, freqs, pts, with_grad=True, allow_not_converged=False):
        """bem_solve_multi: one matrix, len(freqs) right-hand sides.

        Returns lists x[r], pot[r], grad[r] and the infos (dicts)."""
        R = len(freqs)
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        m = len(pts)
        xs = [np.zeros(self.n, np.complex128) for _ in range(R)]
        pots = [np.zeros(m, np.complex128) for _ in range(R)]
        grads = [np.zeros((m, 3), np.complex128) for _ in range(R)] if with_grad else None
        PtrArr = C.c_void_p * R
        fs = (FreqDesc * R)(*[f.desc for f in freqs])
        infos = (SolveInfo * R)()
        allow = (BEM_ERR_NOT_CONVERGED,) if allow_not_converged else ()
        _check(load().bem_solve_multi(self.handle, R, fs, m, _ptr(pts) if m else None,
                                      PtrArr(*[x.ctypes.data for x in xs]),
                                      PtrArr(*[p.ctypes.data if m else None for p in pots]),
                                      PtrArr(*[g.ctypes.data if m else None for g in grads]) if with_grad else None,
                                      infos), allow)
        return xs, pots, grads, [i.as_dict() for i in infos]

    def close(self):
        if getattr(self, "handle", None):
            load().bem_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(solvers, freqs, pts_list=None, with_grad=True, allow_not_converged=False):
    """bem_solve_batch: solve (solver, frequency) instances together.

    Returns a list of (x, pot, grad, info dict, status) per instance."""
    cnt = len(solvers)
    if len(freqs) != cnt:
        raise ValueError("one frequency per solver")
    SolverArr = C.c_void_p * cnt
    FreqArr = FreqDesc * cnt
    PtrArr = C.c_void_p * cnt
    hs = SolverArr(*[s.handle.value for s in solvers])
    fs = FreqArr(*[f.desc for f in freqs])
    xs, pots, grads, ptss = [], [], [], []
    for i, s in enumerate(solvers):
        xs.append(np.zeros(s.n, np.complex128))
        p = np.zeros((0, 3)) if pts_list is None else np.ascontiguousarray(pts_list[i], np.float64).reshape(-1, 3)
        ptss.append(p)
        pots.append(np.zeros(len(p), np.complex128))
        grads.append(np.zeros((len(p), 3), np.complex128) if with_grad else None)
    npts = (C.c_int32 * cnt)(*[len(p) for p in ptss])
    pts_a = PtrArr(*[p.ctypes.data if len(p) else None for p in ptss])
    x_a = PtrArr(*[x.ctypes.data for x in xs])
    pot_a = PtrArr(*[q.ctypes.data if len(q) else None for q in pots])
    grad_a = PtrArr(*[(g.ctypes.data if (g is not None and len(g)) else None) for g in grads])
    infos = (SolveInfo * cnt)()
    sts = (C.c_int32 * cnt)()
    allow = (BEM_ERR_NOT_CONVERGED,) if allow_not_converged else ()
    rc = load().bem_solve_batch(cnt, hs, fs, npts, pts_a, x_a, pot_a, grad_a, infos, sts)
    if rc != BEM_OK and not all(int(v) in (BEM_OK,) + allow for v in sts):
        _check(rc, allow)
    return [(xs[i], pots[i], grads[i], infos[i].as_dict(), int(sts[i])) for i in range(cnt)]


class Server:
    """bem_server_t: solve requests served with continuous batching."""

    def __init__(self, precision=PREC_MIXED, hbm_budget=0.0, max_active=0, restart=0, max_iter=0, tol=0.0,
                 device=0):
        p = ServerParams(precision, hbm_budget, max_active, restart, max_iter, tol, device)
        h = C.c_void_p()
        _check(load().bem_server_create(C.byref(p), C.byref(h)))
        self.handle = h
        self._req = {}

    def submit(self, mesh: Mesh, freq: Frequency, pts):
        """Queue one request; returns its ticket.  Inputs are copied."""
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        t = C.c_uint64()
        _check(load().bem_server_submit(self.handle, mesh.handle, C.byref(freq.desc), len(pts),
                                        _ptr(pts) if len(pts) else None, C.byref(t)))
        self._req[t.value] = (mesh.n, len(pts))
        return t.value

    def wait(self, ticket, timeout=-1.0, allow_not_converged=False):
        """Result of a request: (x, pot, grad, info dict, status); None while pending."""
        n, m = self._req[ticket]
        x = np.zeros(n, np.complex128)
        pot = np.zeros(m, np.complex128)
        grad = np.zeros((m, 3), np.complex128)
        info = RequestInfo()
        rc = load().bem_server_wait(self.handle, ticket, timeout, _ptr(x), _ptr(pot) if m else None,
                                    _ptr(grad) if m else None, C.byref(info))
        if rc == BEM_ERR_PENDING:
            return None
        del self._req[ticket]
        allow = (BEM_ERR_NOT_CONVERGED,) if allow_not_converged else ()
        _check(rc, allow)
        return x, pot, grad, info.as_dict(), rc

    def close(self):
        if getattr(self, "handle", None):
            load().bem_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def issue_peaks(device=0):
    """bem_measure_issue_peaks: measured FP32 FMA, special-function and FP64
    FMA rates of the device (operations per second)."""
    r = np.zeros(3)
    _check(load().bem_measure_issue_peaks(device, r.ctypes.data_as(C.POINTER(C.c_double))))
    return {"fp32_fma_per_s": float(r[0]), "sfu_per_s": float(r[1]), "fp64_fma_per_s": float(r[2])}


def tune_info(n_elem, precision=PREC_MIXED, n_rhs=1):
    """bem_tune_info: the launch shapes the tuner holds for this key (dict)."""
    import json

    buf = C.create_string_buffer(1024)
    _check(load().bem_tune_info(n_elem, precision, n_rhs, buf, len(buf)))
    return json.loads(buf.value.decode())


def footprint_bytes(n_elem, precision=PREC_MIXED, restart=0):
    return load().bem_footprint_bytes(n_elem, precision, restart)


def mesh_footprint_bytes(n_elem, n_sym_planes=0):
    return load().bem_mesh_footprint_bytes(n_elem, n_sym_planes)


def device_memory(device=0):
    """(free, total) bytes of a device."""
    fr, tot = C.c_double(), C.c_double()
    _check(load().bem_device_memory(device, C.byref(fr), C.byref(tot)))
    return fr.value, tot.value
