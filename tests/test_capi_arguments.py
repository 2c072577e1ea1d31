"""The C ABI's argument checks, which run before any device call (so no GPU
is needed): empty meshes, missing arrays, too many elements, unknown
symmetry codes and null handles give BEM_ERR_INVALID with a message in
bem_last_error, and destroying a null handle is a no-op."""
import ctypes as C

import numpy as np
import pytest

from mesh2hrtf_gb300 import capi

LIB = capi.load()


def _status(rc):
    return rc, LIB.bem_last_error().decode()


def _mesh_desc(n_elem=2, n_nodes=4, nodes=True, conn=True, nvert=True, sym=(0, 0, 0)):
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float64)
    cn = np.array([[0, 1, 2, -1], [1, 3, 2, -1]], np.int32)
    nv = np.array([3, 3], np.int32)
    keep = (xyz, cn, nv)
    d = capi.MeshDesc(n_elem, n_nodes, xyz.ctypes.data if nodes else None, cn.ctypes.data if conn else None,
                      nv.ctypes.data if nvert else None, None, None, None, (C.c_int32 * 3)(*sym),
                      (C.c_double * 3)(0.0, 0.0, 0.0))
    return d, keep


@pytest.mark.parametrize("kw,msg", [
    (dict(n_elem=0), "mesh needs elements"),
    (dict(n_elem=-3), "mesh needs elements"),
    (dict(n_nodes=0), "mesh needs elements"),
    (dict(nodes=False), "mesh needs elements"),
    (dict(conn=False), "mesh needs elements"),
    (dict(nvert=False), "mesh needs elements"),
    (dict(n_elem=1 << 30), "elements: at most"),
    (dict(sym=(0, 5, 0)), "symmetry code 5 on axis 1"),
    (dict(sym=(-1, 0, 0)), "symmetry code -1 on axis 0"),
])
def test_mesh_descriptor_is_checked(kw, msg):
    d, keep = _mesh_desc(**kw)
    h = C.c_void_p()
    rc, err = _status(LIB.bem_mesh_create(C.byref(d), C.byref(h)))
    assert rc == capi.BEM_ERR_INVALID and msg in err
    assert not h.value


def test_null_handles_are_rejected():
    h = C.c_void_p()
    assert _status(LIB.bem_mesh_create(None, C.byref(h)))[0] == capi.BEM_ERR_INVALID
    p = capi.SolverParams(capi.PREC_MIXED, 0, 0, 0.0, 0.0, 0, 0, 0)
    assert _status(LIB.bem_solver_create(None, C.byref(p), C.byref(h))) == (capi.BEM_ERR_INVALID, "null argument")
    f = capi.FreqDesc()
    assert _status(LIB.bem_assemble(None, C.byref(f)))[0] == capi.BEM_ERR_INVALID
    assert _status(LIB.bem_solve(None, None)) == (capi.BEM_ERR_INVALID, "null solver")
    assert _status(LIB.bem_solve_direct(None, None))[0] == capi.BEM_ERR_INVALID
    x = np.zeros(8)
    assert _status(LIB.bem_get_solution(None, x.ctypes.data))[0] == capi.BEM_ERR_INVALID
    assert _status(LIB.bem_project(None, 1, x.ctypes.data, x.ctypes.data, None)) == \
        (capi.BEM_ERR_INVALID, "null solver")
    assert _status(LIB.bem_solve_multi(None, 1, C.byref(f), 0, None, None, None, None, None))[0] == \
        capi.BEM_ERR_INVALID
    assert _status(LIB.bem_krylov_copy_info(None, None, None, None, None))[0] == capi.BEM_ERR_INVALID
    assert _status(LIB.bem_solve_batch(-1, None, None, None, None, None, None, None, None, None)) == \
        (capi.BEM_ERR_INVALID, "bad batch arrays")
    assert _status(LIB.bem_solve_batch(2, None, None, None, None, None, None, None, None, None))[0] == \
        capi.BEM_ERR_INVALID
    assert _status(LIB.bem_device_memory(0, None, None)) == (capi.BEM_ERR_INVALID, "null argument")
    # destroying nothing is allowed
    assert LIB.bem_mesh_destroy(None) == capi.BEM_OK
    assert LIB.bem_solver_destroy(None) == capi.BEM_OK
