"""bem_project_static, the projection entry point that allocates nothing.

Callers such as real-time renderers or plug-in hosts evaluate the solved field
at new positions on every processing block and must not allocate device
memory there (an allocation can block or synchronize the device), so they
pass their own device buffers and the library keeps its scratch in a fixed
device array.  This file is collected last on purpose: it runs after every
other test and also passes alone in a fresh process.
"""
import numpy as np
import pytest

from mesh2hrtf_gb300 import capi, meshes

pytestmark = pytest.mark.gpu


def _solved(n_tri=320, prec=capi.PREC_MIXED):
    v, f = meshes.icosphere(n_tri, 0.1)
    m = capi.Mesh(v, f)
    s = capi.Solver(m, precision=prec, tol=1e-10)
    k = 2 * np.pi * 1500.0 / 343.0
    fr = capi.Frequency(k, len(f), point_sources=[0.5, 0.2, 0.1], point_amps=[1e-3 + 2e-4j])
    s.assemble(fr)
    s.solve()
    return m, s


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_static_projection_matches_bem_project_twice(prec):
    torch = pytest.importorskip("torch")
    m, s = _solved(prec=prec)
    # near the surface (subdivided pairs) and far away
    pts = np.vstack([meshes.random_sphere_points(40, 0.6, 21), meshes.random_sphere_points(8, 0.104, 22)])
    pot_ref, grad_ref = s.project(pts)
    dev = torch.device("cuda", 0)
    pts_d = torch.tensor(pts, dtype=torch.float64, device=dev).contiguous()
    stream = torch.cuda.current_stream(dev).cuda_stream
    results = []
    for call in range(2):
        pot_d = torch.full((len(pts), 2), float("nan"), dtype=torch.float64, device=dev)
        grad_d = torch.full((len(pts), 3, 2), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        free0 = torch.cuda.mem_get_info(dev)[0]
        s.project_static(len(pts), pts_d.data_ptr(), pot_d.data_ptr(), grad_d.data_ptr(), stream)
        if call > 0:
            # the defining property: once the first call on the device has
            # looked up the scratch array, a call takes no device memory
            assert torch.cuda.mem_get_info(dev)[0] == free0
        pot = pot_d.cpu().numpy().view(np.complex128).reshape(-1)
        grad = grad_d.cpu().numpy().view(np.complex128).reshape(len(pts), 3)
        results.append((pot, grad))
        assert np.linalg.norm(pot - pot_ref) <= 1e-12 * np.linalg.norm(pot_ref)
        assert np.linalg.norm(grad - grad_ref) <= 1e-12 * np.linalg.norm(grad_ref)
    assert np.array_equal(results[0][0], results[1][0])
    s.close()
    m.close()


def test_static_projection_rejects_large_solvers():
    n = 20 * 41 * 41                      # 33620 > BEM_STATIC_MAX_ELEMENTS
    assert n > capi.STATIC_MAX_ELEMENTS
    v, f = meshes.geodesic_sphere(41, 0.1)
    m = capi.Mesh(v, f)
    s = capi.Solver(m, precision=capi.PREC_MIXED)
    with pytest.raises(capi.BemError) as e:
        s.project_static(0, None, None, None, None)
    assert e.value.status == capi.BEM_ERR_INVALID
    assert "BEM_STATIC_MAX_ELEMENTS" in str(e.value)
    s.close()
    m.close()
