"""The allocation-free gradient entry point (pg_gradient_noalloc).

Callers that cannot allocate device memory -- a time loop living inside a
fixed device budget owned by another framework, or code that must not let
cudaMalloc/cudaFree synchronise the device -- get the cell gradient with the
face-gradient scratch held in a static device array.  This file is collected
last so a failure here comes after every other test has run; it also passes
on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from phase_gb300 import meshes

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def test_noalloc_gradient_matches_pg_gradient_twice(pg):
    torch = pytest.importorskip("torch")
    nodes, cptr, cind = meshes.triangulated(60, 40, 2.0, 1.0, jitter=0.2,
                                            seed=9)
    m = pg.Mesh(nodes, cptr, cind)
    c, f = m.cells(), m.faces()
    L = pg.lib()
    for k in range(2):  # two calls in a row share the static scratch
        phi = np.sin((k + 2) * c["cx"]) * np.cos(3 * c["cy"]) + k
        phi_f = np.sin((k + 2) * f["fx"]) * np.cos(3 * f["fy"]) + k
        _, expect = m.gradient(phi, phi_f)  # existing entry point
        d_phi, d_pf = _dev(torch, phi), _dev(torch, phi_f)
        d_out = torch.full((2 * m.n_cells,), float("nan"),
                           dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.pg_gradient_noalloc(m._h, ctypes.c_void_p(d_phi.data_ptr()),
                                   ctypes.c_void_p(d_pf.data_ptr()),
                                   ctypes.c_void_p(d_out.data_ptr()))
        assert rc == pg.PG_OK, L.pg_last_error().decode()
        got = d_out.cpu().numpy().reshape(-1, 2)
        # same bar as the other gradient parity tests: bit-exact
        assert np.array_equal(got, expect)


def test_noalloc_gradient_at_exactly_its_limit(pg):
    """193 x 2709 quads have 2*193*2709 + 193 + 2709 = 1,048,576 faces: the
    scratch array is used to its last entry."""
    torch = pytest.importorskip("torch")
    nodes, cptr, cind = meshes.rectilinear(193, 2709, 1.0, 14.0)
    m = pg.Mesh(nodes, cptr, cind)
    assert m.n_faces == (1 << 20)
    c, f = m.cells(), m.faces()
    phi = np.cos(2 * c["cx"]) * c["cy"] + 0.25 * c["cy"] ** 2
    phi_f = np.cos(2 * f["fx"]) * f["fy"] + 0.25 * f["fy"] ** 2
    _, expect = m.gradient(phi, phi_f)
    d_phi, d_pf = _dev(torch, phi), _dev(torch, phi_f)
    d_out = torch.full((2 * m.n_cells,), float("nan"), dtype=torch.float64,
                       device="cuda")
    torch.cuda.synchronize()
    rc = pg.lib().pg_gradient_noalloc(m._h, ctypes.c_void_p(d_phi.data_ptr()),
                                      ctypes.c_void_p(d_pf.data_ptr()),
                                      ctypes.c_void_p(d_out.data_ptr()))
    assert rc == pg.PG_OK, pg.lib().pg_last_error().decode()
    assert np.array_equal(d_out.cpu().numpy().reshape(-1, 2), expect)


def test_noalloc_gradient_rejects_host_pointers(pg):
    """A host array passed where device memory is required is refused
    before any kernel is launched."""
    torch = pytest.importorskip("torch")
    nodes, cptr, cind = meshes.rectilinear(16, 8)
    m = pg.Mesh(nodes, cptr, cind)
    host = np.zeros(2 * m.n_faces)
    d = torch.zeros(2 * m.n_faces, dtype=torch.float64, device="cuda")
    rc = pg.lib().pg_gradient_noalloc(
        m._h, ctypes.c_void_p(host.ctypes.data),
        ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()))
    assert rc == pg.PG_BAD_ARG
    assert "device memory" in pg.lib().pg_last_error().decode()


def test_noalloc_gradient_rejects_meshes_beyond_its_limit(pg):
    torch = pytest.importorskip("torch")
    nodes, cptr, cind = meshes.rectilinear(1024, 512)  # 1,050,112 faces
    m = pg.Mesh(nodes, cptr, cind)
    assert m.n_faces > (1 << 20)
    d = torch.zeros(2 * m.n_faces, dtype=torch.float64, device="cuda")
    rc = pg.lib().pg_gradient_noalloc(m._h, ctypes.c_void_p(d.data_ptr()),
                                      ctypes.c_void_p(d.data_ptr()),
                                      ctypes.c_void_p(d.data_ptr()))
    assert rc == pg.PG_BAD_ARG
    assert "at most 1048576" in pg.lib().pg_last_error().decode()
