"""Projection step after the pressure solve (FractionalStep::correctVelocity):
bit-exact against the oracle, and on the rising-bubble system the corrected
face velocities are discretely divergence-free to the solve's tolerance
(div(u* - dt/rho_f grad_f p) = div(u*) - laplacian(dt/rho, p) on an
orthogonal mesh)."""
import numpy as np
import pytest

from phase_gb300 import meshes, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("with_rho", [False, True])
@pytest.mark.parametrize("mesh", ["rect", "tri"])
def test_correct_velocity_matches_oracle(pg, oracle, with_rho, mesh):
    nodes, cptr, cind = (meshes.rectilinear(13, 7, 1.3, 0.7) if mesh == "rect"
                         else meshes.triangulated(9, 8, 1.0, 1.0, jitter=0.2, seed=2))
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    rng = np.random.default_rng(8)
    n, nf = m.n_cells, m.n_faces
    gc, gf = rng.standard_normal((n, 2)), rng.standard_normal((nf, 2))
    uc, uf = rng.standard_normal((n, 2)), rng.standard_normal((nf, 2))
    rc = rng.uniform(1.0, 1000.0, n) if with_rho else None
    rf = rng.uniform(1.0, 1000.0, nf) if with_rho else None
    a = m.correct_velocity(3.7e-3, gc, gf, uc, uf, rc, rf)
    b = om.correct_velocity(3.7e-3, gc, gf, uc, uf, rc, rf)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("mesh", ["rect", "tri"])
def test_set_boundary_faces_matches_oracle(pg, oracle, mesh):
    nodes, cptr, cind = (meshes.rectilinear(11, 6, 1.1, 0.6) if mesh == "rect"
                         else meshes.triangulated(8, 9, 1.0, 1.0, jitter=0.2, seed=3))
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    rng = np.random.default_rng(4)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, rng.integers(0, 3, om.n_faces), 1).astype(np.int32)
    pc, pf = rng.standard_normal(om.n_cells), rng.standard_normal(om.n_faces)
    a = m.set_boundary_faces(bc, pc, pf)
    b = om.set_boundary_faces(bc, pc, pf)
    assert np.array_equal(a, b)
    inner = f["rcell"] >= 0
    assert np.array_equal(a[inner], pf[inner])


def test_projection_makes_faces_divergence_free(pg, oracle):
    nx = 64
    w = workloads.rising_bubble(nx, nx, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    faces, cells = m.faces(), m.cells()
    w = workloads.rising_bubble(nx, nx, seed=3, faces=faces, cells=cells)
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    eqn = pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])
    s = pg.SparseMatrixSolver(tolerance=1e-10, max_iters=20000)
    s.set_eqn(eqn)
    assert s.solve() <= 1e-10 and s.stats.status == pg.PG_OK
    p = s.x()
    # setBoundaryFaces on the device: fixed faces keep their value (here the
    # boundary value), the others take the cell's
    p_face = m.set_boundary_faces(w["bc_type"], p,
                                  np.where(faces["rcell"] < 0, w["bc_value"], 0.0))
    grad_face, grad_cell = m.gradient(p, p_face)
    rho_face = w["dt"] / coeff
    rho_cell = w["rho1"] + np.clip(w["gamma"], 0, 1) * (w["rho2"] - w["rho1"])
    uc0 = np.zeros((m.n_cells, 2))
    _, uf = m.correct_velocity(w["dt"], grad_cell, grad_face, uc0, w["u"],
                               rho_cell, rho_face)
    # src::div(u) per cell, taken from the oracle's right-hand side of
    # fv::laplacian(0, p) == src::div(u) (rhs = -div u)
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])

    def div(u):
        return -om.laplacian(0.0, w["bc_type"], w["bc_value"], u)[3]

    d0, d1 = div(w["u"]), div(uf)
    # ||div u*  - A p||_2 <= 1e-10 ||div u*||_2 bounds the largest cell
    # residual by 1e-10 sqrt(n) max|div u*|
    assert np.abs(d1).max() <= 1e-10 * nx * np.abs(d0).max()
