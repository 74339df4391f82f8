"""Lid-driven cavity, one SIMPLE step (80 x 80): the device momentum
operator and the pCorr system against the oracle.

Bars: momentum matrix equal to the oracle's as a set of non-zero (row,
column) entries -- Phase's CrsEquation::operator+= drops exact zeros that
the device matrix keeps -- with values within 1e-13 of the row scale and
rhs within 1e-13; the pCorr pattern bit-exact with the oracle assembled from
the oracle's own predictor; pCorr coefficients and rhs within 1e-8
(the two predictors are independent solves to 1e-12); pCorr solutions equal
up to the constant null-space component to 1e-6.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import simple

pytestmark = pytest.mark.gpu


def _csr_dict(rp, ci, v, n_rows):
    A = sp.csr_matrix((v, ci, rp), shape=(n_rows, n_rows if ci.size == 0 else
                                          max(n_rows, ci.max() + 1)))
    A.eliminate_zeros()
    return A


def test_momentum_operator_matches_oracle(pg, oracle):
    w = simple.cavity_inputs(24, 20)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = simple.cavity_inputs(24, 20, faces=m.faces())
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    rng = np.random.default_rng(3)
    n = m.n_cells
    u0 = rng.standard_normal((n, 2))
    uf = w["u_face"].copy()
    uf[m.faces()["rcell"] >= 0] = rng.standard_normal((m.n_interior, 2))
    for theta in (1.0, 0.5):
        mom = pg.MomentumEquation(m, w["bc_u"]).assemble(0.005, 0.01, theta, u0, uf)
        rp, ci, v, rhs = mom.export()
        rpo, cio, vo, rhso = om.momentum(0.005, 0.01, theta, u0, uf, w["bc_u"])
        A = sp.csr_matrix((v, ci, rp), shape=(n, n))
        Ao = sp.csr_matrix((vo, cio, rpo), shape=(2 * n, 2 * n))
        # both components share the coefficients
        Ax, Ay = Ao[:n, :n], Ao[n:, n:]
        assert (Ao[:n, n:].nnz == 0) and (Ao[n:, :n].nnz == 0)
        scale = np.abs(Ax).sum(axis=1).A.ravel()
        for B in (Ax, Ay):
            D = (A - B).tocsr()
            D.eliminate_zeros()
            rows = np.repeat(np.arange(n), np.diff(D.indptr))
            assert np.all(np.abs(D.data) <= 1e-13 * scale[rows])
        Az = A.copy()
        Az.eliminate_zeros()
        Bz = Ax.copy()
        Bz.eliminate_zeros()
        assert (abs(Az) > 0).nnz == (abs(Bz) > 0).nnz
        mag = np.abs(rhso) + 1e-300
        assert np.max(np.abs(rhs - rhso) / np.maximum(mag, 1e-12)) < 1e-12


def test_cavity_pcorr_system_and_solve(pg, oracle):
    out = simple.simple_pcorr(pg, 80, 80)
    eqn, mesh, w = out["eqn"], out["mesh"], out["inputs"]
    rp, ci, v, rhs = eqn.export()
    assert mesh.n_cells == 6400 and len(ci) == 31680
    # oracle pipeline from the oracle's own predictor
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    n = om.n_cells
    rpo_m, cio_m, vo_m, rhso_m = om.momentum(0.005, 0.01, 1.0, np.zeros((n, 2)),
                                             w["u_face"], w["bc_u"])
    u = np.empty((n, 2))
    for d in range(2):
        Ao = sp.csr_matrix((vo_m, cio_m, rpo_m), shape=(2 * n, 2 * n))
        sub = Ao[d * n:(d + 1) * n, d * n:(d + 1) * n].tocsr()
        xo, st = oracle.bicgstab(sub.indptr, sub.indices, sub.data,
                                 -rhso_m[d * n:(d + 1) * n], tol=1e-12)
        assert st["status"] == 0
        u[:, d] = xo
    assert np.linalg.norm(u - out["u"]) / np.linalg.norm(u) < 1e-9
    a_p = sp.csr_matrix((vo_m, cio_m, rpo_m)).diagonal()[:n]
    cells = om.cells()
    dco = cells["vol"] / a_p
    gf = om.interpolate_faces(dco)
    f = om.faces()
    uf = np.stack([om.interpolate_faces(u[:, 0]), om.interpolate_faces(u[:, 1])], 1)
    uf[f["rcell"] < 0] = w["u_face"][f["rcell"] < 0]
    rpo, cio, vo, rhso = om.laplacian(gf, w["bc_p"], np.zeros(om.n_faces), uf)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    assert np.allclose(v, vo, rtol=1e-8, atol=0)
    assert np.max(np.abs(rhs - rhso)) <= 1e-8 * np.max(np.abs(rhso))
    # consistent singular system: sum of the rhs is ~0
    assert abs(rhs.sum()) < 1e-10 * np.abs(rhs).sum()
    s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=5000)
    s.set_eqn(eqn)
    err = s.solve()
    x = s.x()
    assert s.stats.status == pg.PG_OK and err <= 1e-8
    xo, st = oracle.bicgstab(rpo, cio, vo, -rhso, tol=1e-11, max_iters=20000)
    d = (x - x.mean()) - (xo - xo.mean())
    assert np.linalg.norm(d) / np.linalg.norm(xo - xo.mean()) < 1e-6


def test_momentum_solved_from_the_device_matrix(pg):
    """Both velocity components solved from the device momentum matrix
    (pg_solver_set_eqn_component) equal the solves of the same matrix handed
    over as a host CSR, to the solve tolerance's scale; the second component
    keeps the first one's factorisation; the device diagonal is the matrix's
    own; a plain equation has only component 0."""
    w = simple.cavity_inputs(40, 32)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = simple.cavity_inputs(40, 32, faces=m.faces())
    rng = np.random.default_rng(7)
    n = m.n_cells
    u0 = rng.standard_normal((n, 2))
    mom = pg.MomentumEquation(m, w["bc_u"]).assemble(0.005, 0.01, 1.0, u0,
                                                      w["u_face"])
    rp, ci, v, rhs = mom.export()
    A = sp.csr_matrix((v, ci, rp), shape=(n, n))
    assert np.array_equal(mom.diagonal(), A.diagonal())
    s_dev = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=5000)
    s_host = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=5000)
    s_host.setRank(n)
    s_host.set(rp, ci, v)
    for d in range(2):
        s_dev.set_eqn(mom, component=d)
        s_dev.setGuess(None)
        assert s_dev.solve() <= 1e-12
        if d == 1:  # the factorisation of component 0 was kept
            assert s_dev.stats.setup_ms < 0.5 * setup0 + 0.05
        else:
            setup0 = s_dev.stats.setup_ms
        b = -rhs[d * n:(d + 1) * n]
        s_host.setRhs(b)
        s_host.setGuess(None)
        assert s_host.solve() <= 1e-12
        x, xh = s_dev.x(), s_host.x()
        assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.01e-12
        assert np.linalg.norm(x - xh) / np.linalg.norm(xh) < 1e-10
    f = m.faces()
    plain = pg.fv.laplacian(1.0, m, np.where(f["rcell"] < 0, 0, 1),
                            np.zeros(m.n_faces))
    with pytest.raises(pg.PhaseError):
        s_dev.set_eqn(plain, component=1)
