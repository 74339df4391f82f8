"""Flow around a cylinder on a graded triangle mesh: the pCorr system of one
PISO-style predictor step, assembled and solved on the device.

Coarse mesh: assembly against the oracle (pattern and off-diagonals
bit-exact, diagonals and rhs within 1e-14 of the row scale) and the
solution against the oracle's BiCGStab on the same partition (1e-9
relative, both converged to 1e-12).  About 500k triangles (h = 0.01 at the
cylinder to 0.1): FP64 and float-float solves meet 1e-8 on the FP64 true
residual."""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import simple

pytestmark = pytest.mark.gpu

ROW_TOL = 1e-14


def test_cylinder_pcorr_matches_oracle(pg, oracle):
    c = simple.cylinder_pcorr(pg, dict(h_near=0.05, h_far=0.5, grading=4.0))
    mesh, eqn = c["mesh"], c["eqn"]
    rp, ci, v, rhs = eqn.export()
    om = oracle.OracleMesh(c["nodes"], c["cptr"], c["cind"])
    f = om.faces()
    bc_p = np.ones(om.n_faces, np.int32)
    bc_p[(c["patch"] == 1) | (c["patch"] == 2)] = 0
    rpo, cio, vo, rhso = om.laplacian(c["gamma_f"], bc_p, np.zeros(om.n_faces),
                                      c["u_face"])
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    off = ci != rows
    assert np.array_equal(v[off], vo[off])
    scale = np.add.reduceat(np.abs(vo), rp[:-1])
    assert np.all(np.abs(v[~off] - vo[~off]) <= ROW_TOL * scale[rows[~off]])
    s = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=5000)
    s.set_eqn(eqn)
    assert s.solve() <= 1e-12 and s.stats.status == pg.PG_OK
    part, _ = s.partition()
    xo, st = oracle.bicgstab(rpo, cio, vo, -rhso, tol=1e-12, max_iters=5000,
                             part=part)
    assert st["status"] == 0
    x = s.x()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cylinder_500k_solves(pg, precision):
    c = simple.cylinder_pcorr(pg)
    n = c["mesh"].n_cells
    assert 450_000 < n < 560_000
    s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=10000,
                              precision=pg.MIXED if precision == "mixed"
                              else pg.FP64)
    s.set_eqn(c["eqn"])
    err = s.solve()
    assert s.stats.status == pg.PG_OK and err <= 1e-8
    rp, ci, v, rhs = c["eqn"].export()
    A = sp.csr_matrix((v, ci, rp))
    x = s.x()
    assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-8
