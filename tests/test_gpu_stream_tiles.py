"""The streamed (cp.async.bulk tile ring) x / r update and FP64 SpMV on
ragged sizes: a single partial tile (143 rows), a last tile with an odd
count (1023 = 3 * 256 + 255 rows: its last element is read from global
memory, the rest by bulk copies), and a last tile of one row (4097 rows).

Bars: every solve meets its FP64 true residual, and the solution agrees
with the oracle's BiCGStab on the device's own partition to 1e-7 relative
when both stop at 1e-12 (one-level Schwarz ILU(0): the oracle's algorithm
exactly; the grids' condition numbers stay below 1e5), in FP64 and in
float-float."""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes

pytestmark = pytest.mark.gpu


def _laplacian(pg, nx, ny, seed):
    nodes, cptr, cind = meshes.rectilinear(nx, ny, 1.0, 1.0)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    # fixed value on the boundary: a nonsingular system
    bc = np.zeros(m.n_faces, np.int32)
    rng = np.random.default_rng(seed)
    return pg.fv.laplacian(rng.uniform(1, 3, m.n_faces), m, bc,
                           np.zeros(m.n_faces),
                           rng.standard_normal((m.n_faces, 2)))


@pytest.mark.parametrize("shape", [(11, 13), (33, 31), (17, 241)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ragged_tiles_match_oracle(pg, oracle, shape, prec):
    nx, ny = shape
    eqn = _laplacian(pg, nx, ny, seed=nx * ny)
    assert eqn.n == nx * ny
    s = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=5000, coarse=0,
                              subdomain_rows=64,
                              precision=pg.MIXED if prec == "mixed" else pg.FP64)
    s.set_eqn(eqn)
    s.solve()
    assert s.stats.status == pg.PG_OK, s.stats.as_dict()
    rp, ci, v, rhs = eqn.export()
    A = sp.csr_matrix((v, ci, rp))
    x = s.x()
    assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-12
    part, _ = s.partition()
    xo, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-12, max_iters=5000,
                             part=part)
    assert st["status"] == 0
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-7
