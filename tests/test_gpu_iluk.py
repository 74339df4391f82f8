"""ILU(k) blocks (Phase's iluFill key, Ifpack2 RILUK "fact: iluk
level-of-fill", TrilinosBelosSparseMatrixSolver.cpp:70) against the
oracle's level-of-fill factorisation on the same partition.

The device builds each subdomain's level-k pattern in the original row
order, schedules the rows by the filled pattern (the order of every
coupled pair is kept, so the factor is the natural-order one) and
factors it on the device; the preconditioner application must therefore
equal the oracle's ILU(k) up to rounding (1e-12 relative, FP64)."""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes, workloads

pytestmark = pytest.mark.gpu


def _tri_eqn(pg, nx=48, ny=40, seed=5):
    nodes, cptr, cind = meshes.triangulated(nx, ny, 1.0, 1.0, jitter=0.2,
                                            seed=seed)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(seed)
    return pg.fv.laplacian(rng.uniform(1.0, 3.0, m.n_faces), m, bc,
                           np.zeros(m.n_faces),
                           rng.standard_normal((m.n_faces, 2)))


def _bubble_eqn(pg, n):
    w = workloads.rising_bubble(n, n, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(n, n, seed=3, faces=m.faces(), cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    return pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])


@pytest.mark.parametrize("fill", [1, 2, 3])
@pytest.mark.parametrize("mesh", ["tri", "bubble"])
def test_iluk_apply_matches_oracle(pg, oracle, mesh, fill):
    eqn = _tri_eqn(pg) if mesh == "tri" else _bubble_eqn(pg, 96)
    rp, ci, v, rhs = eqn.export()
    s = pg.SparseMatrixSolver(subdomain_rows=600, ilu_fill=fill)
    s.set_eqn(eqn)
    assert s.sweep_form() == 0  # filled blocks take the stream form
    part, nparts = s.partition()
    assert nparts > 2
    rng = np.random.default_rng(fill)
    for r in (rng.standard_normal(eqn.n), -rhs):
        z = s.apply_precond(r)
        zo, rc = oracle.iluk_apply(rp, ci, v, r, fill, part)
        assert rc == 0
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-12


def test_iluk_zero_is_ilu0(pg, oracle):
    """ilu_fill 0 is the ILU(0) path; the oracle's ILU(k) at k = 0 agrees."""
    eqn = _tri_eqn(pg)
    rp, ci, v, _ = eqn.export()
    s = pg.SparseMatrixSolver(subdomain_rows=600, ilu_fill=0)
    s.set_eqn(eqn)
    part, _ = s.partition()
    r = np.random.default_rng(9).standard_normal(eqn.n)
    zo, rc = oracle.iluk_apply(rp, ci, v, r, 0, part)
    assert rc == 0
    z = s.apply_precond(r)
    assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iluk_solves_in_fewer_iterations(pg, oracle, precision):
    """ILU(2) blocks cut the BiCGStab iterations on the triangle mesh; the
    device's iteration count tracks the oracle's on the same partition and
    both reach the tolerance on the true residual."""
    eqn = _tri_eqn(pg, 96, 80)
    rp, ci, v, rhs = eqn.export()
    A = sp.csr_matrix((v, ci, rp))
    prec = pg.MIXED if precision == "mixed" else pg.FP64
    its, oits = {}, {}
    for fill in (0, 2):
        s = pg.SparseMatrixSolver(tolerance=1e-10, max_iters=5000,
                                  subdomain_rows=1024, ilu_fill=fill,
                                  precision=prec)
        s.set_eqn(eqn)
        assert s.solve() <= 1e-10 and s.stats.status == pg.PG_OK
        assert np.linalg.norm(-rhs - A @ s.x()) / np.linalg.norm(rhs) <= 1.01e-10
        its[fill] = s.nIters()
        part, _ = s.partition()
        _, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-10, max_iters=5000,
                                part=part, ilu_fill=fill)
        assert st["status"] == 0
        oits[fill] = st["iters"]
    assert its[2] < its[0], its
    assert oits[2] < oits[0], oits
    for fill in (0, 2):
        assert abs(its[fill] - oits[fill]) <= max(3, 0.15 * oits[fill]), (its, oits)


def test_iluk_with_the_coarse_correction(pg, oracle):
    """ILU(1) blocks under the deflated two-level preconditioner match the
    oracle's two-level ILU(1) application."""
    eqn = _bubble_eqn(pg, 128)
    rp, ci, v, _ = eqn.export()
    s = pg.SparseMatrixSolver(subdomain_rows=512, ilu_fill=1, coarse=2,
                              tolerance=1e-8, max_iters=3000)
    s.set_eqn(eqn)
    part, nparts = s.partition()
    assert nparts >= 16
    assert s.solve() <= 1e-8
    _, st = oracle.bicgstab(rp, ci, v, -eqn.export()[3], tol=1e-8,
                            max_iters=3000, part=part, coarse=2, ilu_fill=1)
    assert st["status"] == 0
    assert abs(s.nIters() - st["iters"]) <= max(3, 0.15 * st["iters"])


def test_iluk_plugin_key(pg):
    """Phase's iluFill key reaches the device through the plugin options."""
    from phase_gb300 import caseinfo
    opts = caseinfo.solver_options(caseinfo.parse_info(
        "LinearAlgebra\n{\n pEqn\n {\n  innerPreconditioner RILUK\n"
        "  iluFill 2\n  tolerance 1e-10\n }\n}\n"), "pEqn")
    assert opts["ilu_fill"] == 2
    eqn = _tri_eqn(pg, 24, 20)
    s = pg.SparseMatrixSolver(**opts)
    s.set_eqn(eqn)
    assert s.solve() <= 1e-10
    with pytest.raises(Exception):
        pg.SparseMatrixSolver(ilu_fill=9)
