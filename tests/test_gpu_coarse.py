"""Two-level Schwarz preconditioner (cfg.coarse = 1): the one-level
Schwarz ILU(0) plus the coarse correction Z A_c^-1 Z^T on the space of
subdomain-constant vectors (Nicolaides), A_c = Z^T A Z.

Parity: the device application against the oracle's Schwarz ILU(0) sweeps
plus Z X Z^T, with X the device's coarse inverse, to 1e-12 relative (FP64;
1e-10 float-float); X itself, an FP32 Gauss-Jordan inverse, against the
coarse matrix A_c assembled here from the device's own partition
(||X A_c - I||_2 < 0.05), and the operator's linearity.  Solves: the FP64
true residual meets the tolerance, and the coarse space cuts the iteration
count of the high-contrast rising-bubble system."""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes, workloads

pytestmark = pytest.mark.gpu


def _bubble(pg, nx, ny):
    w = workloads.rising_bubble(nx, ny, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, ny, seed=3, faces=m.faces(), cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    return m, w, pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])


def _coarse(rp, ci, v, part, nparts):
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n))
    Z = sp.csr_matrix((np.ones(n), (np.arange(n), part)), shape=(n, nparts))
    return Z, (Z.T @ A @ Z).toarray()


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mesh", ["bubble", "tri"])
def test_two_level_apply_matches_oracle(pg, oracle, precision, mesh, variant):
    """variant 1: additive, z = B r + Z X Z^T r; variant 2: deflated
    (A-DEF1), z = B (r - A Z y) + Z y with y = X Z^T r."""
    if mesh == "bubble":
        m, w, eqn = _bubble(pg, 128, 96)
        sub = 256
    else:
        nodes, cptr, cind = meshes.triangulated(70, 60, 1.0, 1.0,
                                                jitter=0.25, seed=9)
        m = pg.Mesh(nodes, cptr, cind)
        om = oracle.OracleMesh(nodes, cptr, cind)
        f = om.faces()
        bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)  # FIXED walls
        rng = np.random.default_rng(2)
        eqn = pg.fv.laplacian(rng.uniform(0.5, 2.0, om.n_faces), m, bc,
                              rng.standard_normal(om.n_faces),
                              rng.standard_normal((om.n_faces, 2)))
        sub = 128
    rp, ci, v, rhs = eqn.export()
    keep = ci >= 0
    n = len(rp) - 1
    s = pg.SparseMatrixSolver(subdomain_rows=sub, coarse=variant,
                              precision=pg.FP64 if precision == "fp64" else pg.MIXED)
    s.set_eqn(eqn)
    part, nparts = s.partition()
    assert nparts > 4
    # the CrsEquation slots without placeholders, in CSR form
    rows = np.repeat(np.arange(n), np.diff(rp))[keep]
    A = sp.csr_matrix((v[keep], (rows, ci[keep])), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    arp, aci, av = A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data
    lu, rc = oracle.ilu0(arp, aci, av, part)
    assert rc == 0
    rng = np.random.default_rng(5)
    r1, r2 = rng.standard_normal(n), -rhs
    z1, z2 = s.apply_precond(r1), s.apply_precond(r2)
    # the coarse inverse is FP32 Gauss-Jordan: close to A_c^-1 ...
    Z, Ac = _coarse(arp, aci, av, part, nparts)
    X = s.coarse_inverse().astype(np.float64)
    err = np.linalg.norm(X @ Ac - np.eye(nparts), 2)
    print("||X A_c - I||_2 =", err)
    assert err < 0.05
    # ... and applied exactly (FP64): the operator is the oracle's ILU(0)
    # sweeps plus Z X Z^T
    tol = 1e-12 if precision == "fp64" else 1e-10
    AZ = sp.csr_matrix((av, aci, arp), shape=(n, n)) @ Z
    for r, z in ((r1, z1), (r2, z2)):
        y = X @ (Z.T @ r)
        if variant == 1:
            zo = oracle.ilu0_apply(arp, aci, lu, r, part) + Z @ y
        else:
            zo = oracle.ilu0_apply(arp, aci, lu, r - AZ @ y, part) + Z @ y
        assert np.all(np.isfinite(z))
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < tol
    # a fixed linear operator
    z12 = s.apply_precond(0.75 * r1 - 2.0 * r2)
    assert np.linalg.norm(z12 - (0.75 * z1 - 2.0 * z2)) / np.linalg.norm(z12) < tol


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_level_solve_converges_faster(pg, precision, variant):
    m, w, eqn = _bubble(pg, 256, 256)
    rp, ci, v, rhs = eqn.export()
    keep = ci >= 0
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))[keep]
    A = sp.csr_matrix((v[keep], (rows, ci[keep])), shape=(n, n))
    b = -rhs
    its = {}
    for coarse in (0, variant):
        s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000, coarse=coarse,
                                  precision=pg.FP64 if precision == "fp64" else pg.MIXED)
        s.set_eqn(eqn)
        s.solve()
        assert s.stats.status == pg.PG_OK
        x = s.x()
        assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.01e-8
        its[coarse] = s.nIters()
    print("iterations one-level / two-level:", its)
    assert its[variant] < its[0]


def test_two_level_singular_cavity(pg):
    """The lid-driven cavity's pCorr system is singular (normal-gradient p on
    every wall): the coarse matrix inherits the constant null vector, whose
    vanishing pivot the elimination drops.  The two-level solve converges
    and agrees with the one-level one up to the constant."""
    from phase_gb300 import simple
    out = simple.simple_pcorr(pg)
    xs = {}
    for coarse in (0, 1):
        s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=5000,
                                  subdomain_rows=512, coarse=coarse)
        s.set_eqn(out["eqn"])
        err = s.solve()
        assert s.stats.status == pg.PG_OK and err <= 1e-8, s.stats.as_dict()
        x = s.x()
        xs[coarse] = x - x.mean()
    d = xs[1] - xs[0]
    assert np.linalg.norm(d) / np.linalg.norm(xs[0]) < 1e-5


def test_two_level_gcib_and_cylinder(pg):
    """Non-symmetric ghost-cell IB rows and the 500k-triangle cylinder: the
    two-level solves meet 1e-8 on the FP64 true residual in both precisions,
    in fewer iterations than one-level."""
    from phase_gb300 import simple
    sp_ = workloads.gcib_specs(1, seed=5, min_cells=40_000, max_cells=40_000)[0]
    w = workloads.gcib_case(sp_)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.gcib_case(sp_, m.faces())
    e = pg.Equation(m, pg.GAMMA_SCALAR, w["bc_type"], ib_circles=[w["circle"]])
    e.assemble(gamma_scalar=w["gamma"], bc_value=w["bc_value"], u_face=w["u"])
    cyl = simple.cylinder_pcorr(pg)
    for eqn in (e, cyl["eqn"]):
        rp, ci, v, rhs = eqn.export()
        A = sp.csr_matrix((v, ci, rp))
        its = {}
        for coarse in (0, 1):
            for prec in (pg.FP64, pg.MIXED):
                s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                          coarse=coarse, precision=prec)
                s.set_eqn(eqn)
                err = s.solve()
                assert s.stats.status == pg.PG_OK and err <= 1e-8
                x = s.x()
                assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-8
                its[(coarse, prec)] = s.nIters()
        print("iterations (coarse, precision):", its)
        assert its[(1, pg.FP64)] < its[(0, pg.FP64)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coarse_inverse_reuse_sequence(pg, precision):
    """cfg.coarse_warm = -2: each solve of a time sequence applies the
    previous factorisation's coarse inverse while the new one is built
    beside it (double-buffered).  Every solve still meets the tolerance on
    the FP64 true residual, and a join makes the newest inverse current:
    after the last step the solver's inverse is bit-identical to that of a
    fresh solver on the last system."""
    pytest.importorskip("torch")
    from phase_gb300 import guess
    seq = guess.BubbleSequence(nx=256, seed=3)
    prec = pg.FP64 if precision == "fp64" else pg.MIXED
    s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000, coarse=2,
                              coarse_warm=-2, precision=prec)
    x = None
    for t in (100, 101, 102, 103):
        eqn = seq.assemble(t)
        rp, ci, v, rhs = eqn.export()
        keep = ci >= 0
        n = len(rp) - 1
        rows = np.repeat(np.arange(n), np.diff(rp))[keep]
        A = sp.csr_matrix((v[keep], (rows, ci[keep])), shape=(n, n))
        s.set_eqn(eqn)
        s.setGuess(x)
        s.solve()
        assert s.stats.status == pg.PG_OK
        x = s.x()
        b = -rhs
        assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.01e-8
    X = s.coarse_inverse()
    f = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000, coarse=2,
                              precision=prec)
    f.set_eqn(eqn)
    f.solve()
    np.testing.assert_array_equal(X, f.coarse_inverse())
