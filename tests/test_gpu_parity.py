"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle
on the same seeded inputs.

Bars: mesh geometry, face coefficients, gradients, the CSR pattern and the
off-diagonal coefficients are bit-exact (integer/index work and identically
rounded FP64 arithmetic); diagonals and right-hand sides, which the
face-coloured scatter accumulates in colour order rather than link order,
agree to 1e-14 relative to the row's coefficient scale; solutions agree with
the oracle's to 1e-9 relative when both are converged to 1e-12, and every
solve's true FP64 residual ||b - A x|| / ||b|| meets its tolerance.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes, workloads
import golden_cases

pytestmark = pytest.mark.gpu

ROW_TOL = 1e-14


def mesh_cases():
    return {
        "rect": meshes.rectilinear(12, 9, 1.5, 2.0),
        "tri": meshes.triangulated(9, 7, 1.0, 1.0, jitter=0.25, seed=4),
    }


@pytest.fixture(scope="module", params=["rect", "tri"])
def case(request, pg, oracle):
    nodes, cptr, cind = mesh_cases()[request.param]
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    rng = np.random.default_rng(11)
    f = om.faces()
    nf = om.n_faces
    bc = np.where(f["rcell"] < 0, rng.integers(0, 3, nf), 1).astype(np.int32)
    bv = rng.standard_normal(nf)
    u = rng.standard_normal((nf, 2))
    gamma = rng.uniform(0.1, 3.0, nf)
    return dict(name=request.param, m=m, om=om, bc=bc, bv=bv, u=u, gamma=gamma)


def test_mesh_matches_oracle_bitwise(case):
    m, om = case["m"], case["om"]
    assert (m.n_cells, m.n_faces, m.n_interior, m.n_boundary) == \
        (om.n_cells, om.n_faces, om.n_interior, om.n_boundary)
    a, b = m.faces(), om.faces()
    for k in ("lcell", "rcell", "fx", "fy", "nx", "ny"):
        assert np.array_equal(a[k], b[k]), k
    a, b = m.cells(), om.cells()
    for k in ("cx", "cy", "vol"):
        assert np.array_equal(a[k], b[k]), k


def _check_rows(rp, ci, v, rhs, rpo, cio, vo, rhso):
    assert np.array_equal(rp, rpo), "row_ptr"
    assert np.array_equal(ci, cio), "col_ind (order within rows included)"
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    off = ci != rows
    assert np.array_equal(v[off], vo[off]), "off-diagonal coefficients"
    scale = np.maximum(np.add.reduceat(np.abs(vo), rp[:-1]), 1e-300)
    d = ~off
    assert np.all(np.abs(v[d] - vo[d]) <= ROW_TOL * scale[rows[d]])
    return scale


@pytest.mark.parametrize("kind", ["scalar", "face"])
@pytest.mark.parametrize("with_u", [False, True])
def test_assembly_matches_oracle(case, pg, kind, with_u):
    m, om = case["m"], case["om"]
    g = 1.3 if kind == "scalar" else case["gamma"]
    u = case["u"] if with_u else None
    eqn = pg.fv.laplacian(g, m, case["bc"], case["bv"], u)
    rp, ci, v, rhs = eqn.export()
    rpo, cio, vo, rhso = om.laplacian(g, case["bc"], case["bv"], u)
    _check_rows(rp, ci, v, rhs, rpo, cio, vo, rhso)
    # rhs terms: sum of |contributions| bounds the rounding of the sum
    f = om.faces()
    mag = np.zeros(om.n_cells)
    if with_u:
        flux = np.abs(u[:, 0] * f["nx"]) + np.abs(u[:, 1] * f["ny"])
        np.add.at(mag, f["lcell"], flux)
        inter = f["rcell"] >= 0
        np.add.at(mag, f["rcell"][inter], flux[inter])
    mag += np.abs(rhso) + 1e-300
    assert np.all(np.abs(rhs - rhso) <= 4 * ROW_TOL * mag)


@pytest.mark.parametrize("name", golden_cases.CASES)
def test_device_assembly_matches_reference_golden(pg, name):
    """The device assembly against the output of the reference's own
    CrsEquation (tests/golden, five seeded cases, one with a row grown past
    five slots): pattern, column order and off-diagonal coefficients
    bit-exact; diagonal and rhs to the bars of the oracle comparison."""
    z, gamma, u = golden_cases.load(name)
    m = pg.Mesh(z["nodes"], z["cptr"], z["cind"])
    eqn = pg.fv.laplacian(gamma, m, z["bc_type"], z["bc_value"], u)
    rp, ci, v, rhs = eqn.export()
    rpo, cio, vo, rhso = golden_cases.compact(z)
    _check_rows(rp, ci, v, rhs, rpo, cio, vo, rhso)
    mag = np.abs(rhso) + 1e-300
    if u is not None:
        f = m.faces()
        flux = np.abs(u[:, 0] * f["nx"]) + np.abs(u[:, 1] * f["ny"])
        np.add.at(mag, f["lcell"], flux)
        inter = f["rcell"] >= 0
        np.add.at(mag, f["rcell"][inter], flux[inter])
    assert np.all(np.abs(rhs - rhso) <= 4 * ROW_TOL * mag)


def test_assembly_is_deterministic_and_reassembles(case, pg):
    m = case["m"]
    eqn = pg.Equation(m, pg.GAMMA_FACE, case["bc"])
    eqn.assemble(gamma_face=case["gamma"], bc_value=case["bv"], u_face=case["u"])
    a = eqn.export()
    eqn.assemble(gamma_face=2.0 * case["gamma"], bc_value=case["bv"])
    eqn.assemble(gamma_face=case["gamma"], bc_value=case["bv"], u_face=case["u"])
    b = eqn.export()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_face_coefficients_and_gradient_bitwise(case, pg):
    m, om = case["m"], case["om"]
    c = om.cells()
    gamma = np.clip(np.sin(7 * c["cx"]) + c["cy"], 0, 1)
    a = m.dt_over_rho(gamma, 1000.0, 1.0, 1e-4)
    b = om.dt_over_rho(gamma, 1000.0, 1.0, 1e-4)
    assert np.array_equal(a, b)
    f = om.faces()
    phi = np.cos(3 * c["cx"]) * c["cy"]
    pf = np.cos(3 * f["fx"]) * f["fy"]
    gf, gc = m.gradient(phi, pf)
    gfo, gco = om.gradient(phi, pf)
    assert np.array_equal(gf, gfo) and np.array_equal(gc, gco)


def _system(om, seed=3, gamma_face=True):
    f = om.faces()
    rng = np.random.default_rng(seed)
    bc = np.where(f["rcell"] < 0, 1, 1).astype(np.int32)
    bc[np.flatnonzero(f["rcell"] < 0)[::3]] = 0
    gamma = rng.uniform(0.2, 5.0, om.n_faces) if gamma_face else 1.0
    return om.laplacian(gamma, bc, np.zeros(om.n_faces),
                        rng.standard_normal((om.n_faces, 2)))


@pytest.mark.parametrize("sub_rows", [-1, 16, 0])
def test_solver_matches_oracle(case, pg, oracle, sub_rows):
    om = case["om"]
    rp, ci, v, rhs = _system(om)
    b = -rhs
    s = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=5000,
                              subdomain_rows=sub_rows)
    s.setRank(om.n_cells)
    s.set(rp, ci, v)
    s.setRhs(b)
    err = s.solve()
    assert s.stats.status == pg.PG_OK and err <= 1e-12
    x = s.x()
    part, nparts = s.partition()
    xo, st = oracle.bicgstab(rp, ci, v, b, tol=1e-12, max_iters=5000,
                             part=part)
    assert st["status"] == 0
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9
    # same preconditioner, same algorithm: iteration counts agree closely
    assert abs(s.nIters() - st["iters"]) <= max(2, 0.1 * st["iters"])
    A = sp.csr_matrix((v, ci, rp))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.01e-12


def _bubble_system(pg, nx, ny):
    w = workloads.rising_bubble(nx, ny, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, ny, seed=3, faces=m.faces(),
                                cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    eqn = pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])
    return eqn.export()


@pytest.mark.parametrize("precision", ["fp64", "mixed-steps", "mixed-blobs"])
@pytest.mark.parametrize("mesh", ["bubble", "tri", "bubble-xy"])
def test_ilu_apply_matches_oracle(pg, oracle, precision, mesh):
    """The Schwarz ILU(0) sweeps alone, z = M^-1 r, against the oracle's
    factor and triangular solves on the device's own partition.  FP64:
    1e-12 relative (the factor's FP64 operation order differs); float-float
    factors and sweeps (about 48-bit arithmetic): 1e-10 relative.
    bubble-xy: subdomains cut by cell-centre bisection into 8 x 16 blocks,
    swept two per warp."""
    xy = None
    if mesh == "bubble-xy":
        w = workloads.rising_bubble(128, 96, seed=3)
        m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
        c = m.cells()
        xy = np.stack([c["cx"], c["cy"]], axis=1)
        rp, ci, v, rhs = _bubble_system(pg, 128, 96)
        sub = 128
    elif mesh == "bubble":
        rp, ci, v, rhs = _bubble_system(pg, 128, 96)
        sub = 1024
    else:
        nodes, cptr, cind = meshes.triangulated(70, 60, 1.0, 1.0,
                                                jitter=0.25, seed=9)
        om = oracle.OracleMesh(nodes, cptr, cind)
        rp, ci, v, rhs = _system(om)
        sub = 512
    n = len(rp) - 1
    s = pg.SparseMatrixSolver(
        subdomain_rows=sub,
        precision=pg.FP64 if precision == "fp64" else pg.MIXED,
        mixed_sweep={"fp64": 0, "mixed-steps": 1, "mixed-blobs": 2}[precision])
    s.setRank(n)
    if xy is not None:
        s.set_row_coords(xy)
    s.set(rp, ci, v)
    part, nparts = s.partition()
    assert nparts > 4
    lu, rc = oracle.ilu0(rp, ci, v, part)
    assert rc == 0
    rng = np.random.default_rng(5)
    tol = 1e-12 if precision == "fp64" else 1e-10
    for r in (rng.standard_normal(n), -rhs):
        z = s.apply_precond(r)
        zo = oracle.ilu0_apply(rp, ci, lu, r, part)
        assert np.all(np.isfinite(z))
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < tol


def test_solver_accepts_crsequation_slots(case, pg, oracle):
    """set() receives CrsEquation's arrays with -1 placeholders
    (FiniteVolumeEquation.tpp:72)."""
    om = case["om"]
    rng = np.random.default_rng(5)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rps, cis, vs, rhs = om.laplacian(rng.uniform(1, 2, om.n_faces), bc,
                                     rng.standard_normal(om.n_faces),
                                     slots=True)
    assert np.any(cis < 0)
    s = pg.SparseMatrixSolver(tolerance=1e-10)
    s.setRank(om.n_cells)
    s.set(rps, cis, vs)
    s.setRhs(-rhs)
    assert s.solve() <= 1e-10
    keep = cis >= 0
    rows = np.repeat(np.arange(om.n_cells), np.diff(rps))
    A = sp.csr_matrix((vs[keep], (rows[keep], cis[keep])),
                      shape=(om.n_cells, om.n_cells))
    x = s.x()
    assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-10


@pytest.mark.parametrize("precond", [0, 1])
def test_other_preconditioners(case, pg, oracle, precond):
    om = case["om"]
    rp, ci, v, rhs = _system(om, gamma_face=False)
    s = pg.SparseMatrixSolver(tolerance=1e-10, max_iters=20000, precond=precond)
    s.setRank(om.n_cells)
    s.set(rp, ci, v)
    s.setRhs(-rhs)
    assert s.solve() <= 1e-10
    xo, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-12, max_iters=20000,
                             precond=precond)
    x = s.x()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-7


def test_mixed_precision_reaches_fp64_tolerance(case, pg, oracle):
    om = case["om"]
    rp, ci, v, rhs = _system(om)
    s = pg.SparseMatrixSolver(tolerance=1e-10, precision=pg.MIXED,
                              max_iters=5000)
    s.setRank(om.n_cells)
    s.set(rp, ci, v)
    s.setRhs(-rhs)
    err = s.solve()
    assert s.stats.status == pg.PG_OK and err <= 1e-10
    assert s.stats.outer_iters >= 2
    xo, _ = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-13, max_iters=5000)
    x = s.x()
    # error vs the FP64 oracle, stated: bounded by the residual tolerance
    # times the conditioning of these small systems
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-7


def test_warm_start_and_determinism(case, pg):
    om = case["om"]
    rp, ci, v, rhs = _system(om)
    s = pg.SparseMatrixSolver(tolerance=1e-10)
    s.setRank(om.n_cells)
    s.set(rp, ci, v)
    s.setRhs(-rhs)
    s.solve()
    x1 = s.x()
    it1 = s.nIters()
    # Belos keeps x_ between solves: the same system converges at once
    s.set(rp, ci, v)
    s.setRhs(-rhs)
    s.solve()
    assert s.nIters() == 0
    # a fresh zero guess reproduces the first solve bit for bit
    s.setGuess(np.zeros(om.n_cells))
    s.solve()
    assert s.nIters() == it1
    assert np.array_equal(s.x(), x1)


def test_edge_cases(pg):
    nodes, cptr, cind = meshes.rectilinear(6, 6)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    eqn = pg.fv.laplacian(1.0, m, bc, np.zeros(m.n_faces))
    s = pg.SparseMatrixSolver()
    s.set_eqn(eqn)
    # zero rhs: x = 0, converged
    assert s.solve() == 0.0 and s.stats.status == pg.PG_OK
    assert np.all(s.x() == 0.0)
    rp, ci, v, _ = eqn.export()
    # non-finite rhs is reported, not hidden
    s2 = pg.SparseMatrixSolver()
    s2.setRank(m.n_cells)
    s2.set(rp, ci, v)
    b = np.ones(m.n_cells)
    b[3] = np.nan
    s2.setRhs(b)
    s2.solve()
    assert s2.stats.status == pg.PG_NON_FINITE
    # max iterations
    s3 = pg.SparseMatrixSolver(max_iters=1, tolerance=1e-14)
    s3.setRank(m.n_cells)
    s3.set(rp, ci, v)
    s3.setRhs(np.random.default_rng(0).standard_normal(m.n_cells))
    s3.solve()
    assert s3.stats.status == pg.PG_MAX_ITERS and s3.nIters() == 1
    # bad arguments
    with pytest.raises(pg.PhaseError):
        pg.SparseMatrixSolver(tolerance=-1.0)
    s4 = pg.SparseMatrixSolver()
    s4.setRank(3)
    with pytest.raises(pg.PhaseError):
        s4.setRhs(np.ones(3))  # no matrix yet
    with pytest.raises(pg.PhaseError):
        pg.Equation(m, pg.GAMMA_SCALAR, np.full(m.n_faces, 7, np.int32))
    # zero pivot: an all-zero row
    v0 = v.copy()
    v0[rp[5]:rp[6]] = 0.0
    s5 = pg.SparseMatrixSolver()
    s5.setRank(m.n_cells)
    s5.set(rp, ci, v0)
    s5.setRhs(np.ones(m.n_cells))
    s5.solve()
    assert s5.stats.status in (pg.PG_BREAKDOWN, pg.PG_NON_FINITE,
                               pg.PG_MAX_ITERS)


def test_singular_neumann_system_consistent_rhs(pg, oracle):
    """All-NORMAL_GRADIENT pressure (the lid-driven cavity): A is singular
    with the constants as null space; a consistent rhs still converges and
    the solution matches the oracle's up to a constant."""
    nodes, cptr, cind = meshes.rectilinear(20, 20)
    om = oracle.OracleMesh(nodes, cptr, cind)
    bc = np.ones(om.n_faces, np.int32)
    rp, ci, v, _ = om.laplacian(1.0, bc, np.zeros(om.n_faces))
    rng = np.random.default_rng(2)
    b = rng.standard_normal(om.n_cells)
    b -= b.mean()
    s = pg.SparseMatrixSolver(tolerance=1e-9, max_iters=2000)
    s.setRank(om.n_cells)
    s.set(rp, ci, v)
    s.setRhs(b)
    s.solve()
    x = s.x()
    A = sp.csr_matrix((v, ci, rp))
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1e-8
    xo, st = oracle.bicgstab(rp, ci, v, b, tol=1e-11, max_iters=5000)
    d = (x - x.mean()) - (xo - xo.mean())
    assert np.linalg.norm(d) / np.linalg.norm(xo - xo.mean()) < 1e-6


def test_pattern_change_is_detected(pg):
    s = pg.SparseMatrixSolver(tolerance=1e-10)
    for nx in (5, 5, 6):
        nodes, cptr, cind = meshes.rectilinear(nx, 4)
        m = pg.Mesh(nodes, cptr, cind)
        f = m.faces()
        bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
        rp, ci, v, _ = pg.fv.laplacian(1.0, m, bc, np.zeros(m.n_faces)).export()
        s.setRank(m.n_cells)
        s.set(rp, ci, v)
        b = np.arange(m.n_cells, dtype=float)
        s.setRhs(b)
        assert s.solve() <= 1e-10
        A = sp.csr_matrix((v, ci, rp))
        assert np.linalg.norm(b - A @ s.x()) / np.linalg.norm(b) <= 1.01e-10


@pytest.mark.parametrize("precision,sub_rows",
                         [("fp64", 0), ("mixed", 0), ("fp64", 2048),
                          ("mixed", 512)])
def test_rising_bubble_full_size_properties(pg, oracle, precision, sub_rows):
    """1024x1024 rising-bubble system: pattern bit-exact with the oracle,
    1000x coefficient contrast, and the device solve's true residual meets
    1e-8 in FP64 and with FP32 ILU factors, for several Schwarz subdomain
    sizes (size-independent properties; the full oracle solve is too
    slow)."""
    nx = ny = 1024
    w = workloads.rising_bubble(nx, ny, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, ny, seed=3, faces=m.faces(),
                                cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    assert coeff.max() / coeff.min() == pytest.approx(1000.0, rel=1e-9)
    eqn = pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])
    rp, ci, v, rhs = eqn.export()
    n_if = nx * (ny - 1) + ny * (nx - 1)
    assert len(ci) == nx * ny + 2 * n_if == 5238784
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    rpo, cio, vo, rhso = om.laplacian(coeff, w["bc_type"], w["bc_value"], w["u"])
    _check_rows(rp, ci, v, rhs, rpo, cio, vo, rhso)
    s = pg.SparseMatrixSolver(
        tolerance=1e-8, max_iters=8000, subdomain_rows=sub_rows,
        precision=pg.MIXED if precision == "mixed" else pg.FP64)
    s.set_eqn(eqn)
    err = s.solve()
    assert s.stats.status == pg.PG_OK and err <= 1e-8
    A = sp.csr_matrix((vo, cio, rpo))
    x = s.x()
    assert np.linalg.norm(-rhso - A @ x) / np.linalg.norm(rhso) <= 1.01e-8
