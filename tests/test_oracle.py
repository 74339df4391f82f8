"""CPU tests of the oracle: known answers, the reference's own CrsEquation,
golden vectors and an independent scipy cross-check.  No GPU needed."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from phase_gb300 import meshes
import golden_cases
import refreplay


def rect(oracle, nx, ny, w=1.0, h=1.0):
    nodes, cptr, cind = meshes.rectilinear(nx, ny, w, h)
    return oracle.OracleMesh(nodes, cptr, cind)


def test_rectilinear_counts_and_numbering(oracle):
    om = rect(oracle, 5, 3, 1.0, 1.5)
    assert om.n_cells == 15
    assert om.n_interior == 4 * 3 + 5 * 2
    assert om.n_boundary == 2 * (5 + 3)
    f = om.faces()
    # FiniteVolumeGrid2D::createCell: cell 0 creates its 4 faces first, in
    # node order (0,1), (1,7), (7,6), (6,0)
    assert list(f["lnode"][:4]) == [0, 1, 7, 6]
    assert list(f["rnode"][:4]) == [1, 7, 6, 0]
    # normal = (dy, -dx) of rNode - lNode
    assert f["nx"][0] == 0.0 and f["ny"][0] == -0.2
    c = om.cells()
    assert np.allclose(c["vol"], 0.2 * 0.5)
    assert np.allclose(c["cx"][:5], 0.1 + 0.2 * np.arange(5))


@pytest.mark.parametrize("gamma", [1.0, 2.5])
def test_rectilinear_coefficients(oracle, gamma):
    nx, ny, w, h = 6, 4, 1.2, 2.0
    om = rect(oracle, nx, ny, w, h)
    hx, hy = w / nx, h / ny
    bc = np.ones(om.n_faces, np.int32)
    rp, ci, v, rhs = om.laplacian(gamma, bc, np.zeros(om.n_faces))
    for i in range(om.n_cells):
        row = dict(zip(ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]]))
        for j, a in row.items():
            if j == i:
                continue
            expect = gamma * hy / hx if abs(j - i) == 1 else gamma * hx / hy
            assert a == pytest.approx(expect, rel=1e-14)
        # all-Neumann rows sum to zero
        assert sum(row.values()) == pytest.approx(0.0, abs=1e-12 * gamma)
    assert np.all(rhs == 0.0)


def test_pattern_order_scalar_vs_face_gamma(oracle):
    om = rect(oracle, 3, 3)
    bc = np.ones(om.n_faces, np.int32)
    rp, ci, _, _ = om.laplacian(1.0, bc, np.zeros(om.n_faces))
    # scalar gamma: first neighbour, then diagonal (Laplacian.h:57-58)
    assert list(ci[rp[4]:rp[5]][:2]) != [4] and ci[rp[4] + 1] == 4
    rpf, cif, _, _ = om.laplacian(np.ones(om.n_faces), bc, np.zeros(om.n_faces))
    # face gamma: diagonal first (Laplacian.h:141-142)
    assert cif[rpf[4]] == 4
    assert sorted(cif[rpf[4]:rpf[5]]) == sorted(ci[rp[4]:rp[5]])


def test_laplacian_of_linear_field_is_zero_inside(oracle):
    """A phi + rhs = 0 for a linear phi with FIXED boundary values on a
    rectilinear mesh (two-point flux is exact for linear fields there)."""
    om2 = rect(oracle, 7, 5, 1.0, 1.0)
    c2, f2 = om2.cells(), om2.faces()
    phi2 = 2.0 * c2["cx"] - 3.0 * c2["cy"] + 1.0
    bc2 = np.zeros(om2.n_faces, np.int32)
    bv2 = 2.0 * f2["fx"] - 3.0 * f2["fy"] + 1.0
    rp, ci, v, rhs = om2.laplacian(1.0, bc2, bv2)
    A2 = sp.csr_matrix((v, ci, rp), shape=(om2.n_cells, om2.n_cells))
    assert np.max(np.abs(A2 @ phi2 + rhs)) < 1e-12


def _reference_crs(oracle, om, gamma, bc, bv, u=None):
    r = oracle.RefCrs(om.n_cells, 5)
    ops, rows, cols, vals = refreplay.laplacian_ops(om, gamma, bc, bv)
    r.apply(ops, rows, cols, vals)
    if u is not None:
        r.eq_vector(refreplay.div_u(om, u))
    return r.export()


@pytest.mark.parametrize("kind", ["scalar", "face"])
@pytest.mark.parametrize("mesh", ["rect", "tri"])
def test_slots_match_reference_crsequation(oracle, kind, mesh):
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent: oracle/_ref not built")
    if mesh == "rect":
        om = rect(oracle, 6, 5, 1.0, 2.0)
    else:
        om = oracle.OracleMesh(*meshes.triangulated(5, 4, 1.0, 1.0, 0.2, 1))
    rng = np.random.default_rng(7)
    nf = om.n_faces
    f = om.faces()
    bc = np.where(f["rcell"] < 0, rng.integers(0, 2, nf), 1).astype(np.int32)
    bv = rng.standard_normal(nf)
    gamma = 1.7 if kind == "scalar" else rng.uniform(0.0, 2.0, nf)
    if kind == "face":
        gamma[::7] = 0.0  # explicit zero coefficients are kept
    u = rng.standard_normal((nf, 2))
    ref = _reference_crs(oracle, om, gamma, bc, bv, u)
    mine = om.laplacian(gamma, bc, bv, u, slots=True)
    for a, b in zip(ref, mine):
        assert a.shape == b.shape
        assert np.array_equal(a, b), "oracle differs from CrsEquation.cpp"


def test_row_growth_past_five_slots_matches_reference(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent")
    # a hexagon-fan mesh: the centre cell has 6 neighbours (7 entries)
    ang = np.linspace(0, 2 * np.pi, 7)[:-1]
    ring = np.stack([np.cos(ang), np.sin(ang)], 1)
    outer = 2.0 * np.stack([np.cos(ang + np.pi / 6), np.sin(ang + np.pi / 6)], 1)
    nodes = np.vstack([ring, outer])
    cells = [list(range(6))]
    for k in range(6):
        a, b = k, (k + 1) % 6
        cells.append([a, 6 + k, b])
    cptr = np.cumsum([0] + [len(c) for c in cells]).astype(np.int64)
    cind = np.array(sum(cells, []), np.int64)
    om = oracle.OracleMesh(nodes, cptr, cind)
    bc = np.ones(om.n_faces, np.int32)
    ref = _reference_crs(oracle, om, 1.0, bc, np.zeros(om.n_faces))
    mine = om.laplacian(1.0, bc, np.zeros(om.n_faces), slots=True)
    assert ref[0][1] - ref[0][0] == 7
    for a, b in zip(ref, mine):
        assert np.array_equal(a, b)


def test_golden_fixtures_present():
    """tests/golden holds the reference CrsEquation's output for the five
    seeded cases of tests/golden/make_golden.py."""
    assert len(golden_cases.CASES) >= 5


def test_golden_fixtures_regenerate_identically(oracle, tmp_path):
    """The committed fixtures are what tests/golden/make_golden.py writes
    from the reference's CrsEquation (where its sources can be built)."""
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent: oracle/_ref not built")
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(golden_cases.GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    names = []
    for name, mesh, kind, with_u in mg.cases():
        mg.make(name, mesh, kind, with_u, out_dir=str(tmp_path))
        names.append(name)
    assert sorted(names) == golden_cases.CASES
    for name in names:
        a = np.load(os.path.join(golden_cases.GOLDEN, name + ".npz"))
        b = np.load(os.path.join(str(tmp_path), name + ".npz"))
        assert sorted(a.files) == sorted(b.files)
        for k in a.files:
            assert np.array_equal(a[k], b[k]), (name, k)


@pytest.mark.parametrize("name", golden_cases.CASES)
def test_oracle_matches_reference_golden(oracle, name):
    """The oracle reproduces the fixtures the reference's own CrsEquation
    wrote (slot arrays, placeholders and the rows grown past five slots
    included) bit for bit, and its compact form is those arrays without
    the placeholders."""
    z, gamma, u = golden_cases.load(name)
    om = oracle.OracleMesh(z["nodes"], z["cptr"], z["cind"])
    ref = (z["row_ptr"], z["col_ind"], z["vals"], z["rhs"])
    mine = om.laplacian(gamma, z["bc_type"], z["bc_value"], u, slots=True)
    for a, b in zip(ref, mine):
        assert a.shape == b.shape
        assert np.array_equal(a, b), "oracle differs from the reference fixture"
    compact = om.laplacian(gamma, z["bc_type"], z["bc_value"], u)
    for a, b in zip(golden_cases.compact(z), compact):
        assert np.array_equal(a, b)


def test_reference_plus_drops_zeros_and_placeholders(oracle):
    """CrsEquation::operator+= (CrsEquation.cpp:185-229) rebuilds the CSR
    without zero values and -1 slots: the semantics GCIB rows rely on."""
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent")
    a = oracle.RefCrs(3, 5)
    a.apply([0, 0, 0, 0], [0, 0, 1, 2], [0, 1, 1, 2], [2.0, 0.0, 3.0, 4.0])
    b = oracle.RefCrs(3, 5)
    b.apply([0, 0], [0, 2], [2, 0], [5.0, 6.0])
    a.plus(b)
    rp, ci, v, _ = a.export()
    assert list(rp) == [0, 2, 3, 5]
    assert list(ci) == [0, 2, 1, 2, 0]
    assert list(v) == [2.0, 5.0, 3.0, 4.0, 6.0]


def test_dt_over_rho_and_interpolation(oracle):
    om = rect(oracle, 4, 4)
    c = om.cells()
    g = np.clip(c["cx"] * 1.3 - 0.1, 0.0, 1.0)
    gf = om.interpolate_faces(g)
    f = om.faces()
    inter = f["rcell"] >= 0
    # equal spacing: distance weight 1/2
    expect = 0.5 * g[f["lcell"][inter]] + 0.5 * g[f["rcell"][inter]]
    assert np.allclose(gf[inter], expect, rtol=0, atol=1e-15)
    assert np.array_equal(gf[~inter], g[f["lcell"][~inter]])
    co = om.dt_over_rho(g, 1000.0, 1.0, 1e-4)
    rho = 1000.0 + np.clip(gf, 0, 1) * (1.0 - 1000.0)
    assert np.allclose(co, 1e-4 / rho, rtol=1e-15)


def test_gradient_of_linear_field(oracle):
    om = rect(oracle, 6, 6)
    c, f = om.cells(), om.faces()
    phi = 3.0 * c["cx"] - 2.0 * c["cy"]
    pf = 3.0 * f["fx"] - 2.0 * f["fy"]
    gf, gc = om.gradient(phi, pf)
    assert np.allclose(gc[:, 0], 3.0, atol=1e-12)
    assert np.allclose(gc[:, 1], -2.0, atol=1e-12)


def _poisson_system(oracle, nx, ny, seed=0):
    om = rect(oracle, nx, ny, 1.0, 1.0)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)  # FIXED walls
    rng = np.random.default_rng(seed)
    gamma = rng.uniform(0.5, 2.0, om.n_faces)
    rp, ci, v, rhs = om.laplacian(gamma, bc, np.zeros(om.n_faces))
    b = rng.standard_normal(om.n_cells)
    return rp, ci, v, b


@pytest.mark.parametrize("precond", [0, 1, 2, 3])
def test_bicgstab_matches_scipy_direct(oracle, precond):
    rp, ci, v, b = _poisson_system(oracle, 24, 20)
    x, st = oracle.bicgstab(rp, ci, v, b, tol=1e-10, max_iters=2000,
                            precond=precond, ilut_fill=5)
    assert st["status"] == 0
    A = sp.csr_matrix((v, ci, rp))
    xd = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8
    assert st["rel_residual"] <= 1e-10


def test_threaded_bicgstab_is_reproducible(oracle):
    """The oracle's dot products sum fixed per-thread chunks in thread order,
    so a threaded solve repeats bit for bit (the CPU baseline's iteration
    counts depend on it)."""
    rp, ci, v, b = _poisson_system(oracle, 60, 50)
    n = len(rp) - 1
    part = (np.arange(n) * 4 // n).astype(np.int32)
    runs = [oracle.bicgstab(rp, ci, v, b, tol=1e-13, max_iters=60, part=part,
                            threads=4) for _ in range(3)]
    for x, st in runs[1:]:
        assert st["iters"] == runs[0][1]["iters"]
        assert np.array_equal(x, runs[0][0])


def test_history_from_a_guess(oracle):
    """The residual-history solve from an initial guess: from the exact
    solution it starts at (nearly) zero residual; from a perturbed one it
    starts at the perturbation's residual and follows the full solve's
    iteration from the same guess."""
    rp, ci, v, b = _poisson_system(oracle, 30, 24)
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n))
    xs = spla.spsolve(A.tocsc(), b)
    h, _, _ = oracle.bicgstab_history(rp, ci, v, b, 5, x0=xs)
    assert h[0] < 1e-12
    x0 = xs + 1e-3 * np.random.default_rng(3).standard_normal(n)
    h0, _, _ = oracle.bicgstab_history(rp, ci, v, b, 5)
    h1, _, _ = oracle.bicgstab_history(rp, ci, v, b, 5, x0=x0)
    r0 = np.linalg.norm(b - A @ x0) / np.linalg.norm(b)
    assert abs(h1[0] - r0) <= 1e-12 * max(r0, 1.0)
    assert h1[0] < 1e-2 < h0[0]


def test_ilu0_matches_scipy_spilu_pattern_zero_fill(oracle):
    """ILU(0) factors satisfy (L U)_ij = a_ij on the pattern of A."""
    rp, ci, v, _ = _poisson_system(oracle, 9, 7)
    lu, rc = oracle.ilu0(rp, ci, v)
    assert rc == 0
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
    F = sp.csr_matrix((lu, ci, rp), shape=(n, n)).toarray()
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    P = L @ U
    mask = A != 0
    assert np.allclose(P[mask], A[mask], rtol=1e-12, atol=1e-12)


def test_schwarz_ilu0_blocks_are_independent(oracle):
    rp, ci, v, b = _poisson_system(oracle, 16, 16)
    n = len(rp) - 1
    part = (np.arange(n) // 64).astype(np.int32)
    x, st = oracle.bicgstab(rp, ci, v, b, tol=1e-10, part=part)
    assert st["status"] == 0
    lu, rc = oracle.ilu0(rp, ci, v, part)
    # entries that couple two subdomains are dropped from the factor
    rows = np.repeat(np.arange(n), np.diff(rp))
    cross = part[rows] != part[ci]
    assert np.all(lu[cross] == 0.0)


def test_momentum_operator_known_answers(oracle):
    """ddt + div - laplacian(nu): with no flux the x and y blocks equal
    V/dt I - L(nu) with L the scalar Laplacian (FIXED walls), and the lid
    value enters the x rhs only."""
    from phase_gb300 import simple
    w = simple.cavity_inputs(6, 5)
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    w = simple.cavity_inputs(6, 5, faces=om.faces())
    n = om.n_cells
    rp, ci, v, rhs = om.momentum(0.005, 0.01, 1.0, np.zeros((n, 2)),
                                 w["u_face"], w["bc_u"])
    A = sp.csr_matrix((v, ci, rp), shape=(2 * n, 2 * n)).toarray()
    rpl, cil, vl, rhsl = om.laplacian(0.01, w["bc_u"], w["u_face"][:, 0])
    L = sp.csr_matrix((vl, cil, rpl), shape=(n, n)).toarray()
    vol = om.cells()["vol"]
    expect = np.diag(vol / 0.005) - L
    assert np.allclose(A[:n, :n], expect, rtol=1e-14, atol=1e-14)
    assert np.allclose(A[n:, n:], expect, rtol=1e-14, atol=1e-14)
    assert np.all(A[:n, n:] == 0) and np.all(A[n:, :n] == 0)
    assert np.allclose(rhs[:n], -rhsl, rtol=1e-14, atol=1e-14)
    assert np.all(rhs[n:] == 0.0) and np.any(rhs[:n] != 0.0)


def test_projection_property_of_correct_velocity(oracle):
    """After fv::laplacian(dt/rho, p) == src::div(u*) is solved (scipy direct)
    and u* is corrected with the face gradient (FractionalStep::
    correctVelocity), src::div of the corrected face velocity vanishes."""
    from phase_gb300 import workloads
    w = workloads.rising_bubble(32, 32, seed=3)
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    f = om.faces()
    w = workloads.rising_bubble(32, 32, seed=3, faces=f, cells=om.cells())
    coeff = om.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    rp, ci, v, rhs = om.laplacian(coeff, w["bc_type"], w["bc_value"], w["u"])
    A = sp.csr_matrix((v, ci, rp), shape=(om.n_cells,) * 2)
    p = spla.spsolve(A.tocsc(), -rhs)
    bnd = f["rcell"] < 0
    p_face = np.zeros(om.n_faces)
    p_face[bnd] = np.where(w["bc_type"][bnd] == 0, w["bc_value"][bnd],
                           p[f["lcell"][bnd]])
    assert np.array_equal(p_face, om.set_boundary_faces(
        w["bc_type"], p, np.where(bnd, w["bc_value"], 0.0)))
    gf, gc = om.gradient(p, p_face)
    _, uf = om.correct_velocity(w["dt"], gc, gf, np.zeros((om.n_cells, 2)),
                                w["u"], None, w["dt"] / coeff)

    def div(u):
        return -om.laplacian(0.0, w["bc_type"], w["bc_value"], u)[3]

    assert np.abs(div(uf)).max() <= 1e-9 * np.abs(div(w["u"])).max()


@pytest.mark.parametrize("coarse", [1, 2])
def test_two_level_oracle_converges_in_fewer_iterations(oracle, coarse):
    """The oracle's two-level Schwarz ILU(0) (the device solver's algorithm,
    restated on the CPU for the algorithm-matched baseline) reaches 1e-8 on
    a 1000:1 rising-bubble system in a fraction of the one-level count."""
    from phase_gb300 import workloads
    nx = 96
    w = workloads.rising_bubble(nx, nx, seed=3)
    om = oracle.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, nx, seed=3, faces=om.faces(),
                                cells=om.cells())
    coeff = om.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    rp, ci, v, rhs = om.laplacian(coeff, w["bc_type"], w["bc_value"], w["u"])
    n = len(rp) - 1
    i, j = np.arange(n) % nx, np.arange(n) // nx
    part = ((j // 16) * (nx // 8) + i // 8).astype(np.int32)  # 8 x 16 blocks
    its = {}
    for c in (0, coarse):
        x, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-8, max_iters=20000,
                                part=part, coarse=c, threads=2)
        A = sp.csr_matrix((v, ci, rp))
        assert st["status"] == 0
        assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-8
        its[c] = st["iters"]
    assert its[coarse] < 0.5 * its[0], its


@pytest.mark.parametrize("krylov", [1, 2])
def test_oracle_tfqmr_and_gmres_solve(oracle, krylov):
    """The oracle's TFQMR and GMRES (Belos' other solvers in Phase's cases)
    with the Schwarz ILU(0) right preconditioner reach the tolerance on the
    true residual, and agree with scipy's direct solve."""
    nodes, cptr, cind = meshes.triangulated(30, 24, 1.0, 1.0, jitter=0.2,
                                            seed=3)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(4)
    rp, ci, v, rhs = om.laplacian(rng.uniform(1, 3, om.n_faces), bc,
                                  np.zeros(om.n_faces),
                                  rng.standard_normal((om.n_faces, 2)))
    n = len(rp) - 1
    part = (np.arange(n) * 4 // n).astype(np.int32)
    x, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-10, max_iters=2000,
                            part=part, krylov=krylov, krylov_dim=30)
    A = sp.csr_matrix((v, ci, rp))
    assert st["status"] == 0, st
    assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-10
    xd = spla.spsolve(A.tocsc(), -rhs)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8


def _dense_iluk_levels(A, k):
    """The level-of-fill pattern of ILU(k) by the textbook rule on a dense
    array (Saad, Iterative Methods for Sparse Linear Systems, sec. 10.3.3),
    an independent restatement for small cases."""
    n = A.shape[0]
    big = 10 ** 6
    lev = np.where(A != 0, 0, big)
    for i in range(n):
        for m in range(i):
            if lev[i, m] > k:
                continue
            for j in range(m + 1, n):
                if lev[m, j] <= k:
                    lev[i, j] = min(lev[i, j], lev[i, m] + lev[m, j] + 1)
    return lev <= k


@pytest.mark.parametrize("k", [0, 1, 2])
def test_iluk_is_exact_on_its_level_of_fill_pattern(oracle, k):
    """ILU(k): (L U)_ij = a_ij on the level-k pattern (from an independent
    dense restatement), and on the 5-point Poisson matrix ILU(0) equals the
    oracle's ILU(0) and ILU(1) adds the known fill diagonals at offsets
    +-(nx - 1)."""
    nx, ny = 9, 7
    rp, ci, v, _ = _poisson_system(oracle, nx, ny)
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
    mask = _dense_iluk_levels(A, k)
    # (L U)^-1 e_j column by column gives M^-1; M = L U
    Minv = np.stack([oracle.iluk_apply(rp, ci, v, e, k)[0] for e in np.eye(n)], 1)
    M = np.linalg.inv(Minv)
    assert np.allclose(M[mask], A[mask], rtol=1e-11, atol=1e-11)
    # L U has nothing outside the pattern's product closure; its pattern
    # holds the filled entries: with k = 1 the offsets +-(nx - 1) appear
    if k == 1:
        offs = {j - i for i, j in zip(*np.nonzero(mask))}
        assert offs == {0, 1, -1, nx, -nx, nx - 1, -(nx - 1)}
    if k == 0:
        lu, rc = oracle.ilu0(rp, ci, v)
        rng = np.random.default_rng(1)
        r = rng.standard_normal(n)
        z0 = oracle.ilu0_apply(rp, ci, lu, r)
        zk, rc = oracle.iluk_apply(rp, ci, v, r, 0)
        assert rc == 0 and np.allclose(zk, z0, rtol=1e-13, atol=0)


def test_iluk_full_fill_is_the_exact_block_solve(oracle):
    """With a level of fill above the subdomain size every block is
    factored exactly: ILU(k) applies the block-diagonal inverse."""
    rp, ci, v, _ = _poisson_system(oracle, 8, 6)
    n = len(rp) - 1
    part = (np.arange(n) * 3 // n).astype(np.int32)
    A = sp.csr_matrix((v, ci, rp), shape=(n, n)).toarray()
    B = np.where(part[:, None] == part[None, :], A, 0.0)
    rng = np.random.default_rng(2)
    r = rng.standard_normal(n)
    z, rc = oracle.iluk_apply(rp, ci, v, r, n, part)
    assert rc == 0
    assert np.allclose(z, np.linalg.solve(B, r), rtol=1e-11, atol=1e-12)


def test_iluk_solve_takes_fewer_iterations(oracle):
    """BiCGStab with Schwarz ILU(2) blocks needs fewer iterations than with
    ILU(0) on a jittered triangle mesh, and reaches the same tolerance."""
    nodes, cptr, cind = meshes.triangulated(40, 32, 1.0, 1.0, jitter=0.2,
                                            seed=5)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(6)
    rp, ci, v, rhs = om.laplacian(rng.uniform(1, 3, om.n_faces), bc,
                                  np.zeros(om.n_faces),
                                  rng.standard_normal((om.n_faces, 2)))
    n = len(rp) - 1
    part = (np.arange(n) * 4 // n).astype(np.int32)
    A = sp.csr_matrix((v, ci, rp))
    its = {}
    for k in (0, 2):
        x, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-10, max_iters=2000,
                                part=part, ilu_fill=k)
        assert st["status"] == 0, st
        assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-10
        its[k] = st["iters"]
    assert its[2] < its[0], its


# ------------------------------------------------------------ direct solve
def test_sparse_lu_oracle_matches_dense_solve(oracle):
    """The oracle's band LU (EigenSparseMatrixSolver semantics) against
    numpy's dense LAPACK solve on a pressure system."""
    rp, ci, v, b = _poisson_system(oracle, 30, 22, seed=4)
    x, info = oracle.sparse_lu_solve(rp, ci, v, b)
    A = sp.csr_matrix((v, ci, rp)).toarray()
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-12
    assert info["replaced"] == 0 and 0 < info["band"][0] <= 60


def test_sparse_lu_oracle_pivots_placeholders_and_repeats(oracle):
    """Zero diagonals need row interchanges; -1 columns are skipped and
    repeated columns summed, as setFromTriplets does
    (EigenSparseMatrixSolver.cpp:31-40)."""
    rng = np.random.default_rng(7)
    n = 300
    A = sp.random(n, n, density=0.02, random_state=8, format="lil")
    for i in range(n):
        A[i, (i + 1) % n] = 1.0 + rng.random()  # keeps A nonsingular
        A[i, i] = 0.0 if i % 3 == 0 else 0.1 * rng.standard_normal()
    A = A.tocsr()
    A.sort_indices()
    rp, ci, v = A.indptr, A.indices, A.data
    # rebuild with a placeholder and a split (repeated) entry in every row
    rows_c, rows_v = [], []
    for i in range(n):
        c = list(ci[rp[i]:rp[i + 1]])
        w = list(v[rp[i]:rp[i + 1]])
        c += [-1, c[0]]
        w += [123.0, 0.25 * w[0]]
        w[0] *= 0.75
        rows_c.append(c)
        rows_v.append(w)
    rp2 = np.concatenate([[0], np.cumsum([len(c) for c in rows_c])])
    ci2 = np.concatenate(rows_c).astype(np.int32)
    v2 = np.concatenate(rows_v)
    b = rng.standard_normal(n)
    x, info = oracle.sparse_lu_solve(rp2, ci2, v2, b)
    xd = np.linalg.solve(A.toarray(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-10


def test_sparse_lu_oracle_singular_neumann_gets_a_solution(oracle):
    """All-Neumann pressure system (singular, consistent rhs): the vanishing
    last pivot is replaced and the result solves the system."""
    om = rect(oracle, 20, 16, 1.0, 1.0)
    f = om.faces()
    bc = np.ones(om.n_faces, np.int32)  # normal gradient everywhere
    rng = np.random.default_rng(3)
    rp, ci, v, _ = om.laplacian(rng.uniform(0.5, 2.0, om.n_faces), bc,
                                np.zeros(om.n_faces))
    A = sp.csr_matrix((v, ci, rp))
    b = rng.standard_normal(om.n_cells)
    b -= b.mean()  # consistent: orthogonal to the constant null vector
    x, info = oracle.sparse_lu_solve(rp, ci, v, b)
    assert info["replaced"] >= 1
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
