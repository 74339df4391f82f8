"""Ghost-cell immersed-boundary pressure equation (FractionalStepGCIB):
device equation against the oracle on channel meshes with a cylinder.

Bars: cell classes and the CSR pattern identical; fluid-row off-diagonals
bit-exact (same FP64 arithmetic), fluid diagonals and rhs within 1e-14 of
the row scale; IB-row coefficients, which come from a 4x4 inverse computed
by two different eliminations, within 1e-11 of the row scale; the solve of
the non-symmetric system agrees with the oracle's to 1e-8 relative when
both are converged to 1e-12."""
import numpy as np
import pytest

from phase_gb300 import meshes

pytestmark = pytest.mark.gpu


def _case(pg, oracle, nx, ny, circle, ib_bc, seed=5):
    L, H = 6.0, 3.0
    nodes, cptr, cind = meshes.rectilinear(nx, ny, L, H)
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    patch = meshes.rect_patch_of_faces(f["fx"], f["fy"], f["rcell"], L, H)
    bc = np.ones(om.n_faces, np.int32)
    bc[patch == 1] = 0                     # outlet p = 0
    rng = np.random.default_rng(seed)
    gamma = rng.uniform(0.5, 2.0, om.n_faces)
    u = rng.standard_normal((om.n_faces, 2))
    bv = np.zeros(om.n_faces)
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[circle], ib_bc=ib_bc)
    eqn.assemble(gamma_face=gamma, bc_value=bv, u_face=u)
    ref = om.gcib_laplacian(gamma, bc, bv, u, [circle], ib_bc=ib_bc)
    return eqn, ref


@pytest.mark.parametrize("ib_bc", [1, 0])
@pytest.mark.parametrize("circle", [(2.0, 1.5, 0.5), (3.3, 1.21, 0.77)])
def test_gcib_equation_matches_oracle(pg, oracle, ib_bc, circle):
    eqn, (rpo, cio, vo, rhso, clso) = _case(pg, oracle, 120, 60, circle, ib_bc)
    assert np.array_equal(eqn.cell_class(), clso)
    assert (clso == 1).sum() > 10 and (clso == 2).sum() > 10
    rp, ci, v, rhs = eqn.export()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    scale = np.add.reduceat(np.abs(vo), rpo[:-1])[rows]
    fluid = clso[rows] == 0
    off = ci != rows
    assert np.array_equal(v[fluid & off], vo[fluid & off])
    assert np.all(np.abs(v - vo)[fluid & ~off] <= 1e-14 * scale[fluid & ~off])
    assert np.all(np.abs(v - vo)[~fluid] <= 1e-11 * scale[~fluid])
    rs = np.add.reduceat(np.abs(vo), rpo[:-1])
    assert np.all(np.abs(rhs - rhso) <= 1e-14 * np.maximum(rs, np.abs(rhso)))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gcib_solve_matches_oracle(pg, oracle, precision):
    eqn, (rpo, cio, vo, rhso, clso) = _case(pg, oracle, 96, 48,
                                            (2.4, 1.4, 0.6), 1)
    s = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=20000,
                              precision=pg.MIXED if precision == "mixed"
                              else pg.FP64)
    s.set_eqn(eqn)
    assert s.solve() <= 1e-12 and s.stats.status == pg.PG_OK
    part, _ = s.partition()
    xo, st = oracle.bicgstab(rpo, cio, vo, -rhso, tol=1e-12, max_iters=20000,
                             part=part)
    assert st["status"] == 0
    x = s.x()
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8


def test_gcib_exact_zeros_are_dropped_as_crsequation_does(pg, oracle):
    """CrsEquation::operator+ (CrsEquation.cpp:185-229) leaves out entries
    that are exactly zero.  With gamma = 0 on a fifth of the interior faces
    the Laplacian's coefficients there are exactly 0: the exported CSR drops
    them as the oracle's CrsEquation merge does (pattern identical), while
    a plain pressure equation (operator==(Vector), no merge) keeps them."""
    L, H, nx, ny = 6.0, 3.0, 60, 30
    nodes, cptr, cind = meshes.rectilinear(nx, ny, L, H)
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    patch = meshes.rect_patch_of_faces(f["fx"], f["fy"], f["rcell"], L, H)
    bc = np.ones(om.n_faces, np.int32)
    bc[patch == 1] = 0
    rng = np.random.default_rng(8)
    gamma = rng.uniform(0.5, 2.0, om.n_faces)
    zero = (f["rcell"] >= 0) & (rng.random(om.n_faces) < 0.2)
    gamma[zero] = 0.0
    u = rng.standard_normal((om.n_faces, 2))
    bv = np.zeros(om.n_faces)
    circle = (2.0, 1.5, 0.5)
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[circle], ib_bc=1)
    eqn.assemble(gamma_face=gamma, bc_value=bv, u_face=u)
    rpo, cio, vo, rhso, clso = om.gcib_laplacian(gamma, bc, bv, u, [circle],
                                                 ib_bc=1)
    rp, ci, v, rhs = eqn.export()
    assert len(ci) < eqn.nnz  # entries were dropped
    assert not np.any(vo == 0.0)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    scale = np.add.reduceat(np.abs(vo), rpo[:-1])[rows]
    assert np.all(np.abs(v - vo) <= 1e-11 * scale)
    # the plain equation keeps the zero-valued slots, as CrsEquation does
    plain = pg.fv.laplacian(gamma, m, bc, bv, u)
    rpp, cip, vp, _ = plain.export()
    rpq, ciq, vq, _ = om.laplacian(gamma, bc, bv, u)
    assert np.array_equal(rpp, rpq) and np.array_equal(cip, ciq)
    assert np.count_nonzero(vp == 0.0) == np.count_nonzero(vq == 0.0) > 0


def _channel(pg, oracle, nx=120, ny=60, seed=5):
    L, H = 6.0, 3.0
    nodes, cptr, cind = meshes.rectilinear(nx, ny, L, H)
    m = pg.Mesh(nodes, cptr, cind)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    patch = meshes.rect_patch_of_faces(f["fx"], f["fy"], f["rcell"], L, H)
    bc = np.ones(om.n_faces, np.int32)
    bc[patch == 1] = 0
    rng = np.random.default_rng(seed)
    fields = dict(gamma=rng.uniform(0.5, 2.0, om.n_faces),
                  u=rng.standard_normal((om.n_faces, 2)),
                  bv=np.zeros(om.n_faces))
    return m, om, bc, fields


def _matches_oracle(eqn, ref, tight_ib=1e-11):
    rpo, cio, vo, rhso, clso = ref
    assert np.array_equal(eqn.cell_class(), clso)
    rp, ci, v, rhs = eqn.export()
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    scale = np.add.reduceat(np.abs(vo), rpo[:-1])[rows]
    assert np.all(np.abs(v - vo) <= tight_ib * scale)
    rs = np.add.reduceat(np.abs(vo), rpo[:-1])
    assert np.all(np.abs(rhs - rhso) <= 1e-14 * np.maximum(rs, np.abs(rhso)))


@pytest.mark.parametrize("ib_bc", [1, 0])
def test_moving_body_updates_match_oracle(pg, oracle, ib_bc):
    """A body moving as OscillatingMotion moves it (centre x0 + a sin(w t)),
    updated step by step on the device (pg_eqn_update_gcib): after every
    step the assembled equation equals the oracle's freshly built one and a
    freshly created device equation (bit for bit), and the pattern-changed
    flag is set exactly when the oracle's classes or pattern changed."""
    m, om, bc, fl = _channel(pg, oracle)
    c0 = np.array([2.0, 1.5, 0.5])
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[c0], ib_bc=ib_bc,
                      ib_ref=0.25)
    prev = om.gcib_laplacian(fl["gamma"], bc, fl["bv"], fl["u"], [c0],
                             ib_bc=ib_bc, ib_ref=0.25)
    seen = {True: 0, False: 0}
    for step in range(1, 13):
        t = 0.01 * step
        # small steps keep every class; every third one moves a cell width
        amp = 0.3 if step % 3 == 0 else 2e-4
        c = c0 + np.array([amp * np.sin(2 * np.pi * t),
                           0.5 * amp * np.sin(4 * np.pi * t), 0.0])
        ref_val = 0.25 + 0.01 * step
        changed = eqn.move_ib([c], ib_ref=ref_val)
        eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
        ref = om.gcib_laplacian(fl["gamma"], bc, fl["bv"], fl["u"], [c],
                                ib_bc=ib_bc, ib_ref=ref_val)
        _matches_oracle(eqn, ref)
        same = (np.array_equal(ref[4], prev[4]) and np.array_equal(ref[0], prev[0])
                and np.array_equal(ref[1], prev[1]))
        assert changed == (not same), step
        seen[changed] += 1
        fresh = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[c], ib_bc=ib_bc,
                            ib_ref=ref_val)
        fresh.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
        for a, b in zip(eqn.export(), fresh.export()):
            assert np.array_equal(a, b)
        prev = ref
    assert seen[True] >= 3 and seen[False] >= 3, seen


def test_moving_body_keeps_or_redoes_the_solver_analysis(pg, oracle):
    """A move that keeps every class leaves the pattern, so the solver keeps
    its analysis (same partition object, no re-analysis needed) and solves
    the moved system; a move across cells changes the pattern and the
    solver re-analyses.  Both solves agree with the oracle's."""
    m, om, bc, fl = _channel(pg, oracle, 96, 48)
    c = np.array([2.4, 1.4, 0.6])
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[c], ib_bc=1)
    eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
    s = pg.SparseMatrixSolver(tolerance=1e-12, max_iters=20000)
    s.set_eqn(eqn)
    assert s.solve() <= 1e-12
    prev = om.gcib_laplacian(fl["gamma"], bc, fl["bv"], fl["u"], [c], ib_bc=1)
    part0, _ = s.partition()
    # 1e-7 keeps every class and every nearest node (an image point moves
    # 2e-7 in cells of 0.0625); 0.2 moves the body three cells
    for dx, expect_change in ((1e-7, False), (0.2, True)):
        c = c + np.array([dx, 0.0, 0.0])
        ref = om.gcib_laplacian(fl["gamma"], bc, fl["bv"], fl["u"], [c], ib_bc=1)
        same = all(np.array_equal(ref[i], prev[i]) for i in (0, 1, 4))
        assert same != expect_change
        assert eqn.move_ib([c]) == expect_change
        eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
        s.set_eqn(eqn)
        assert s.solve() <= 1e-12 and s.stats.status == pg.PG_OK
        rpo, cio, vo, rhso, _ = ref
        prev = ref
        part, _ = s.partition()
        if not expect_change:
            assert np.array_equal(part, part0)
        xo, st = oracle.bicgstab(rpo, cio, vo, -rhso, tol=1e-12,
                                 max_iters=20000, part=part)
        assert st["status"] == 0
        assert np.linalg.norm(s.x() - xo) / np.linalg.norm(xo) < 1e-8


def test_moving_body_error_leaves_the_equation(pg, oracle):
    """A body moved against the inlet wall puts image points outside the
    mesh, where the nearest node has two cells: the update fails with
    PG_BAD_ARG naming the cell, and the equation keeps its previous body
    (classes and assembled values unchanged); a valid move then works."""
    m, om, bc, fl = _channel(pg, oracle, 60, 30)
    c = [2.0, 1.5, 0.5]
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[c], ib_bc=1)
    eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
    cls0 = eqn.cell_class()
    exp0 = eqn.export()
    with pytest.raises(pg.PhaseError, match="four cells"):
        eqn.move_ib([(0.3, 1.5, 0.5)])
    assert np.array_equal(eqn.cell_class(), cls0)
    eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
    for a, b in zip(eqn.export(), exp0):
        assert np.array_equal(a, b)
    c2 = (2.5, 1.5, 0.5)
    eqn.move_ib([c2])
    eqn.assemble(gamma_face=fl["gamma"], bc_value=fl["bv"], u_face=fl["u"])
    _matches_oracle(eqn, om.gcib_laplacian(fl["gamma"], bc, fl["bv"], fl["u"],
                                           [c2], ib_bc=1))
