"""The line form of the ILU(0) sweep (structured blocks: one grid line per
lane, the level chain carried by warp shuffles) against the stream form
on the same analysis.

Both forms subtract a row's products in the order of its factor slots, so
on the same permutation they must agree bit for bit: in every
preconditioner application (plain, with the deflated coarse correction,
FP64 and float-float) and therefore in whole solves (iteration counts and
solutions identical).  PG_LINE_SWEEP=0 at the hand-over keeps the line
ordering of the analysis but runs the stream kernel; PG_LINE=0 leaves the
line form out of the analysis altogether (the original level order), and
that solver agrees with the oracle as before."""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes, workloads

pytestmark = pytest.mark.gpu


def _bubble_eqn(pg, n):
    w = workloads.rising_bubble(n, n, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(n, n, seed=3, faces=m.faces(), cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    return pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])


def _solver(pg, eqn, env, **cfg):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        s = pg.SparseMatrixSolver(**cfg)
        s.set_eqn(eqn)
        s.partition()  # the analysis has run with this environment
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return s


@pytest.mark.parametrize("n,sub", [(256, 512), (256, 1024), (128, 128)])
@pytest.mark.parametrize("coarse", [0, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_line_and_stream_sweeps_agree_bitwise(pg, n, sub, coarse, precision):
    eqn = _bubble_eqn(pg, n)
    prec = pg.MIXED if precision == "mixed" else pg.FP64
    # mixed_sweep 2: the float-float level-blob form (the line form's twin)
    cfg = dict(tolerance=1e-8, max_iters=5000, subdomain_rows=sub,
               coarse=coarse, precision=prec, mixed_sweep=2)
    s_line = _solver(pg, eqn, {}, **cfg)
    s_stream = _solver(pg, eqn, {"PG_LINE_SWEEP": "0"}, **cfg)
    p1, k1 = s_line.partition()
    p2, k2 = s_stream.partition()
    assert k1 == k2 and np.array_equal(p1, p2)
    assert s_line.sweep_form() == 1 and s_stream.sweep_form() == 0
    rng = np.random.default_rng(4)
    r = rng.standard_normal(eqn.n)
    z1 = s_line.apply_precond(r)
    z2 = s_stream.apply_precond(r)
    assert np.array_equal(z1, z2)
    assert s_line.solve() <= 1e-8 and s_stream.solve() <= 1e-8
    assert s_line.nIters() == s_stream.nIters()
    assert np.array_equal(s_line.x(), s_stream.x())


def test_line_ordering_solves_as_before(pg, oracle):
    """The line ordering only permutes rows inside a level: the solve with
    it and the one without (PG_LINE=0) both match the oracle's solve on the
    same partition (a 128 x 128 grid with face coefficients in [1, 2], where
    FP64 reaches 1e-12)."""
    nodes, cptr, cind = meshes.rectilinear(128, 128, 1.0, 1.0)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(6)
    eqn = pg.fv.laplacian(rng.uniform(1.0, 2.0, m.n_faces), m, bc,
                          np.zeros(m.n_faces),
                          rng.standard_normal((m.n_faces, 2)))
    rp, ci, v, rhs = eqn.export()
    A = sp.csr_matrix((v, ci, rp))
    xs = []
    for env in ({}, {"PG_LINE": "0"}):
        s = _solver(pg, eqn, env, tolerance=1e-12, max_iters=20000,
                    subdomain_rows=256)
        assert s.sweep_form() == (0 if env else 1)
        assert s.solve() <= 1e-12
        xs.append(s.x())
        part, _ = s.partition()
    xo, st = oracle.bicgstab(rp, ci, v, -rhs, tol=1e-12, max_iters=20000,
                             part=part)
    for x in xs:
        assert np.linalg.norm(-rhs - A @ x) / np.linalg.norm(rhs) <= 1.01e-12
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9


@pytest.mark.parametrize("mesh", ["rect", "tri"])
def test_sweep_form_by_mesh(pg, mesh):
    """A 100 x 37 grid cut into ~300-row subdomains (cuts moved to grid
    lines, so every block is a full rectangle) takes the line form; a
    triangle mesh takes the stream form.  Both solve to the tolerance."""
    if mesh == "rect":
        nodes, cptr, cind = meshes.rectilinear(100, 37, 1.0, 1.3)
    else:
        nodes, cptr, cind = meshes.triangulated(40, 30, 1.0, 1.0, jitter=0.2,
                                                seed=4)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    eqn = pg.fv.laplacian(1.0, m, bc, np.zeros(m.n_faces))
    s = pg.SparseMatrixSolver(tolerance=1e-10, subdomain_rows=300)
    s.set_eqn(eqn)
    rng = np.random.default_rng(2)
    rp, ci, v, _ = eqn.export()
    b = rng.standard_normal(eqn.n)
    s.setRhs(b)
    assert s.sweep_form() == (1 if mesh == "rect" else 0)
    assert s.solve() <= 1e-10
    A = sp.csr_matrix((v, ci, rp))
    assert np.linalg.norm(b - A @ s.x()) / np.linalg.norm(b) <= 1.01e-10


def _ilu_apply_f32_weights(rp, ci, lu, part, r):
    """z = (LU)^-1 r per subdomain in FP64 arithmetic with the factor stored
    as the device's FP32 records hold it: L multipliers and 1/u_ii rounded
    to FP32, the diagonal applied as a product."""
    n = len(rp) - 1
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    z = np.array(r, np.float64)
    rows = [np.asarray(ci[rp[i]:rp[i + 1]]) for i in range(n)]
    vals = [f32(lu[rp[i]:rp[i + 1]]) for i in range(n)]
    dinv = np.empty(n)
    for i in range(n):
        d = lu[rp[i]:rp[i + 1]][rows[i] == i][0]
        dinv[i] = np.float32(1.0 / d)
    for i in range(n):
        c, w = rows[i], vals[i]
        sel = (c < i) & (part[c] == part[i])
        z[i] -= np.dot(w[sel], z[c[sel]]) if sel.any() else 0.0
    for i in range(n - 1, -1, -1):
        c, w = rows[i], vals[i]
        sel = (c > i) & (part[c] == part[i])
        acc = z[i] - (np.dot(w[sel], z[c[sel]]) if sel.any() else 0.0)
        z[i] = acc * dinv[i]
    return z


@pytest.mark.parametrize("sub", [128, 1024])
def test_fp32_weight_sweep_matches_rounded_factors(pg, oracle, sub):
    """mixed_sweep 3: the ILU(0) factor stored in FP32 and swept in
    float-float arithmetic equals the FP64 sweep of the same FP32-rounded
    factor (1e-10 relative; the sweep arithmetic is about 48-bit).  128-row
    blocks of the 128 x 96 grid are paired in a warp, 1024-row blocks take
    a warp each."""
    w = workloads.rising_bubble(128, 96, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(128, 96, seed=3, faces=m.faces(), cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    eqn = pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])
    rp, ci, v, rhs = eqn.export()
    s = pg.SparseMatrixSolver(subdomain_rows=sub, precision=pg.MIXED,
                              mixed_sweep=3)
    s.set_eqn(eqn)
    assert s.sweep_form() == 1
    part, nparts = s.partition()
    assert nparts > 4
    lu, rc = oracle.ilu0(rp, ci, v, part)
    assert rc == 0
    rng = np.random.default_rng(5)
    for r in (rng.standard_normal(eqn.n), -rhs):
        z = s.apply_precond(r)
        zo = _ilu_apply_f32_weights(rp, ci, lu, part, r)
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-10


def test_fp32_weight_sweep_solves_the_bubble(pg):
    """The float-float solver with FP32-stored factors (a fixed linear
    preconditioner) reaches the FP64 true residual 1e-8 on the 256 x 256
    bubble with the deflated coarse correction, in about as many
    iterations as with float-pair factors."""
    eqn = _bubble_eqn(pg, 256)
    its = {}
    for ms in (2, 3):
        s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=5000, coarse=2,
                                  precision=pg.MIXED, mixed_sweep=ms)
        s.set_eqn(eqn)
        assert s.solve() <= 1e-8 and s.stats.status == pg.PG_OK
        its[ms] = s.nIters()
        rp, ci, v, rhs = eqn.export()
        A = sp.csr_matrix((v, ci, rp))
        assert np.linalg.norm(-rhs - A @ s.x()) / np.linalg.norm(rhs) <= 1.01e-8
    assert its[3] <= 1.25 * its[2] + 4, its
