"""Solution parity on every workload: the device's converged pressure
correction against the oracle's, at the tolerance the reference solves to
and at the tightest tolerance FP64 reaches.

The reference stops its BiCGStab at ||b - A x|| / ||b|| <= 1e-8
(TrilinosBelosSparseMatrixSolver.cpp:52-55).  Two solvers stopped at the
same residual differ in x by up to ||A^-1|| ||r||, which on these systems
(1000:1 coefficient contrast, |A||x| / |b| up to 1e7) is far above 1e-9:
the oracle's own one-level solve to 1e-8 is ~1e-6 away from the converged
solution on the rising bubble.  So each workload is checked three ways,
all against x*, the oracle's one-level Schwarz-ILU(0) BiCGStab (the
reference's algorithm, 16 subdomains) run to the tightest tolerance FP64
attains on it:

* tight: the device FP64 solve run to the same tight tolerance agrees with
  x* to the bar of the workload (1e-9 where the attainable residual
  allows it);
* same tolerance: at 1e-8 the device's error ||x - x*|| / ||x*|| (FP64 and
  float-float, the deployed two-level preconditioner) is no larger than
  a small multiple of the oracle's own error at 1e-8 (the reference's
  algorithm at the reference's tolerance);
* every solve's FP64 true residual meets its tolerance.

Singular systems (the all-Neumann cavity) are compared with the constant
null-space component removed.  The measured errors are printed, and
appended as JSON lines to the file named by PG_PARITY_LOG when it is set.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from phase_gb300 import meshes, simple, workloads

pytestmark = pytest.mark.gpu

N_SUB = 16  # the oracle's Schwarz subdomains (one per MPI rank of a 16-core run)


def _rel(x, ref, singular):
    if singular:
        x, ref = x - x.mean(), ref - ref.mean()
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def _true_rel(A, x, b):
    return float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))


def _log(rec):
    print(json.dumps(rec))
    path = os.environ.get("PG_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")


def _oracle(oracle, rp, ci, v, b, tol, max_iters):
    n = b.size
    part = (np.arange(n, dtype=np.int64) * N_SUB // n).astype(np.int32)
    threads = min(len(os.sched_getaffinity(0)), N_SUB)
    return oracle.bicgstab(rp, ci, v, b, tol=tol, max_iters=max_iters,
                           part=part, threads=threads)


def _device(pg, eqn, tol, max_iters, precision):
    s = pg.SparseMatrixSolver(tolerance=tol, max_iters=max_iters, coarse=2,
                              precision=pg.MIXED if precision == "mixed"
                              else pg.FP64)
    s.set_eqn(eqn)
    s.solve()
    return s.x(), s.stats


def _check(name, pg, oracle, eqn, tight, floor, tight_dev, tight_bar,
           same_tol_factor=10.0, singular=False, max_iters=30000):
    """tight: the tolerance x* is asked for; floor: the true residual x*
    must reach (FP64 BiCGStab breaks down near eps |A||x| / |b| on the
    high-contrast systems, before a 1e-11 target); tight_dev: the device's
    tight solve; tight_bar: the bar on |x_tight - x*|; same_tol_factor: the
    device's 1e-8 error may be at most this multiple of the oracle's."""
    rp, ci, v, rhs = eqn.export()
    b = -rhs
    A = sp.csr_matrix((v, ci, rp))
    xs, st = _oracle(oracle, rp, ci, v, b, tight, max_iters)
    r_star = _true_rel(A, xs, b)
    assert st["status"] in (0, 2) and r_star <= floor, (st, r_star)
    xo8, st8 = _oracle(oracle, rp, ci, v, b, 1e-8, max_iters)
    assert st8["status"] == 0 and _true_rel(A, xo8, b) <= 1.01e-8
    e_ref8 = _rel(xo8, xs, singular)
    rec = dict(workload=name, n=int(b.size), tight=tight, r_star=r_star,
               oracle_iters_tight=st["iters"], oracle_iters_1e8=st8["iters"],
               oracle_err_1e8=e_ref8, device_tight=tight_dev)
    xt, stt = _device(pg, eqn, tight_dev, max_iters, "fp64")
    assert stt.status == pg.PG_OK, stt.as_dict()
    assert _true_rel(A, xt, b) <= 1.01 * tight_dev
    rec["device_err_tight"] = _rel(xt, xs, singular)
    rec["device_iters_tight"] = stt.iters
    for prec in ("fp64", "mixed"):
        x8, s8 = _device(pg, eqn, 1e-8, max_iters, prec)
        assert s8.status == pg.PG_OK, s8.as_dict()
        assert _true_rel(A, x8, b) <= 1.01e-8
        rec[f"device_err_1e8_{prec}"] = _rel(x8, xs, singular)
        rec[f"device_iters_1e8_{prec}"] = s8.iters
    _log(rec)
    assert rec["device_err_tight"] <= tight_bar, rec
    for prec in ("fp64", "mixed"):
        assert rec[f"device_err_1e8_{prec}"] <= max(
            same_tol_factor * e_ref8, tight_bar), rec
    return rec


def test_cavity_80x80_solution_parity(pg, oracle):
    out = simple.simple_pcorr(pg, 80, 80)
    _check("lid-driven cavity 80x80 SIMPLE pCorr", pg, oracle, out["eqn"],
           tight=1e-12, floor=1e-11, tight_dev=1e-12, tight_bar=1e-9,
           singular=True)


def test_gcib_channel_solution_parity(pg, oracle):
    L, H, nx, ny = 6.0, 3.0, 192, 96
    nodes, cptr, cind = meshes.rectilinear(nx, ny, L, H)
    m = pg.Mesh(nodes, cptr, cind)
    f = m.faces()
    patch = meshes.rect_patch_of_faces(f["fx"], f["fy"], f["rcell"], L, H)
    bc = np.ones(m.n_faces, np.int32)
    bc[patch == 1] = 0
    rng = np.random.default_rng(5)
    eqn = pg.Equation(m, pg.GAMMA_FACE, bc, ib_circles=[(2.4, 1.4, 0.6)],
                      ib_bc=1)
    eqn.assemble(gamma_face=rng.uniform(0.5, 2.0, m.n_faces),
                 bc_value=np.zeros(m.n_faces),
                 u_face=rng.standard_normal((m.n_faces, 2)))
    _check("ghost-cell IB channel 192x96", pg, oracle, eqn, tight=1e-12,
           floor=1e-11, tight_dev=1e-12, tight_bar=2e-9)


def test_cylinder_500k_solution_parity(pg, oracle):
    c = simple.cylinder_pcorr(pg)
    assert 450_000 < c["mesh"].n_cells < 560_000
    _check("cylinder channel ~500k triangles pCorr", pg, oracle, c["eqn"],
           tight=1e-11, floor=1e-9, tight_dev=1e-10, tight_bar=1e-8)


def test_rising_bubble_1m_solution_parity(pg, oracle):
    nx = ny = 1024
    w = workloads.rising_bubble(nx, ny, seed=3)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, ny, seed=3, faces=m.faces(),
                                cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    eqn = pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])
    # FP64 stalls near 2e-10 on this system (|A||x| / |b| = 2.7e6): the
    # oracle breaks down there and the device's reliable updates stop
    # gaining below ~1e-10
    _check("rising bubble 1024x1024", pg, oracle, eqn, tight=1e-11,
           floor=1e-9, tight_dev=5e-10, tight_bar=1e-6, max_iters=8000)
