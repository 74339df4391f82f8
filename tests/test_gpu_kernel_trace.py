"""Kernel time inside a solve (pg_solver_trace_kernels /
pg_solver_kernel_times), the measurement the bench's roofline uses.

Bars: a traced solve launches its chunks directly instead of replaying CUDA
graphs and returns the same iteration count and bit-identical solution as
the untraced solve (tracing changes no arithmetic); every launch group is
booked once (two SpMVs, two sweeps, two deflation stages and one update per
BiCGStab iteration, whole chunks of eight); the times are positive and no
group is dropped; the graph path works again after tracing is switched
off."""
import numpy as np
import pytest

from phase_gb300 import workloads

pytestmark = pytest.mark.gpu


def _bubble(pg, n=128):
    w = workloads.rising_bubble(n, n, seed=5)
    m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(n, n, seed=5, faces=m.faces(), cells=m.cells())
    coeff = m.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    return pg.fv.laplacian(coeff, m, w["bc_type"], w["bc_value"], w["u"])


def _solve(s, eqn):
    s.set_eqn(eqn)
    s.setGuess(None)
    s.solve()
    assert s.stats.status == 0
    return s.x(), s.nIters()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_traced_solve_matches_and_books_every_group(pg, prec):
    eqn = _bubble(pg)
    s = pg.SparseMatrixSolver(tolerance=1e-10, max_iters=5000, coarse=2,
                              precision=pg.MIXED if prec == "mixed" else pg.FP64,
                              mixed_sweep=3)
    x0, it0 = _solve(s, eqn)
    s.trace_kernels(True)
    x1, it1 = _solve(s, eqn)
    kt = s.kernel_times()
    s.trace_kernels(False)
    assert it1 == it0
    assert np.array_equal(x0, x1)
    spmv, sweep, upd, coarse = (kt[k][1] for k in ("spmv", "sweep", "update",
                                                   "coarse"))
    assert kt["dropped"] == 0
    assert upd >= it1 and upd % 8 == 0
    assert spmv == 2 * upd and sweep == spmv and coarse == sweep
    for k in ("spmv", "sweep", "update", "coarse"):
        assert kt[k][0] > 0.0
    # graphs again once the trace is off
    x2, it2 = _solve(s, eqn)
    assert it2 == it0 and np.array_equal(x0, x2)
