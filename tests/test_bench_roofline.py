"""The bench's roofline bookkeeping, checked on the CPU with a stand-in
solver: launch times come from the traced solve when there is one (the
isolated back-to-back times stay beside them), the dominant kernel is the
one with the largest in-solve share, and the byte counts follow the
preconditioner's form (the deflated form's sweep moves p - A Z y in and z
out; the deflation stage does the Krylov update)."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location(
        "bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Eqn:
    """A 5-point Laplacian on an nx x ny grid in CSR form."""

    def __init__(self, nx, ny):
        n = nx * ny
        j, i = np.divmod(np.arange(n), nx)
        cols = []
        for dj, di in ((-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)):
            jj, ii = j + dj, i + di
            ok = (jj >= 0) & (jj < ny) & (ii >= 0) & (ii < nx)
            cols.append(np.where(ok, jj * nx + ii, -1))
        cols = np.stack(cols, axis=1)
        keep = cols >= 0
        self.n, self.nnz = n, int(keep.sum())
        self.rp = np.concatenate([[0], np.cumsum(keep.sum(axis=1))]).astype(np.int32)
        self.ci = cols[keep].astype(np.int32)
        self.v = np.where(cols[keep] == np.repeat(np.arange(n), keep.sum(axis=1)),
                          4.0, -1.0)

    def export(self):
        return self.rp, self.ci, self.v, np.ones(self.n)


class _Cfg:
    mixed_sweep = 3


class _Solver:
    cfg = _Cfg()

    def __init__(self, n, parts, coarse_ms=0.021):
        self.n, self.parts, self.coarse_ms = n, parts, coarse_ms

    def profile(self, reps=50):
        # pg_solver_profile's keys; coarse 0 without a coarse space
        return dict(spmv=0.02, precond=0.03, update=0.025, factor=1.0,
                    precond_dd=0.02, spmv_dd=0.016, update_dd=0.017,
                    coarse=self.coarse_ms, coarse_inverse=0.7)

    def partition(self):
        part = (np.arange(self.n) * self.parts // self.n).astype(np.int32)
        return part, self.parts

    def sweep_form(self):
        return 1


def test_in_solve_times_drive_the_roofline(bench):
    eqn = _Eqn(256, 256)
    s = _Solver(eqn.n, 128)
    in_solve = {"iters": 10, "kinds": {"spmv": (0.50, 20), "sweep": (0.40, 20),
                                       "update": (0.20, 10), "coarse": (0.60, 20),
                                       "dropped": 0}}
    r = bench.kernel_roofline(None, s, eqn.n, eqn.nnz, dd=True, eqn=eqn,
                              coarse=2, in_solve=in_solve)
    assert r["kernel"] == "coarse"
    assert r["timing"].startswith("inside a solve")
    assert r["launch_ms"] == pytest.approx(0.03)
    assert r["per_kernel_ms"]["spmv"] == pytest.approx(0.025)
    assert r["isolated_launch_ms"]["spmv"] == pytest.approx(0.016)
    # (the line rounds GB/s to 0.1 and fractions to 1e-4)
    assert r["achieved"] == pytest.approx(
        r["algorithmic_bytes"] / 0.03e-3 / 1e9, abs=0.06)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], abs=6e-5)
    ins = r["in_solve"]
    assert ins["iterations"] == 10 and ins["dropped"] == 0
    assert ins["kernel_ms"] == pytest.approx(1.7)
    assert ins["kernel_us_per_iteration"] == pytest.approx(170.0)
    # the deflated form's sweep: FP32 weights of the in-subdomain
    # off-diagonals and 1/u_ii, and 16 bytes of vectors a row
    part, _ = s.partition()
    rows = np.repeat(np.arange(eqn.n), np.diff(eqn.rp))
    off_in = int(np.sum(part[rows] == part[eqn.ci])) - eqn.n
    b_sweep = 4 * off_in + 4 * eqn.n + 16 * eqn.n
    assert r["per_kernel_gbs"]["ilu_apply"] == pytest.approx(
        b_sweep / 0.02e-3 / 1e9, abs=0.06)


def test_back_to_back_times_without_a_trace(bench):
    eqn = _Eqn(256, 256)
    s = _Solver(eqn.n, 128, coarse_ms=0.0)
    r = bench.kernel_roofline(None, s, eqn.n, eqn.nnz, dd=False, eqn=eqn,
                              coarse=0)
    assert r["in_solve"] is None
    assert r["timing"].startswith("back-to-back")
    assert r["per_kernel_ms"] == r["isolated_launch_ms"]
    # one-level form: the sweep fuses the Krylov update (r, p, v in; p, z out)
    # with 8-byte weights
    part, _ = s.partition()
    rows = np.repeat(np.arange(eqn.n), np.diff(eqn.rp))
    off_in = int(np.sum(part[rows] == part[eqn.ci])) - eqn.n
    b_sweep = 8 * off_in + 8 * eqn.n + 40 * eqn.n
    assert r["per_kernel_gbs"]["ilu_apply"] == pytest.approx(
        b_sweep / 0.03e-3 / 1e9, abs=0.06)
    assert "coarse" not in r["per_kernel_ms"]
