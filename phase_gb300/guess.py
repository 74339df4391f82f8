"""Learned initial guess for the pressure solve (message-passing network of
libphase_gb300, include/phase_gb300.h pg_mpnn_*).

The training data are (A_t, b_t, x_{t-1}, x_t) triples dumped by the plain
solver over a sequence of rising-bubble time steps: the bubble rises half a
cell per step and each step's predictor velocity u* is reseeded, so A and b
change every step.  Phase obtains these by advection; the sequence here is
synthesised with the case's sizes, densities and boundary conditions.

    python -m phase_gb300.guess --nx 1024 --steps 2000 --out weights.npy

trains on the first 80 % of the steps, validates on the next 10 % and
reports iterations and milliseconds of the held-out last 10 % for the zero
guess, the previous solution (Phase's warm start) and the learned guess.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import workloads

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "rising_bubble_mpnn.npy")


def _pg():
    import phase_gb300 as pg
    return pg


class _DeviceView:
    """Zero-copy view of library device memory for torch
    (__cuda_array_interface__)."""

    def __init__(self, ptr: int, n: int, typestr: str = "<f8"):
        self.__cuda_array_interface__ = {
            "shape": (n,), "typestr": typestr, "data": (ptr, False),
            "version": 3, "strides": None}


class Mpnn:
    """ctypes wrapper of pg_mpnn (device pointers are plain ints)."""

    def __init__(self, seed=0):
        pg = _pg()
        h = ctypes.c_void_p()
        pg._check(pg.lib().pg_mpnn_create(seed, ctypes.byref(h)))
        self._h = h
        self.n_params = pg.lib().pg_mpnn_num_params(h)

    def __del__(self):
        pg = _pg()
        if getattr(self, "_h", None) and pg._lib is not None:
            pg._lib.pg_mpnn_destroy(self._h)
            self._h = None

    def set_graph(self, row_ptr, col_ind):
        pg = _pg()
        rp = np.ascontiguousarray(row_ptr, np.int32)
        ci = np.ascontiguousarray(col_ind, np.int32)
        pg._check(pg.lib().pg_mpnn_set_graph(self._h, pg._ptr(rp), pg._ptr(ci),
                                             rp.size - 1))

    def predict_device(self, vals, b, x_prev, out):
        """All arguments are device pointers (ints); returns the guess's
        ||b - A g|| / ||b||."""
        pg = _pg()
        rel = ctypes.c_double()
        pg._check(pg.lib().pg_mpnn_predict(
            self._h, ctypes.c_void_p(vals), ctypes.c_void_p(b),
            ctypes.c_void_p(x_prev), ctypes.c_void_p(out), ctypes.byref(rel),
            pg.PG_DEVICE))
        return rel.value

    def gradient(self, vals, b, x_prev, x_star):
        """Host arrays in; (loss gradient per parameter, loss) out."""
        pg = _pg()
        arrs = [np.ascontiguousarray(a, np.float64) for a in (vals, b, x_prev, x_star)]
        g = np.empty(self.n_params, np.float32)
        loss = ctypes.c_double()
        pg._check(pg.lib().pg_mpnn_gradient(self._h, *(pg._ptr(a) for a in arrs),
                                            pg.PG_HOST, pg._ptr(g),
                                            ctypes.byref(loss)))
        return g, loss.value

    def predict(self, vals, b, x_prev):
        """Host arrays in; (guess, ||b - A g|| / ||b||) out."""
        pg = _pg()
        arrs = [np.ascontiguousarray(a, np.float64) for a in (vals, b, x_prev)]
        out = np.empty(arrs[1].size)
        rel = ctypes.c_double()
        pg._check(pg.lib().pg_mpnn_predict(self._h, *(pg._ptr(a) for a in arrs),
                                           pg._ptr(out), ctypes.byref(rel),
                                           pg.PG_HOST))
        return out, rel.value

    def train_step_device(self, vals, b, x_prev, x_star, lr):
        pg = _pg()
        loss = ctypes.c_double()
        pg._check(pg.lib().pg_mpnn_train_step(
            self._h, ctypes.c_void_p(vals), ctypes.c_void_p(b),
            ctypes.c_void_p(x_prev), ctypes.c_void_p(x_star), ctypes.c_float(lr),
            pg.PG_DEVICE, ctypes.byref(loss)))
        return loss.value

    def get_params(self):
        pg = _pg()
        p = np.empty(self.n_params, np.float32)
        pg._check(pg.lib().pg_mpnn_get_params(self._h, pg._ptr(p)))
        return p

    def save(self, path):
        pg = _pg()
        pg._check(pg.lib().pg_mpnn_save(self._h, str(path).encode()))

    def load(self, path):
        pg = _pg()
        pg._check(pg.lib().pg_mpnn_load(self._h, str(path).encode()))

    def set_params(self, p):
        pg = _pg()
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        pg._check(pg.lib().pg_mpnn_set_params(self._h, pg._ptr(p)))


class BubbleSequence:
    """Device-resident rising-bubble sequence: step t's system is assembled
    on the GPU from the bubble position and a reseeded u*."""

    def __init__(self, nx=1024, seed=3, host_fields=False):
        """host_fields: generate each step's gamma and u* on the host with
        workloads.rising_bubble_step (reproducible off the GPU, so a CPU run
        can build the same systems) instead of with torch on the device;
        prefetch() moves them to the device ahead of time."""
        import torch
        pg = _pg()
        self.host_fields = host_fields
        self._cache = {}
        self.torch = torch
        self.nx = nx
        w = workloads.rising_bubble(nx, nx, seed=seed)
        self.mesh = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
        self.faces, self.cells = self.mesh.faces(), self.mesh.cells()
        self.bc_type, self.bc_value, self.patch = workloads.rising_bubble_bcs(
            self.faces, nx, nx)
        self.eqn = pg.Equation(self.mesh, pg.GAMMA_FACE, self.bc_type)
        self.dev = torch.device("cuda")
        self.d_bv = torch.from_numpy(self.bc_value).to(self.dev)
        self.n = self.mesh.n_cells
        self.nnz = self.eqn.nnz
        rp, ci, _, _ = self.eqn.export()
        self.row_ptr, self.col_ind = rp, ci
        self.seed = seed

    def centre(self, t, span=2000):
        """Bubble centre at step t: rises from y = 0.5 to 1.5 over ``span``
        steps (0.26 cells per step at 1024 x 1024), staying inside the
        column for the whole sequence."""
        return (0.5, 0.5 + min(t, span) / span)

    def _fields(self, t):
        """gamma (cells) and u* (faces) of step t, generated on the device:
        the bubble of workloads.bubble_gamma at centre(t), and the swirl of
        workloads.divergent_velocity with seeded noise (torch generator)."""
        torch = self.torch
        if not hasattr(self, "_cx"):
            T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)
            self._cx, self._cy = T(self.cells["cx"]), T(self.cells["cy"])
            self._fx, self._fy = T(self.faces["fx"]), T(self.faces["fy"])
            wall = (self.patch == 0) | (self.patch == 1) | (self.patch == 2)
            self._wall = T(wall)
        cx0, cy0 = self.centre(t)
        hx, hy = workloads.RB_WIDTH / self.nx, workloads.RB_HEIGHT / self.nx
        eps = 1.5 * max(hx, hy)
        phi = workloads.RB_RADIUS - torch.hypot(self._cx - cx0, self._cy - cy0)
        h = 0.5 * (1.0 + phi / eps + torch.sin(np.pi * phi / eps) / np.pi)
        gamma = torch.where(phi > eps, torch.ones_like(h),
                            torch.where(phi < -eps, torch.zeros_like(h), h))
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(1000 * self.seed + t)
        x, y = self._fx, self._fy
        u = torch.empty((x.numel(), 2), dtype=torch.float64, device=self.dev)
        u[:, 0] = 0.1 * torch.sin(np.pi * x) * torch.cos(0.5 * np.pi * y)
        u[:, 1] = 0.1 * torch.cos(np.pi * x) * torch.sin(0.5 * np.pi * y) + 0.02
        u += 0.01 * torch.randn(u.shape, generator=gen, dtype=torch.float64,
                                device=self.dev)
        u[self._wall] = 0.0
        return gamma.contiguous(), u.contiguous()

    def prefetch(self, steps):
        """Generate (host mode) and upload the fields of the given steps."""
        torch = self.torch
        for t in steps:
            if t in self._cache:
                continue
            g, u = workloads.rising_bubble_step(self.faces, self.cells,
                                                self.patch, self.nx, t,
                                                seed=self.seed)
            self._cache[t] = (torch.from_numpy(g).to(self.dev),
                              torch.from_numpy(np.ascontiguousarray(u)).to(self.dev))

    def assemble(self, t):
        """Assemble step t on the device; returns the equation."""
        torch = self.torch
        if self.host_fields:
            self.prefetch([t])
            gamma, u = self._cache[t]
        else:
            gamma, u = self._fields(t)
        # the library stream reads what torch's stream wrote: order the two
        # on the device (no host wait), and keep torch from reusing the
        # fields' memory before the library's reads are done
        if not hasattr(self, "_lib_stream"):
            self._lib_stream = torch.cuda.ExternalStream(_pg().stream_handle(),
                                                         device=self.dev)
            self._coeff = torch.empty(self.mesh.n_faces, dtype=torch.float64,
                                      device=self.dev)
        ready = torch.cuda.Event()
        ready.record(torch.cuda.current_stream(self.dev))
        self._lib_stream.wait_event(ready)
        gamma.record_stream(self._lib_stream)
        u.record_stream(self._lib_stream)
        self._gamma = gamma
        self._u = u.view(-1)
        self.mesh.dt_over_rho_device(gamma.data_ptr(), self._coeff.data_ptr(),
                                     workloads.RB_RHO1, workloads.RB_RHO2,
                                     workloads.RB_DT)
        self.eqn.assemble_device(gamma_face=self._coeff.data_ptr(),
                                 bc_value=self.d_bv.data_ptr(),
                                 u_face=self._u.data_ptr())
        return self.eqn

    def device_system(self, t):
        """(vals address, b tensor) of step t on the device, b = -rhs_."""
        torch = self.torch
        eqn = self.assemble(t)
        v, r = eqn.device_values()
        _pg().synchronize()  # the library stream has written rhs_
        rhs = torch.as_tensor(_DeviceView(r, self.n), device=self.dev)
        b = -rhs
        # the library stream does not order with torch's: finish b first
        torch.cuda.synchronize()
        return v, b


def dump_sequence(path, nx=1024, steps=range(1, 11), coarse=1, seed=3):
    """Solve the rising-bubble sequence with the plain FP64 solver (warm from
    the previous step, as a time loop runs it) and write the (A_t, b_t, x_t)
    triples to ``path`` in the triples.py format."""
    from . import triples
    pg = _pg()
    seq = BubbleSequence(nx, seed=seed)
    keep = seq.col_ind >= 0  # CrsEquation placeholder slots are dropped
    rows = np.repeat(np.arange(seq.n), np.diff(seq.row_ptr))[keep]
    rp = np.zeros(seq.n + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    w = triples.TripleWriter(path, rp, seq.col_ind[keep], nx=nx, seed=seed,
                             workload="rising bubble", tolerance=1e-8)
    solver = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                   coarse=coarse)
    for t in steps:
        eqn = seq.assemble(int(t))
        solver.set_eqn(eqn)
        solver.solve()
        if solver.stats.status != pg.PG_OK:
            raise RuntimeError(f"dump: step {t} did not converge")
        _, _, v, rhs = eqn.export()
        w.write(int(t), v[keep], -rhs, solver.x())
    return w


def train(nx=1024, steps=2000, epochs=8, lr=2e-3, out=DEFAULT_WEIGHTS,
          eval_steps=20, log=print):
    import torch
    pg = _pg()
    seq = BubbleSequence(nx)
    n = seq.n
    dev = seq.dev
    n_train = int(0.8 * steps)
    n_val = int(0.1 * steps)
    # 1. dump triples with the plain solver (warm-started, as in a time loop)
    solver = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000)
    xs = torch.zeros((steps + 1, n), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    t0 = time.time()
    iters = []
    for t in range(1, steps + 1):
        solver.set_eqn(seq.assemble(t))
        solver.solve()
        if solver.stats.status != pg.PG_OK:
            raise RuntimeError(f"dump: step {t} did not converge "
                               f"({solver.stats.as_dict()})")
        solver.x_device(xs[t].data_ptr())
        iters.append(solver.nIters())
    log(f"dumped {steps} solves in {time.time() - t0:.1f} s "
        f"(mean {np.mean(iters):.0f} iterations)")
    # 2. train on steps 1..n_train (x_prev = x_{t-1}); cosine learning-rate
    #    decay to lr/20; the parameters of the epoch with the best validation
    #    residual are kept
    net = Mpnn(seed=1)
    net.set_graph(seq.row_ptr, seq.col_ind)
    rng = np.random.default_rng(0)
    hist = []
    best = (float("inf"), None, -1)
    t0 = time.time()
    n_steps = epochs * (n_train - 1)
    k = 0
    for ep in range(epochs):
        order = rng.permutation(np.arange(2, n_train + 1))
        losses = []
        for t in order:
            v, b = seq.device_system(int(t))
            lr_k = lr * (0.05 + 0.95 * 0.5 * (1.0 + np.cos(np.pi * k / n_steps)))
            k += 1
            loss = net.train_step_device(v, b.data_ptr(), xs[t - 1].data_ptr(),
                                         xs[t].data_ptr(), lr_k)
            losses.append(loss)
        val = []
        for t in range(n_train + 1, n_train + n_val + 1):
            v, b = seq.device_system(t)
            g = torch.empty(n, dtype=torch.float64, device=dev)
            val.append(net.predict_device(v, b.data_ptr(),
                                          xs[t - 1].data_ptr(), g.data_ptr()))
        hist.append(dict(epoch=ep, train_loss=float(np.mean(losses)),
                         val_rel_residual=float(np.mean(val))))
        log(f"epoch {ep}: train loss {np.mean(losses):.4f}, validation "
            f"||b - A g||/||b|| {np.mean(val):.4f} ({time.time() - t0:.1f} s)")
        if np.mean(val) < best[0]:
            best = (float(np.mean(val)), net.get_params(), ep)
    net.set_params(best[1])
    log(f"kept epoch {best[2]} (validation {best[0]:.4f})")
    params = net.get_params()
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.save(out, params)
    # 3. held-out comparison: zero guess, previous solution, learned guess
    test = list(range(n_train + n_val + 1, steps + 1))[:eval_steps]
    report = evaluate(seq, net, xs, test, log, precisions=("fp64", "mixed"))
    report.update(train_history=hist, best_epoch=best[2],
                  n_params=int(net.n_params), nx=nx,
                  steps=steps, split=[n_train, n_val, steps - n_train - n_val])
    return report


def evaluate(seq, net, xs, test, log=print, precisions=("fp64",)):
    """Iterations and device ms of the held-out steps for the three guesses
    (zero, previous step's solution, learned) with the given solvers."""
    import torch
    pg = _pg()
    n = seq.n
    res = {}
    for prec in precisions:
        s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                  precision=pg.FP64 if prec == "fp64" else pg.MIXED)
        rows = {"zero": [], "previous": [], "learned": []}
        for t in test:
            v, b = seq.device_system(t)
            eqn = seq.eqn
            g = torch.empty(n, dtype=torch.float64, device=seq.dev)
            rel = net.predict_device(v, b.data_ptr(),
                                     xs[t - 1].data_ptr(), g.data_ptr())
            for kind in rows:
                s.set_eqn(eqn)
                if kind == "zero" or (kind == "learned" and rel >= 1.0):
                    s.setGuess(None)  # fallback: the zero guess is better
                elif kind == "previous":
                    s.setGuess(xs[t - 1].cpu().numpy())
                else:
                    s.setGuess(g.cpu().numpy())
                s.solve()
                rows[kind].append((s.nIters(), s.stats.ms))
        res[prec] = {k: dict(iters=float(np.mean([a for a, _ in r])),
                             ms=float(np.mean([m for _, m in r])))
                     for k, r in rows.items()}
        log(f"{prec}: " + ", ".join(f"{k} {v['iters']:.0f} it / {v['ms']:.1f} ms"
                                    for k, v in res[prec].items()))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--eval-steps", type=int, default=20)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--report", default=None)
    a = ap.parse_args()
    import __graft_entry__
    __graft_entry__.build()
    rep = train(a.nx, a.steps, a.epochs, a.lr, a.out, a.eval_steps)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
