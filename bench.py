#!/usr/bin/env python
"""Benchmark of the Phase pressure solve on one GB300.

Default (--mode sequence): the rising-bubble pressure-correction sequence
on 1024x1024 quads (1,048,576 cells, 5,238,784 nonzeros, dt/rho face
coefficients with 1000x contrast, p fixed on y+ and normal-gradient
elsewhere, rhs = src::div(u*) of a seeded divergent velocity; the bubble
rises one step at a time).  Two solvers run the same steps, each warm from
its own previous solution as a time loop runs them:

  plain FP64      FP64 BiCGStab + two-level Schwarz ILU(0) (subdomain ILU(0)
                  blocks plus a deflated coarse correction on the
                  subdomain-constant vectors; --coarse 1 additive, 0 none),
                  guess = previous step's x
  learned+mixed   float-float BiCGStab + the same preconditioner (about
                  48-bit arithmetic on the FP32 pipes, FP64 true residual at
                  every reliable update, FP64 hand-over if it stalls),
                  guess = the message-passing network's prediction from
                  (A, b, previous x), replaced by the zero guess when the
                  prediction's residual is not below ||b||

A third arm, float-float warm from its own previous x without the network
(`mixed_prev_x_ms`), shows what the learned guess competes with.  All stop
at ||b - A x||_2 / ||b||_2 <= 1e-8 on the FP64 true residual.
One step = device assembly of fv::laplacian(dt/rho, p) == src::div(u*) +
hand-over + (inference) + ILU(0) factorisation + BiCGStab, inputs resident
in HBM; `value` is the learned+mixed ms per solve, `plain_fp64_ms` the
plain one on the same steps.  `e2e` times the learned+mixed solve through
the C ABI with host buffers (CrsEquation's 5-slot layout, rhs and previous
x uploaded, the solution read back).

--mode single: one system solved from a zero guess (the kernel roofline
and sweep configuration).  --impl reference times the CPU implementation
(the oracle's OpenMP BiCGStab with one ILU(0) subdomain per thread --
Ifpack2 Schwarz/RILUK as run on that many MPI ranks) on the same workload:
in sequence mode the same held-out steps, each warm from its previous CPU
solution; in single mode the zero-guess solve on a bounded sample.
`iters_saved_by_guess` compares the learned arm's iteration counts with the
float-float arm warm from the previous x, step by step.  With --coarse-reuse 1
every arm's solve applies the previous step's coarse inverse while the new
one is built beside it (measured slower on this sequence: more iterations
on several steps, and the inversion competes with the solve).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = ("ms per pCorr solve to 1e-8 rel. residual: plain FP64 vs "
          "learned+mixed, GB300")
WORKLOAD = "rising-bubble pressure system 1024x1024 (1M cells, nnz 5238784)"


def workload_name(nx):
    if nx == 1024:
        return WORKLOAD
    return f"rising-bubble pressure system {nx}x{nx} ({nx * nx} cells)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--subdomain-rows", type=int, default=0)
    ap.add_argument("--mixed-sweep", type=int, default=3, choices=[0, 1, 2, 3],
                    help="mixed ILU(0) sweep form: 0 timed choice, 1 steps, "
                         "2 level blobs, 3 FP32-stored factor weights (line "
                         "form of structured blocks)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--coarse", type=int, choices=(0, 1, 2), default=2,
                    help="two-level Schwarz coarse correction on the "
                         "subdomain-constant vectors: 0 none, 1 additive, "
                         "2 deflated (A-DEF1)")
    ap.add_argument("--coarse-reuse", type=int, choices=(0, 1), default=0,
                    help="sequence mode: each solve applies the previous "
                         "step's coarse inverse while the new one is built "
                         "beside it (the solver's coarse_warm = -2)")
    ap.add_argument("--learned-coarse-warm", type=int, default=0,
                    help="one-level iterations the learned arm runs while "
                         "the coarse inverse is built (0: it waits, its "
                         "inference overlapping the inversion; -1: the "
                         "solver's default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="sequence mode: leave out the cylinder and batched "
                         "summaries")
    ap.add_argument("--mode", default="sequence",
                    choices=["sequence", "single", "batch", "direct",
                             "cylinder"])
    ap.add_argument("--systems", type=int, default=256,
                    help="batch mode: number of immersed-boundary systems")
    ap.add_argument("--t0", type=int, default=1801,
                    help="first timed step of the sequence (held-out range)")
    return ap.parse_args()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU solve
def cpu_solve_sample(rp, ci, v, b, seconds, threads, fallback_iters=None,
                     fallback_what="the FP64 BiCGStab iteration count of this "
                                   "system", x0=None):
    """Time the oracle's BiCGStab + Schwarz-ILU(0) (one contiguous block per
    thread) from x0 (None: zero) on a bounded sample; returns (ms per solve,
    info).  A run that
    reaches 1e-8 inside the sample is timed as is; otherwise the measured ms
    per iteration is multiplied by fallback_iters (the FP64 iteration count
    of the same system, when the caller knows it) or by an extrapolation of
    the residual decay."""
    import numpy as np
    import oracle_bind as ob
    n = b.size
    part = (np.arange(n, dtype=np.int64) * threads // n).astype(np.int32)
    h, ms, sms = ob.bicgstab_history(rp, ci, v, b, 5, part=part,
                                     threads=threads, x0=x0)
    per_iter = ms / max(1, len(h) - 1)
    budget = int(max(20, min(20000, seconds * 1000.0 / max(per_iter, 1e-3))))
    h, ms, sms = ob.bicgstab_history(rp, ci, v, b, budget, part=part,
                                     threads=threads, x0=x0)
    its = len(h) - 1
    per_iter = ms / max(1, its)
    hit = np.flatnonzero(h <= 1e-8)
    if hit.size:
        need = int(hit[0])
        how = f"ran to 1e-8 in {need} iterations"
    elif fallback_iters:
        need = int(fallback_iters)
        how = (f"ran {its} iterations ({h[its]:.2e} rel. residual) at "
               f"{per_iter:.3f} ms each; timed as {need} iterations, "
               f"{fallback_what}")
    else:
        k0 = its // 2
        rate = (h[its] / h[k0]) ** (1.0 / max(1, its - k0))
        need = int(its + math.ceil(math.log(1e-8 / h[its]) / math.log(rate))) \
            if 0 < rate < 1 else -1
        how = (f"ran {its} iterations ({h[its]:.2e} rel. residual), "
               f"extrapolated to 1e-8 at {need} iterations from the "
               f"residual decay rate {rate:.5f}/iteration")
    value = sms + per_iter * need if need > 0 else float("nan")
    return value, dict(iterations=need, ms_per_iter=per_iter, setup_ms=sms,
                       sample=how)


def build_system(nx, want_device=True):
    import numpy as np
    import phase_gb300 as pg
    from phase_gb300 import workloads
    w = workloads.rising_bubble(nx, nx, seed=3)
    mesh = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
    w = workloads.rising_bubble(nx, nx, seed=3, faces=mesh.faces(),
                                cells=mesh.cells())
    coeff = mesh.dt_over_rho(w["gamma"], w["rho1"], w["rho2"], w["dt"])
    return mesh, w, coeff


def slots_layout(rp, ci, v):
    """Expand a compact CSR into CrsEquation's layout: 5 slots per row (more
    when a row is longer), unused slots with column -1
    (CrsEquation.cpp:9-14)."""
    import numpy as np
    n = len(rp) - 1
    cnt = np.diff(rp)
    width = np.maximum(cnt, 5)
    srp = np.zeros(n + 1, np.int32)
    np.cumsum(width, out=srp[1:])
    sci = np.full(srp[-1], -1, np.int32)
    sv = np.zeros(srp[-1])
    rows = np.repeat(np.arange(n), cnt)
    pos = srp[rows] + (np.arange(len(ci)) - rp[rows])
    sci[pos] = ci
    sv[pos] = v
    return srp, sci, sv


def in_subdomain_nnz(eqn, part):
    """Entries whose row and column lie in the same Schwarz subdomain (the
    entries of the ILU(0) factor)."""
    import numpy as np
    rp, ci, _, _ = eqn.export()
    rows = np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp))
    keep = ci >= 0
    return int(np.count_nonzero(part[rows[keep]] == part[ci[keep]]))


def az_nnz(eqn, part):
    """Nonzeros of A Z, Z the subdomain indicator vectors: per row, the
    number of distinct subdomains among its columns."""
    import numpy as np
    rp, ci, _, _ = eqn.export()
    rows = np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp))
    keep = ci >= 0
    K = int(part.max()) + 1
    return int(np.unique(rows[keep] * K + part[ci[keep]]).size)


def traced_solve(solver, eqn, x0):
    """One solve of eqn from x0 with the kernel trace on: the device time
    of each launch-group kind inside the solve (CUDA events on the library
    stream between the groups; the chunks are launched directly)."""
    solver.set_eqn(eqn)
    solver.setGuess(x0)
    solver.trace_kernels(True)
    try:
        solver.solve()
        kt = solver.kernel_times()
    finally:
        solver.trace_kernels(False)
    return {"iters": solver.nIters(), "kinds": kt}


def kernel_roofline(pg, solver, n, nnz, dd, eqn=None, coarse=0, in_solve=None):
    """Per-launch CUDA-event times of the hot kernels of one solver and the
    roofline of the dominant one.  With in_solve (traced_solve's result)
    the launch times are those inside a real solve, where the iteration's
    working set (> 129 MB) does not stay in L2; the back-to-back times of
    each kernel alone on its current system (pg_solver_profile, inputs
    partly L2-resident) are kept beside them.  Compulsory bytes per launch:
    A values + int32 columns + row pointers; ILU(0) factor values + 2-byte
    columns (off-diagonal entries of A bound the factor's) + 1/u_ii; 8-byte
    vector entries in both precisions."""
    import numpy as np
    prof = solver.profile(reps=50)
    part, K = solver.partition()
    off_in = in_subdomain_nnz(eqn, part) - n  # off-diagonal factor entries
    form = solver.sweep_form()
    b_spmv = 12 * nnz + 4 * (n + 1) + 3 * 8 * n          # A, x, rhat in; v out
    # factor weights (8 B, or 4 B for the mixed solver's FP32-stored factor;
    # the stream form adds a 2-byte column each, the line form's columns are
    # implicit), 1/u_ii, and the vectors: r p v in, p z out when the sweep
    # fuses the Krylov update; with the deflated coarse correction the
    # deflation stage does that and the sweep reads p - A Z y and writes z
    wb = 4 if (dd and form == 1 and solver.cfg.mixed_sweep == 3) else 8
    vec_prec = 2 * 8 * n if coarse == 2 else 5 * 8 * n
    b_prec = (wb if form == 1 else wb + 2) * off_in + wb * n + vec_prec
    b_upd = 9 * 8 * n                                    # x r ph sh s t rh in; x r out
    sfx = "_dd" if dd else ""
    ms_of = {"spmv": prof["spmv" + sfx], "ilu_apply": prof["precond" + sfx],
             "update": prof["update" + sfx]}
    shares = {"spmv": 2 * ms_of["spmv"], "ilu_apply": 2 * ms_of["ilu_apply"],
              "update": ms_of["update"]}
    bytes_of = {"spmv": b_spmv, "ilu_apply": b_prec, "update": b_upd}
    if prof["coarse"] > 0:
        ms_of["coarse"] = prof["coarse"]
        shares["coarse"] = 2 * prof["coarse"]
        if coarse == 2:
            # deflation: r p v in, p out (with the subdomain sums); FP32
            # K x K inverse, sums in, y out; p, A Z (row pointers, int32
            # columns, 8-byte values) and y in, p - A Z y out
            bytes_of["coarse"] = (4 * 8 * n + 4 * K * K + 24 * K + 2 * 8 * n
                                  + 4 * (n + 1) + 12 * az_nnz(eqn, part))
        else:
            # additive: FP32 K x K inverse, K float-pair sums, z in/out
            bytes_of["coarse"] = 4 * K * K + 8 * K + 2 * 8 * n
    iso_ms = dict(ms_of)
    timing = "back-to-back launches of each kernel alone (pg_solver_profile)"
    in_solve_out = None
    if in_solve is not None:
        kt = in_solve["kinds"]
        key = {"spmv": "spmv", "ilu_apply": "sweep", "update": "update",
               "coarse": "coarse"}
        if all(kt[key[k]][1] > 0 for k in ms_of):
            ms_of = {k: kt[key[k]][0] / kt[key[k]][1] for k in ms_of}
            shares = {k: kt[key[k]][0] for k in ms_of}
            timing = ("inside a solve: CUDA events between the launch groups "
                      "of a traced solve of the same system")
        total = sum(kt[key[k]][0] for k in key)
        in_solve_out = {
            "iterations": in_solve["iters"],
            "kernel_ms": round(total, 4),
            "kernel_us_per_iteration": round(1e3 * total / max(1, in_solve["iters"]), 2),
            "per_kind_ms": {k: round(kt[key[k]][0], 4) for k in key},
            "per_kind_launch_groups": {k: kt[key[k]][1] for k in key},
            "dropped": kt["dropped"]}
    dom = max(shares, key=shares.get)
    peak, peak_kind = measured_peaks()
    achieved = bytes_of[dom] / (ms_of[dom] * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
            "timing": timing, "in_solve": in_solve_out,
            "isolated_launch_ms": {k: round(v, 5) for k, v in iso_ms.items()},
            "isolated_per_kernel_frac": {
                k: round(bytes_of[k] / (iso_ms[k] * 1e-3) / 1e9 / peak, 4)
                for k in bytes_of},
            "sweep_form": {1: "line", 0: "stream"}.get(form, "none"),
            "factor_weight_bytes": wb,
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "algorithmic_bytes": bytes_of[dom],
            "launch_ms": round(ms_of[dom], 5),
            "per_kernel_gbs": {k: round(bytes_of[k] / (ms_of[k] * 1e-3) / 1e9, 1)
                               for k in bytes_of},
            "per_kernel_frac": {k: round(bytes_of[k] / (ms_of[k] * 1e-3) / 1e9
                                         / peak, 4) for k in bytes_of},
            "per_kernel_ms": {k: round(v, 5) for k, v in ms_of.items()},
            "factor_ms": round(prof["factor"], 4),
            "coarse_inverse_ms": round(prof["coarse_inverse"], 4),
            "frac_of_8tbs": round(achieved / 8000.0, 4)}


def run_sequence(args):
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300 as pg
    from phase_gb300 import guess

    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    seq = guess.BubbleSequence(args.nx, host_fields=True)
    n, nnz, dev = seq.n, int(seq.nnz), seq.dev
    stream = torch.cuda.ExternalStream(pg.stream_handle(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    net = guess.Mpnn()
    net.set_graph(seq.row_ptr, seq.col_ind)
    have_w = os.path.exists(guess.DEFAULT_WEIGHTS)
    if have_w:
        net.set_params(np.load(guess.DEFAULT_WEIGHTS))
    # with --coarse-reuse every arm applies the previous step's coarse
    # inverse while the new one is built; without it the learned arm
    # overlaps the inversion with the network's inference and then waits
    # for it (--learned-coarse-warm), the others warm up beside it
    reuse = -2 if args.coarse_reuse else None
    sp = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                               subdomain_rows=args.subdomain_rows,
                               coarse=args.coarse,
                               coarse_warm=reuse if reuse else -1)
    sm = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                               precision=pg.MIXED,
                               mixed_sweep=args.mixed_sweep,
                               subdomain_rows=args.subdomain_rows,
                               coarse=args.coarse,
                               coarse_warm=reuse if reuse
                               else args.learned_coarse_warm)
    xp_p = torch.zeros(n, dtype=torch.float64, device=dev)
    xp_m = torch.zeros(n, dtype=torch.float64, device=dev)
    g = torch.empty(n, dtype=torch.float64, device=dev)
    b_buf = torch.empty(n, dtype=torch.float64, device=dev)

    def plain_step(t):
        sp.set_eqn(seq.assemble(t))
        sp.setGuess_device(xp_p.data_ptr())
        sp.solve()
        sp.x_device(xp_p.data_ptr())
        return dict(sp.stats.as_dict())

    xp_q = torch.zeros(n, dtype=torch.float64, device=dev)
    sq = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                               precision=pg.MIXED,
                               mixed_sweep=args.mixed_sweep,
                               subdomain_rows=args.subdomain_rows,
                               coarse=args.coarse,
                               coarse_warm=reuse if reuse else -1)

    def mixed_prev_step(t):
        """Float-float solve warm from its own previous x (no network)."""
        sq.set_eqn(seq.assemble(t))
        sq.setGuess_device(xp_q.data_ptr())
        sq.solve()
        sq.x_device(xp_q.data_ptr())
        return dict(sq.stats.as_dict())

    def learned_step(t):
        eqn = seq.assemble(t)
        # hand the system over first: the solver factors its preconditioner
        # on a side stream while the network runs
        sm.set_eqn(eqn)
        v, r = eqn.device_values()
        # b = -rhs_ in a fixed buffer, so the captured inference graph
        # (keyed on its input addresses) is replayed every step; computed on
        # the library stream, which orders it after the assembly and before
        # the network without a host wait (the factorisation runs beside
        # them on the solver's own streams)
        with torch.cuda.stream(stream):
            torch.neg(torch.as_tensor(guess._DeviceView(r, n), device=dev),
                      out=b_buf)
        rel = net.predict_device(v, b_buf.data_ptr(), xp_m.data_ptr(),
                                 g.data_ptr()) if have_w else float("inf")
        use = rel < 1.0
        sm.setGuess_device(g.data_ptr() if use else 0)
        sm.solve()
        sm.x_device(xp_m.data_ptr())
        out = dict(sm.stats.as_dict())
        out.update(guess_rel=rel, learned=bool(use))
        return out

    def timed(step_fn, ts, clocks=None):
        evs, stats = [], []
        for t in ts:
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                flush.fill_(float(t))      # L2 flush (256 MB > 129 MB L2)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            stats.append(step_fn(t))
            with torch.cuda.stream(stream):
                e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs], stats

    W, K, t0 = max(3, args.warmup), args.steps, args.t0
    warm = list(range(t0 - W, t0))
    steps = list(range(t0, t0 + K))
    # the step fields come from the host generator (the reference arm
    # builds the same systems) and are on the device before timing
    seq.prefetch(warm + steps + ([steps[0] - 1] if not args.no_e2e else []))
    # plain FP64 arm
    for t in warm:
        plain_step(t)
    # x of step t0 - 1: the warm start of the CPU baseline's sample
    pg.synchronize()
    x_prev_host = xp_p.cpu().numpy().copy()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms_p, st_p = timed(plain_step, steps)
    # float-float arm warm from the previous x (what the network competes
    # with)
    for t in warm:
        mixed_prev_step(t)
    ms_q, st_q = timed(mixed_prev_step, steps)
    # learned+mixed arm (headline), with the launch count
    for t in warm:
        learned_step(t)
    if world > 1:
        torch.distributed.barrier()
    launches0 = pg.kernel_launches()
    t_wall = time.perf_counter()
    ms_m, st_m = timed(learned_step, steps)
    wall = time.perf_counter() - t_wall
    launches = pg.kernel_launches() - launches0
    clk = clocks.stop()
    ms = sum(ms_m) / len(ms_m)
    plain_ms = sum(ms_p) / len(ms_p)
    if world > 1:
        tt = torch.tensor([ms, plain_ms], dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms, plain_ms = float(tt[0]), float(tt[1])
    # zero-guess FP64 solve of the first timed step (the reference arm's
    # configuration)
    sz = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                               subdomain_rows=args.subdomain_rows,
                               coarse=args.coarse)
    eqn = seq.assemble(t0)
    sz.set_eqn(eqn)
    sz.setGuess(None)
    sz.solve()
    zero = dict(sz.stats.as_dict())
    # kernel time inside real solves (after the timed region): step t0 again
    # from the step-(t0-1) solution, traced, by the float-float and the FP64
    # solver
    in_m = traced_solve(sm, eqn, x_prev_host)
    in_p = traced_solve(sp, eqn, x_prev_host)
    roof_m = kernel_roofline(pg, sm, n, nnz, dd=True, eqn=eqn,
                             coarse=args.coarse, in_solve=in_m)
    roof_p = kernel_roofline(pg, sp, n, nnz, dd=False, eqn=eqn,
                             coarse=args.coarse, in_solve=in_p)
    # DRAM traffic needs a profiler, and no number of this line is taken
    # under one: the per-launch dram__bytes of the same kernels are in the
    # ncu summaries under profiles/
    roof_m["traffic"] = roof_p["traffic"] = None

    e2e = None
    if not args.no_e2e:
        e2e = e2e_learned(pg, guess, seq, net, have_w, steps, torch, dev,
                          args.coarse, reuse if reuse
                          else args.learned_coarse_warm, args.mixed_sweep)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        eqn = seq.assemble(t0)  # the shared equation: re-assemble step t0
        rp, ci, v, rhs = eqn.export()
        threads = len(os.sched_getaffinity(0))
        # the oracle runs the reference's one-level preconditioner from the
        # GPU arms' warm start (the previous step's solution); a sample that
        # does not reach 1e-8 is timed at the one-level FP64 iteration count
        # of the same solve, measured on the device
        s1 = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000, coarse=0)
        s1.set_eqn(eqn)
        s1.setGuess(x_prev_host)
        s1.solve()
        val, info = cpu_solve_sample(rp, ci, v, -rhs, args.cpu_seconds, threads,
                                     fallback_iters=s1.nIters(),
                                     fallback_what="the one-level FP64 "
                                     "BiCGStab iteration count of this solve",
                                     x0=x_prev_host)
        cpu = {"value": round(val, 1), "unit": "ms", "cores": threads,
               "kind": "port",
               "sample": f"oracle BiCGStab + Schwarz-ILU(0), {threads} "
                         f"subdomains, FP64, step {t0} system from the "
                         f"step-{t0 - 1} solution: " + info["sample"],
               "iterations": info["iterations"],
               "ms_per_iter": round(info["ms_per_iter"], 3)}

    # the same step on the host cores with the device's own algorithm (the
    # oracle's deflated two-level Schwarz ILU(0) on the device's partition),
    # which splits the GPU/CPU ratio into algorithm and hardware
    cpu2 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.coarse:
        cpu2 = cpu_two_level(sp, seq.assemble(t0), x_prev_host, args.coarse)

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        extras["cylinder"] = cylinder_summary(pg, torch, args)
        extras["batch"] = batch_summary(pg, torch, args)
        extras["direct"] = direct_summary(pg, args)

    converged = all(st["status"] == 0 and st["rel_residual"] <= 1e-8
                    for st in st_m + st_p + st_q)
    if rank == 0:
        mean = lambda xs: round(float(np.mean(xs)), 1)
        out = {
            "metric": METRIC, "value": round(ms, 3), "unit": "ms",
            "plain_fp64_ms": round(plain_ms, 3),
            "speedup_vs_plain_fp64": round(plain_ms / ms, 3),
            "mixed_prev_x_ms": round(sum(ms_q) / len(ms_q), 3),
            "e2e_ms": e2e["value"] if e2e else None,
            "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32x2 (float-float) + f64 residual"
                     + (", f32 ILU factor" if args.mixed_sweep == 3 else ""),
            "data": "synthetic (seeded rising-bubble sequence, no dataset)",
            "converged": converged,
            "config": {"workload": workload_name(args.nx) + ", time steps "
                                                         f"{steps[0]}..{steps[-1]}",
                       "n_cells": n, "nnz": nnz, "tolerance": 1e-8,
                       "preconditioner": "Schwarz ILU(0), "
                       f"{sm.partition()[1]} subdomains"
                       + {0: "", 1: " + additive coarse correction",
                          2: " + deflated coarse correction (A-DEF1)"}[args.coarse],
                       "mixed_sweep": {0: "timed choice", 1: "steps",
                                       2: "level blobs",
                                       3: "FP32-stored factor, line form"}[args.mixed_sweep],
                       "coarse_reuse": bool(args.coarse_reuse),
                       "learned_coarse_warm": args.learned_coarse_warm,
                       "learned_weights": os.path.relpath(guess.DEFAULT_WEIGHTS, ROOT)
                       if have_w else None,
                       "l2": "256 MB flush write before every step; working "
                             "set > 129 MB L2"},
            "learned_mixed": {"ms": [round(x, 3) for x in ms_m],
                              "iters": [s_["iters"] for s_ in st_m],
                              "fp64_iters": [s_["fp64_iters"] for s_ in st_m],
                              "guess_rel_residual": [round(s_["guess_rel"], 4)
                                                     for s_ in st_m],
                              "learned_guess_used": [s_["learned"] for s_ in st_m],
                              "rel_residual": [s_["rel_residual"] for s_ in st_m]},
            "plain_fp64": {"ms": [round(x, 3) for x in ms_p],
                           "iters": [s_["iters"] for s_ in st_p],
                           "rel_residual": [s_["rel_residual"] for s_ in st_p]},
            "mixed_prev_x": {"ms": [round(x, 3) for x in ms_q],
                             "iters": [s_["iters"] for s_ in st_q],
                             "fp64_iters": [s_["fp64_iters"] for s_ in st_q],
                             "rel_residual": [s_["rel_residual"] for s_ in st_q]},
            # the guess's effect alone: the same float-float solver from the
            # network's guess vs from the previous step's x
            "iters_saved_by_guess": {
                "per_step": [q["iters"] - m_["iters"] for q, m_ in zip(st_q, st_m)],
                "mean": round(sum(q["iters"] - m_["iters"]
                                  for q, m_ in zip(st_q, st_m)) / len(st_m), 2),
                "against": "float-float solve warm from the previous x"},
            "plain_fp64_zero_guess": {"ms": round(zero["ms"], 3),
                                      "iters": zero["iters"],
                                      "rel_residual": zero["rel_residual"]},
            "solves_per_s": round(1000.0 / ms * world, 3),
            "roofline": roof_m, "roofline_plain_fp64": roof_p,
            "cpu_baseline": cpu, "cpu_two_level": cpu2, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk,
            "wall_s": round(wall, 3),
        }
        out.update(extras)
        if not converged:
            out["invalid"] = "a timed solve stopped above the 1e-8 residual"
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_two_level(solver, eqn, x0, coarse):
    """The oracle's BiCGStab with the device solver's preconditioner: Schwarz
    ILU(0) on the device's partition plus the subdomain-constant coarse
    space (explicit coarse inverse, as on the device), FP64, all host
    threads, from x0 (the previous step's solution)."""
    import oracle_bind as ob
    rp, ci, v, rhs = eqn.export()
    part, K = solver.partition()
    threads = len(os.sched_getaffinity(0))
    x, st = ob.bicgstab(rp, ci, v, -rhs, tol=1e-8, max_iters=20000, part=part,
                        x0=x0, threads=threads, coarse=coarse)
    return {"value": round(st["ms"] + st["setup_ms"], 1), "unit": "ms",
            "cores": threads, "kind": "port", "iterations": st["iters"],
            "setup_ms": round(st["setup_ms"], 1),
            "rel_residual": st["rel_residual"], "converged": st["status"] == 0,
            "sample": f"oracle BiCGStab + Schwarz-ILU(0) on the device's {K} "
                      f"subdomains + {'deflated' if coarse == 2 else 'additive'}"
                      " coarse correction (the device's algorithm), FP64, the "
                      "first timed step from the previous step's solution"}


def cylinder_summary(pg, torch, args):
    """The ~500k-triangle cylinder-channel pCorr system (one PISO-style
    predictor step): FP64 and mixed two-level solves to 1e-8 from a zero
    guess, device time per solve (mean of three), and the FP64 kernels'
    roofline."""
    import numpy as np
    from phase_gb300 import simple
    c = simple.cylinder_pcorr(pg)
    eqn = c["eqn"]
    out = {"workload": "cylinder channel, graded Delaunay triangles",
           "n_cells": int(eqn.n), "nnz": int(eqn.nnz), "tolerance": 1e-8}
    for name, prec in (("fp64", pg.FP64), ("mixed", pg.MIXED)):
        s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                  coarse=args.coarse, precision=prec,
                                  mixed_sweep=args.mixed_sweep)
        ms, its, ok = [], [], True
        for _ in range(4):  # every hand-over factors anew (pg_solver_set_eqn)
            s.set_eqn(eqn)
            s.setGuess(None)
            s.solve()
            ms.append(s.stats.ms)
            its.append(s.stats.iters)
            ok &= s.stats.status == pg.PG_OK and s.stats.rel_residual <= 1e-8
        out[name] = {"ms": round(float(np.mean(ms[1:])), 3),
                     "iters": its[1:], "converged": bool(ok),
                     "sweep_form": {1: "line", 0: "stream"}.get(s.sweep_form())}
        r = kernel_roofline(pg, s, eqn.n, int(eqn.nnz), dd=prec == pg.MIXED,
                            eqn=eqn, coarse=args.coarse,
                            in_solve=traced_solve(s, eqn, None))
        out[name]["per_kernel_frac"] = r["per_kernel_frac"]
        out[name]["per_kernel_ms"] = r["per_kernel_ms"]
        out[name]["isolated_per_kernel_frac"] = r["isolated_per_kernel_frac"]
    return out


def batch_summary(pg, torch, args, n_systems=256):
    """The 256 ghost-cell IB channel systems (quad meshes of 2k-200k cells,
    log-uniform) solved as one batch: solves/s (mean of three batch
    solves after one warm-up)."""
    import numpy as np
    from phase_gb300 import workloads
    t0 = time.perf_counter()
    eqns = []
    for sp_ in workloads.gcib_specs(n_systems, seed=5):
        w = workloads.gcib_case(sp_)
        m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
        w = workloads.gcib_case(sp_, m.faces())
        e = pg.Equation(m, pg.GAMMA_SCALAR, w["bc_type"],
                        ib_circles=[w["circle"]])
        e.assemble(gamma_scalar=w["gamma"], bc_value=w["bc_value"],
                   u_face=w["u"])
        eqns.append((m, e))
    b = pg.BatchSolver(tolerance=1e-8, max_iters=20000, coarse=args.coarse)
    b.set_eqns([e for _, e in eqns])
    setup_s = time.perf_counter() - t0
    b.solve()
    ms, ok, iters = [], True, []
    for _ in range(3):
        st = b.solve()
        ms.append(b.ms)
        ok &= all(s_.status == pg.PG_OK and s_.rel_residual <= 1e-8 for s_ in st)
        iters = [s_.iters for s_ in st]
    bm = float(np.mean(ms))
    return {"workload": f"{n_systems} ghost-cell IB channel pressure systems, "
                        "quad meshes 2k-200k cells (log-uniform)",
            "total_cells": int(sum(e.n for _, e in eqns)),
            "ms_per_batch": round(bm, 3),
            "solves_per_s": round(1000.0 * n_systems / bm, 2),
            "iters": {"min": int(min(iters)), "median": float(np.median(iters)),
                      "max": int(max(iters))},
            "converged": bool(ok), "host_setup_s": round(setup_s, 2)}


def direct_summary(pg, args, nx_list=(80, 1024), cpu_nx=128):
    """The direct backend (the drop-in for EigenSparseMatrixSolver, which
    factorises and solves on every call): per workload the device time of
    the factorisation and of the solve (mean of three after a warm-up), the
    host analysis once per pattern, the factorisation's flops, and the FP64
    true residual; the CPU leg is the oracle's band LU (single thread) on
    the bubble system of the cpu_nx mesh, beside the device on the same
    system."""
    import numpy as np
    from phase_gb300 import simple
    out = {}

    def run(name, eqn):
        lu = pg.SparseLU()
        fac, sol, res = [], [], []
        for _ in range(4):
            lu.set_eqn(eqn)  # new values: factorised again
            lu.solve()
            st = lu.stats
            fac.append(st.factor_ms)
            sol.append(st.solve_ms)
            res.append(st.rel_residual)
        st = lu.stats
        f_ms = float(np.mean(fac[1:]))
        out[name] = {"n": int(eqn.n), "analyse_ms": round(st.analyse_ms, 1),
                     "factor_ms": round(f_ms, 3),
                     "solve_ms": round(float(np.mean(sol[1:])), 3),
                     "factor_gflops": round(st.flops / f_ms * 1e-6, 1),
                     "fronts": st.n_fronts, "heights": st.n_heights,
                     "max_front": st.max_front,
                     "factor_entries": int(st.factor_entries),
                     "replaced_pivots": st.replaced_pivots,
                     "rel_residual": float(max(res))}
        return lu

    for nx in nx_list:
        if nx == 80:
            eqn = simple.simple_pcorr(pg, 80, 80)["eqn"]
            run("cavity_80x80_pcorr", eqn)
        else:
            mesh, w, coeff = build_system(nx)
            eqn = pg.fv.laplacian(coeff, mesh, w["bc_type"], w["bc_value"],
                                  w["u"])
            run(f"rising_bubble_{nx}x{nx}", eqn)
    if not args.no_cpu_baseline:
        import oracle_bind
        mesh, w, coeff = build_system(cpu_nx)
        eqn = pg.fv.laplacian(coeff, mesh, w["bc_type"], w["bc_value"], w["u"])
        lu = run(f"rising_bubble_{cpu_nx}x{cpu_nx}", eqn)
        rp, ci, v, rhs = eqn.export()
        t0 = time.perf_counter()
        xo, info = oracle_bind.sparse_lu_solve(rp, ci, v, -rhs)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        x = lu.x()
        out["cpu_baseline"] = {
            "kind": "port", "cores": 1, "ms": round(cpu_ms, 1),
            "sample": f"oracle band LU (RCM order, partial pivoting) of the "
                      f"{cpu_nx}x{cpu_nx} rising-bubble system, factorise + "
                      f"solve; bandwidths {info['band']}",
            "device_ms": round(out[f"rising_bubble_{cpu_nx}x{cpu_nx}"]["factor_ms"]
                               + out[f"rising_bubble_{cpu_nx}x{cpu_nx}"]["solve_ms"], 3),
            "x_rel_diff": float(np.linalg.norm(x - xo) / np.linalg.norm(xo))}
    return out


def e2e_learned(pg, guess, seq, net, have_w, steps, torch, dev, coarse,
                coarse_warm=0, mixed_sweep=0):
    """The learned+mixed solve through the C ABI with host buffers: the
    caller holds the step's CrsEquation (5-slot layout), its rhs and the
    previous solution on the host; they are uploaded, the network predicts
    from host inputs, the solver runs from its guess, and x comes back."""
    import numpy as np
    s2 = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                               precision=pg.MIXED, coarse=coarse,
                               coarse_warm=coarse_warm, mixed_sweep=mixed_sweep)
    # the caller's geometry hint: cell centroids cut the Schwarz subdomains
    s2.setRank(seq.n)
    s2.set_row_coords(np.stack([seq.cells["cx"], seq.cells["cy"]], axis=1))
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    x_prev = pin(np.zeros(seq.n))
    times, sts, h2d, d2h = [], [], 0, 0
    for k, t in enumerate([steps[0] - 1] + list(steps)):
        rp, ci, v, rhs = seq.assemble(t).export()
        srp, sci, sv = slots_layout(rp, ci, v)
        srp, sci, sv, b, vv = pin(srp), pin(sci), pin(sv), pin(-rhs), pin(v)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        s2.setRank(seq.n)
        s2.set(srp, sci, sv)
        s2.setRhs(b)
        rel = float("inf")
        if have_w:
            g, rel = net.predict(vv, b, x_prev)
        s2.setGuess(g if rel < 1.0 else None)
        s2.solve()
        x = s2.x()
        dt = (time.perf_counter() - t1) * 1e3
        x_prev[:] = x
        if k == 0:
            continue  # first step only provides x_prev
        times.append(dt)
        sts.append(dict(s2.stats.as_dict()))
        h2d = int(srp.nbytes + sci.nbytes + sv.nbytes + b.nbytes
                  + (vv.nbytes + b.nbytes + x_prev.nbytes if have_w else 0)
                  + (x.nbytes if rel < 1.0 else 0))
        d2h = int(x.nbytes + (x.nbytes if have_w else 0))
    return {"value": round(sum(times) / len(times), 3), "unit": "ms",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "iters": [s_["iters"] for s_ in sts],
            "rel_residual": [s_["rel_residual"] for s_ in sts],
            "path": "setRank + set(rowPtr, colInd[-1 slots], vals) + setRhs + "
                    "pg_mpnn_predict(host) + setGuess + solve + x() via the C "
                    "ABI, pinned host buffers, learned+mixed"}


def run_batch(args):
    """Config 5: independent ghost-cell IB pressure systems (quad channels of
    2k-200k cells, log-uniform, one cylinder each) solved to 1e-8 as one
    batch (one analysis, one factorisation launch, one graph launch) and,
    for comparison, one solver call per system."""
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300 as pg
    from phase_gb300 import shard, workloads
    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    all_specs = workloads.gcib_specs(args.systems, seed=5)
    # ranks split the systems by nonzeros (no exchange on the data path)
    mine = shard.my_share([5 * sp_["nx"] * sp_["ny"] for sp_ in all_specs],
                          rank, world)
    specs = [all_specs[i] for i in mine]
    t_setup = time.perf_counter()
    systems = []
    for sp_ in specs:
        w = workloads.gcib_case(sp_)
        m = pg.Mesh(w["nodes"], w["cptr"], w["cind"])
        w = workloads.gcib_case(sp_, m.faces())
        e = pg.Equation(m, pg.GAMMA_SCALAR, w["bc_type"],
                        ib_circles=[w["circle"]])
        e.assemble(gamma_scalar=w["gamma"], bc_value=w["bc_value"],
                   u_face=w["u"])
        systems.append((m, e))
    eqns = [e for _, e in systems]
    b = pg.BatchSolver(tolerance=1e-8, max_iters=20000, coarse=args.coarse)
    b.set_eqns(eqns)
    setup_s = time.perf_counter() - t_setup
    for _ in range(max(1, args.warmup)):
        b.solve()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32,
                        device="cuda")
    launches0 = pg.kernel_launches()
    batch_ms, stats = [], None
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        stats = b.solve()
        batch_ms.append(b.ms)
    launches = pg.kernel_launches() - launches0
    if world > 1:
        t = torch.tensor(batch_ms, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        batch_ms = [float(x) for x in t]
    ok = all(st.status == pg.PG_OK and st.rel_residual <= 1e-8 for st in stats)
    # one solver call per system (the reference's one solve() per equation),
    # on one GPU only: the comparison is for the whole batch
    s = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000)
    single_ms, single_ok = [], True
    for e in (eqns if world == 1 else []):
        s.set_eqn(e)
        s.setGuess(None)
        s.solve()
        single_ok &= s.stats.status == pg.PG_OK
        single_ms.append(s.stats.ms)
    # one two-level solver per system (coarse correction; its analysis and
    # first factorisation in a warm-up pass, then timed)
    two_ms, two_ok, two_iters = [], True, []
    if world == 1:
        s2s = [pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                     coarse=args.coarse or 1)
               for _ in eqns]
        for s2, e in zip(s2s, eqns):
            s2.set_eqn(e)
            s2.setGuess(None)
            s2.solve()
        torch.cuda.synchronize()
        for s2, e in zip(s2s, eqns):
            s2.set_eqn(e)
            s2.setGuess(None)
            s2.solve()
            two_ok &= s2.stats.status == pg.PG_OK and s2.stats.rel_residual <= 1e-8
            two_ms.append(s2.stats.ms)
            two_iters.append(s2.stats.iters)
        del s2s
    bm = float(np.mean(batch_ms))
    n_cells = [e.n for e in eqns]
    iters = [st.iters for st in stats]
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    out = {
        "metric": "solves/s, batched GCIB pCorr systems vs per-system launches",
        "value": round(1000.0 * len(all_specs) / bm, 2), "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(1, args.warmup),
        "ms_per_step": round(bm, 3), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded GCIB channel cases, no dataset)",
        "config": {"workload": f"{len(all_specs)} ghost-cell IB channel pressure "
                               "systems, quad meshes 2k-200k cells "
                               "(log-uniform), one cylinder r in [0.1, 0.5] each",
                   "total_cells": int(sum(n_cells)), "tolerance": 1e-8,
                   "preconditioner": "Schwarz ILU(0)"
                   + (" + block-diagonal coarse correction" if args.coarse
                      else ""),
                   "tuning": b.tuning()},
        "converged": bool(ok and single_ok),
        "batch_ms": [round(x, 3) for x in batch_ms],
        "per_system_launches_ms_total": round(float(np.sum(single_ms)), 3)
        if single_ms else None,
        "per_system_solves_per_s": round(1000.0 * len(eqns) / float(np.sum(single_ms)), 2)
        if single_ms else None,
        "speedup_vs_per_system": round(float(np.sum(single_ms)) / bm, 3)
        if single_ms else None,
        "iters": {"min": int(min(iters)), "median": float(np.median(iters)),
                  "max": int(max(iters))},
        "per_system_two_level_ms_total": round(float(np.sum(two_ms)), 3)
        if two_ms else None,
        "per_system_two_level_solves_per_s":
            round(1000.0 * len(eqns) / float(np.sum(two_ms)), 2) if two_ms else None,
        "per_system_two_level_converged": bool(two_ok) if two_ms else None,
        "per_system_two_level_iters": {"min": int(min(two_iters)),
                                       "median": float(np.median(two_iters)),
                                       "max": int(max(two_iters))}
        if two_iters else None,
        "host_setup_s": round(setup_s, 2),
        "gpu_launches": int(launches),
        "rank0_systems": len(eqns),
    }
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_single(args):
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300 as pg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    nx = args.nx
    mesh, w, coeff = build_system(nx)
    n = mesh.n_cells
    dev = torch.device("cuda", local)
    d_coeff = torch.from_numpy(coeff).to(dev)
    d_bv = torch.from_numpy(w["bc_value"]).to(dev)
    d_u = torch.from_numpy(np.ascontiguousarray(w["u"]).ravel()).to(dev)
    eqn = pg.Equation(mesh, pg.GAMMA_FACE, w["bc_type"])
    prec = pg.MIXED if args.precision == "mixed" else pg.FP64
    solver = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                   precision=prec,
                                   subdomain_rows=args.subdomain_rows,
                                   mixed_sweep=args.mixed_sweep,
                                   coarse=args.coarse)
    stream = torch.cuda.ExternalStream(pg.stream_handle(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        eqn.assemble_device(gamma_face=d_coeff.data_ptr(),
                            bc_value=d_bv.data_ptr(), u_face=d_u.data_ptr())
        solver.set_eqn(eqn)
        solver.setGuess(None)
        solver.solve()
        return solver.stats.as_dict()

    for _ in range(max(3, args.warmup)):
        st = step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    stats = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = pg.kernel_launches()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))          # L2 flush (256 MB > 129 MB L2)
            ev[k][0].record(stream)
        stats.append(step())
        with torch.cuda.stream(stream):
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = pg.kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t[0])

    # kernel-level roofline on the same system: per-launch CUDA-event times
    # of the hot kernels (FP64 ones, or the float-float ones of the mixed
    # solver; both move 8-byte values and vector entries)
    a_nnz = int(eqn.nnz)
    in_solve = traced_solve(solver, eqn, None)
    roofline = kernel_roofline(pg, solver, n, a_nnz, dd=prec == pg.MIXED,
                               eqn=eqn, coarse=args.coarse, in_solve=in_solve)
    roofline["traffic"] = None  # needs a profiler: see the ncu summaries
    iters = max(1, stats[-1]["iters"])

    # e2e through the reference-facing call sequence with host buffers
    e2e = None
    if not args.no_e2e:
        rp, ci, v, rhs = eqn.export()
        srp, sci, sv = slots_layout(rp, ci, v)
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
        srp, sci, sv, b = pin(srp), pin(sci), pin(sv), pin(-rhs)
        xh = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
        s2 = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000,
                                   precision=prec,
                                   subdomain_rows=args.subdomain_rows,
                                   coarse=args.coarse)
        s2.setRank(n)
        cells = mesh.cells()
        s2.set_row_coords(np.stack([cells["cx"], cells["cy"]], axis=1))

        def e2e_step():
            s2.setRank(n)
            s2.set(srp, sci, sv)
            s2.setRhs(b)
            s2.setGuess(None)
            s2.solve()
            xh[:] = s2.x()
            return s2.stats.as_dict()

        for _ in range(2):
            e2e_step()
        times = []
        for _ in range(max(1, min(args.steps, 3))):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            e2e_st = e2e_step()
            times.append((time.perf_counter() - t1) * 1e3)
        e2e = {"value": round(sum(times) / len(times), 3), "unit": "ms",
               "h2d_bytes_per_step": int(srp.nbytes + sci.nbytes + sv.nbytes
                                         + b.nbytes),
               "d2h_bytes_per_step": int(xh.nbytes),
               "iters": e2e_st["iters"], "rel_residual": e2e_st["rel_residual"],
               "path": "setRank + set(rowPtr, colInd[-1 slots], vals) + setRhs"
                       " + solve + x() via the C ABI, pinned host buffers"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rp, ci, v, rhs = eqn.export()
        threads = len(os.sched_getaffinity(0))
        s1 = pg.SparseMatrixSolver(tolerance=1e-8, max_iters=20000, coarse=0)
        s1.set_eqn(eqn)
        s1.setGuess(None)
        s1.solve()
        val, info = cpu_solve_sample(rp, ci, v, -rhs, args.cpu_seconds,
                                     threads, fallback_iters=s1.nIters(),
                                     fallback_what="the one-level FP64 "
                                     "BiCGStab iteration count of this system")
        cpu = {"value": round(val, 1), "unit": "ms", "cores": threads,
               "kind": "port",
               "sample": f"oracle BiCGStab + Schwarz-ILU(0), {threads} "
                         f"subdomains, FP64, same system, zero guess: "
                         + info["sample"],
               "iterations": info["iterations"],
               "ms_per_iter": round(info["ms_per_iter"], 3)}

    # every timed solve must have met the tolerance on the FP64 true
    # residual; a step that did not is not a measurement of the metric
    converged = all(st["status"] == 0 and st["rel_residual"] <= 1e-8
                    for st in stats)
    if e2e is not None:
        converged = converged and e2e["rel_residual"] <= 1e-8
    if rank == 0:
        last = stats[-1]
        out = {
            "metric": METRIC, "value": round(ms, 3), "unit": "ms",
            "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype":
                "f64" if prec == pg.FP64 else "f32x2 (float-float) + f64 residual",
            "converged": converged,
            "data": "synthetic (seeded rising-bubble fields, no dataset)",
            "config": {"workload": workload_name(nx), "n_cells": n, "nnz": a_nnz,
                       "precision": args.precision,
                       "preconditioner": "Schwarz ILU(0), "
                       f"{solver.partition()[1]} subdomains"
                       + {0: "", 1: " + additive coarse correction",
                          2: " + deflated coarse correction (A-DEF1)"}[args.coarse],
                       "tolerance": 1e-8, "guess": "zero",
                       "l2": "256 MB flush write before every step; working "
                             "set > 129 MB L2"},
            "iters": last["iters"], "rel_residual": last["rel_residual"],
            "solve_ms": round(last["ms"], 3),
            "factor_ms": round(last["setup_ms"], 3),
            "ms_per_iter": round(last["ms"] / iters, 4),
            "step_ms_all": [round(x, 3) for x in step_ms],
            "solves_per_s": round(1000.0 / ms * world, 2),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk,
            "wall_s": round(wall, 3),
        }
        if not converged:
            out["invalid"] = ("a timed solve stopped above the 1e-8 relative "
                              "residual: statuses "
                              + str([st["status"] for st in stats]))
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    """CPU implementation of the same solves (the oracle: OpenMP BiCGStab
    with one ILU(0) subdomain per host thread, as Phase runs Ifpack2
    Schwarz/RILUK with one MPI rank per core), all host threads.

    sequence mode: the same time steps as our arm, each system built with
    the same host generator and solved from the previous step's CPU
    solution, as a time loop runs it.  single mode: the zero-guess solve of
    the static system, on a bounded sample."""
    import numpy as np
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle_bind as ob
    from phase_gb300 import workloads
    ob.lib()
    nx = args.nx
    w = workloads.rising_bubble(nx, nx, seed=3)
    om = ob.OracleMesh(w["nodes"], w["cptr"], w["cind"])
    faces, cells = om.faces(), om.cells()
    w = workloads.rising_bubble(nx, nx, seed=3, faces=faces, cells=cells)
    threads = len(os.sched_getaffinity(0))

    def system(t):
        if t is None:
            gamma, u = w["gamma"], w["u"]
        else:
            gamma, u = workloads.rising_bubble_step(faces, cells, w["patch"],
                                                    nx, t, seed=3)
        coeff = om.dt_over_rho(gamma, w["rho1"], w["rho2"], w["dt"])
        return om.laplacian(coeff, w["bc_type"], w["bc_value"], u)

    if args.mode == "sequence":
        W, K, t0 = max(3, args.warmup), args.steps, args.t0
        n = om.n_cells
        part = (np.arange(n, dtype=np.int64) * threads // n).astype(np.int32)
        x = None
        vals, its, rels = [], [], []
        for t in list(range(t0 - W, t0 + K)):
            rp, ci, v, rhs = system(t)
            x, st = ob.bicgstab(rp, ci, v, -rhs, tol=1e-8, max_iters=6000,
                                part=part, x0=x, threads=threads)
            if t >= t0:
                vals.append(st["ms"] + st["setup_ms"])
                its.append(st["iters"])
                rels.append(st["rel_residual"])
        value = float(np.mean(vals))
        workload = workload_name(nx) + f", time steps {t0}..{t0 + K - 1}"
        sample = (f"{K} consecutive time steps, each solved to 1e-8 (max 6000 "
                  f"iterations) from the previous step's solution; iterations "
                  f"{its}, rel. residuals {[f'{r:.1e}' for r in rels]}")
    else:
        rp, ci, v, rhs = system(None)
        vals = []
        info = None
        for _ in range(args.steps):
            val, info = cpu_solve_sample(rp, ci, v, -rhs, 40.0, threads)
            vals.append(val)
        value = float(np.median(vals))
        workload = workload_name(nx)
        sample = info["sample"]
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "ms",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(value, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded rising-bubble sequence, no dataset)",
        "config": {"workload": workload, "n_cells": int(om.n_cells),
                   "nnz": int(len(ci)), "precision": "fp64",
                   "preconditioner": f"Schwarz ILU(0), {threads} subdomains",
                   "tolerance": 1e-8},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 1), "unit": "ms",
                         "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 1), "unit": "ms",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_direct(args):
    """--mode direct: the direct backend alone (the summary of the default
    line), for profiling."""
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300 as pg
    print(json.dumps({"direct": direct_summary(pg, args, nx_list=(args.nx,))}))


def run_cylinder(args):
    """--mode cylinder: the cylinder-channel pCorr system alone (the summary
    of the default line), for profiling."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300 as pg
    print(json.dumps({"cylinder": cylinder_summary(pg, torch, args)}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        {"sequence": run_sequence, "single": run_single,
         "batch": run_batch, "direct": run_direct,
         "cylinder": run_cylinder}[args.mode](args)


if __name__ == "__main__":
    main()
