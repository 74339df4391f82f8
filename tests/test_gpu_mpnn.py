"""Learned initial guess: the GPU network's loss and gradients against an
FP64 CPU restatement, and what training gains over the previous solution.

Bars: loss within 1e-3 relative (FP32 activations vs FP64); parameter
gradients of the GPU backward pass within 3e-2 relative of FP64 central
finite differences on the restatement (on the 40 largest gradients);
after training on a short sequence, the guess's residual ||b - A g||/||b||
on held-out steps is below the previous solution's.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import mpnn_oracle
from phase_gb300 import meshes

pytestmark = pytest.mark.gpu


def _system(oracle, nx=14, ny=11, seed=0):
    nodes, cptr, cind = meshes.rectilinear(nx, ny, 1.0, 1.2)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    rng = np.random.default_rng(seed)
    bc = np.where(f["rcell"] < 0, 1, 1).astype(np.int32)
    bc[np.flatnonzero(f["rcell"] < 0)[:nx]] = 0
    gamma = np.exp(rng.uniform(-3, 3, om.n_faces))
    rp, ci, v, rhs = om.laplacian(gamma, bc, np.zeros(om.n_faces),
                                  rng.standard_normal((om.n_faces, 2)))
    b = -rhs
    xs, _ = oracle.bicgstab(rp, ci, v, b, tol=1e-13, max_iters=5000)
    c = om.cells()
    xp = xs + 0.3 * np.sin(3 * c["cx"]) * np.std(xs) + 0.05 * rng.standard_normal(xs.size) * np.std(xs)
    return rp, ci, v, b, xp, xs


def test_mpnn_loss_and_gradients_match_cpu_restatement(pg, oracle):
    from phase_gb300.guess import Mpnn
    rp, ci, v, b, xp, xs = _system(oracle)
    net = Mpnn(seed=5)
    rng = np.random.default_rng(1)
    params = (0.25 * rng.standard_normal(net.n_params)).astype(np.float32)
    net.set_params(params)
    net.set_graph(rp, ci)
    g_gpu, loss_gpu = net.gradient(v, b, xp, xs)
    w = mpnn_oracle.round_bf16(params).astype(np.float64)
    loss_cpu, _ = mpnn_oracle.loss(w, rp, ci, v, b, xp, xs)
    assert abs(loss_gpu - loss_cpu) / loss_cpu < 1e-3
    idx = np.argsort(-np.abs(g_gpu))[:40]
    for k in idx:
        h = 1e-4 * max(abs(w[k]), 1e-2)
        wp, wm = w.copy(), w.copy()
        wp[k] += h
        wm[k] -= h
        fd = (mpnn_oracle.loss(wp, rp, ci, v, b, xp, xs)[0] -
              mpnn_oracle.loss(wm, rp, ci, v, b, xp, xs)[0]) / (2 * h)
        assert abs(g_gpu[k] - fd) <= 3e-2 * abs(fd) + 1e-6, (k, g_gpu[k], fd)


def test_fused_inference_matches_training_forward_and_restatement(pg, oracle):
    """pg_mpnn_predict runs the forward pass as one kernel per layer with
    the dense products on tensor cores (TF32 with split activations, FP32
    accuracy).  Its guess matches the training forward (FP32 FMAs) up to the
    summation order: the FP64 loss of the predicted guess equals the loss
    the training path reports to 1e-5 relative; and it agrees with the FP64
    restatement's guess (FP32 activations: the correction g - x_prev within
    1e-3 relative), as does the reported residual."""
    from phase_gb300.guess import Mpnn
    # 23 x 17 = 391 cells: six full 64-cell tiles and a ragged one
    rp, ci, v, b, xp, xs = _system(oracle, 23, 17, seed=3)
    net = Mpnn(seed=2)
    rng = np.random.default_rng(7)
    params = (0.25 * rng.standard_normal(net.n_params)).astype(np.float32)
    net.set_params(params)
    net.set_graph(rp, ci)
    g, rel = net.predict(v, b, xp)
    _, loss_train = net.gradient(v, b, xp, xs)
    A = sp.csr_matrix((v, ci, rp))
    r0 = A @ xp - b
    res = A @ g - b
    loss_pred = (res @ res) / (r0 @ r0) + ((g - xs) @ (g - xs)) / ((xp - xs) @ (xp - xs))
    assert abs(loss_pred - loss_train) <= 1e-5 * loss_train
    w = mpnn_oracle.round_bf16(params).astype(np.float64)
    _, g_cpu = mpnn_oracle.loss(w, rp, ci, v, b, xp, xs)
    assert np.linalg.norm((g - xp) - (g_cpu - xp)) <= 1e-3 * np.linalg.norm(g_cpu - xp)
    rel_cpu = np.linalg.norm(A @ g_cpu - b) / np.linalg.norm(b)
    assert abs(rel - rel_cpu) <= 1e-3 * rel_cpu
    assert abs(rel - np.linalg.norm(res) / np.linalg.norm(b)) <= 1e-12 * rel


def test_training_beats_previous_solution(pg):
    torch = pytest.importorskip("torch")
    from phase_gb300.guess import BubbleSequence, Mpnn
    seq = BubbleSequence(64)
    n = seq.n
    steps = 40
    s = pg.SparseMatrixSolver(tolerance=1e-10, max_iters=5000)
    xs = torch.zeros((steps + 1, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for t in range(1, steps + 1):
        s.set_eqn(seq.assemble(t))
        s.solve()
        s.x_device(xs[t].data_ptr())
    net = Mpnn(seed=2)
    net.set_graph(seq.row_ptr, seq.col_ind)
    for ep in range(6):
        for t in range(2, 33):
            v, b = seq.device_system(t)
            net.train_step_device(v, b.data_ptr(), xs[t - 1].data_ptr(),
                                  xs[t].data_ptr(), 3e-3)
    learned, previous = [], []
    for t in range(34, steps + 1):
        v, b = seq.device_system(t)
        g = torch.empty(n, dtype=torch.float64, device="cuda")
        learned.append(net.predict_device(v, b.data_ptr(), xs[t - 1].data_ptr(),
                                          g.data_ptr()))
        bb = b.cpu().numpy()
        rp, ci, vv, _ = seq.eqn.export()
        A = sp.csr_matrix((vv, ci, rp))
        xprev = xs[t - 1].cpu().numpy()
        previous.append(np.linalg.norm(bb - A @ xprev) / np.linalg.norm(bb))
    assert np.mean(learned) < np.mean(previous)


def test_weights_file_round_trip(pg, tmp_path):
    from phase_gb300 import guess
    a, b = guess.Mpnn(seed=3), guess.Mpnn(seed=4)
    f = tmp_path / "w.bin"
    a.save(f)
    b.load(f)
    assert np.array_equal(a.get_params(), b.get_params())
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a weights file")
    with pytest.raises(pg.PhaseError):
        b.load(bad)


def test_triple_dump_of_a_sequence(pg, tmp_path):
    """The sequence dump (triples.py format) holds systems whose stored
    solutions meet the solver tolerance."""
    import scipy.sparse as sp
    from phase_gb300 import guess, triples
    guess.dump_sequence(str(tmp_path / "d"), nx=64, steps=[5, 6, 7])
    r = triples.TripleReader(str(tmp_path / "d"))
    assert r.steps == [5, 6, 7] and r.n == 64 * 64
    for t, vals, b, x in r:
        A = sp.csr_matrix((vals, r.col_ind, r.row_ptr), shape=(r.n, r.n))
        assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) <= 1.01e-8
