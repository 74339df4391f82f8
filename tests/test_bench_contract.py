"""The bench's JSON line contract, checked on the CPU through the reference
arm (the oracle's OpenMP solve; no GPU needed) on a small grid."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args],
                       capture_output=True, text=True, timeout=600, env=e,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


def test_reference_arm_line():
    out = run_bench("--impl", "reference", "--nx", "64", "--steps", "2",
                    "--warmup", "3")
    lines = [l for l in out.splitlines() if l.strip()]
    assert len(lines) == 1, "exactly one JSON line"
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("ms per pCorr solve")
    assert d["unit"] == "ms" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["ms_per_step"] == d["value"]
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 2, 3)
    assert "workload" in d["config"] and "model" not in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["value"] == d["value"] and cb["unit"] == "ms" and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_print_nothing():
    out = run_bench("--impl", "reference", "--nx", "64", "--steps", "1",
                    "--warmup", "3", env={"RANK": "1", "WORLD_SIZE": "2"})
    assert out.strip() == ""


def test_cpu_sample_from_a_warm_start(oracle):
    """The CPU baseline's bounded sample from the previous solution (the GPU
    arms' warm start) converges in fewer iterations than from zero."""
    import importlib.util

    import numpy as np
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    spec = importlib.util.spec_from_file_location(
        "bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    from phase_gb300 import meshes
    om = oracle.OracleMesh(*meshes.rectilinear(40, 30, 1.0, 1.0))
    f = om.faces()
    rng = np.random.default_rng(5)
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rp, ci, v, _ = om.laplacian(rng.uniform(0.5, 2.0, om.n_faces), bc,
                                np.zeros(om.n_faces))
    b = rng.standard_normal(om.n_cells)
    n = om.n_cells
    xs = spla.spsolve(sp.csr_matrix((v, ci, rp), shape=(n, n)).tocsc(), b)
    x0 = xs + 1e-4 * rng.standard_normal(n)
    cold, ic = bench.cpu_solve_sample(rp, ci, v, b, 0.5, 2)
    warm, iw = bench.cpu_solve_sample(rp, ci, v, b, 0.5, 2, x0=x0)
    assert ic["sample"].startswith("ran to 1e-8")
    assert iw["sample"].startswith("ran to 1e-8")
    assert 0 < iw["iterations"] < ic["iterations"]
    assert 0 < warm and 0 < cold
