"""CPU tests of the C ABI library: it builds, loads, exports every entry
point declared in include/phase_gb300.h, and fails loudly (no CPU path)
when no GPU is present."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "phase_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300
    return phase_gb300


def test_exports_every_declared_symbol(built):
    syms = declared_symbols()
    assert len(syms) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", built.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (pg_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    # the Python binding declares exactly the header's entry points
    assert sorted(built.PROTOTYPES) == syms


def test_defaults_match_belos(built):
    c = built.default_cfg()
    # TrilinosBelosSparseMatrixSolver::setup defaults (tol 1e-8, 500 iters)
    assert c.tolerance == 1e-8 and c.max_iters == 500
    assert c.precond == built.PREC_ILU0


def test_no_silent_cpu_path_without_gpu(built):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from phase_gb300 import meshes
    with pytest.raises(built.PhaseError) as ei:
        built.Mesh(*meshes.rectilinear(4, 4))
    assert ei.value.status == built.PG_CUDA_ERROR
    with pytest.raises(built.PhaseError):
        built.SparseMatrixSolver()


def test_header_is_c99_and_links_from_c(built, tmp_path):
    """A C caller: the header compiles as strict C99 and the program links
    against the library and reads the default configuration (no GPU call)."""
    exe = str(tmp_path / "c_abi_check")
    lib_dir = os.path.dirname(built.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "c_abi_check.c"),
                    "-L", lib_dir, "-lphase_gb300", "-Wl,-rpath," + lib_dir,
                    "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "max_iters 500" in r.stdout


def test_kernel_trace_entry_points_check_arguments(built):
    # argument checks come before any CUDA call: no GPU needed
    lib = built.lib()
    assert lib.pg_solver_trace_kernels(None, 1) == built.PG_BAD_ARG
    ms = np.zeros(4)
    cnt = np.zeros(4, np.int64)
    assert lib.pg_solver_kernel_times(None, ms.ctypes.data, cnt.ctypes.data,
                                      None) == built.PG_BAD_ARG
