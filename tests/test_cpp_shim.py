"""The C++ SparseMatrixSolver plugin: compiles against the stand-in Phase
headers (CPU) and solves through libphase_gb300 (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "phase_gb300", "cpp")


def compile_shim(out):
    import __graft_entry__
    __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(CPP, "standin"),
           "-I", CPP, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_test.cpp"),
           os.path.join(CPP, "Gb300SparseMatrixSolver.cpp"),
           "-L", os.path.join(ROOT, "phase_gb300"), "-lphase_gb300",
           "-Wl,-rpath," + os.path.join(ROOT, "phase_gb300"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_shim_compiles(tmp_path):
    compile_shim(str(tmp_path / "shim_test"))


@pytest.mark.gpu
def test_shim_solves_on_gpu(tmp_path):
    exe = str(tmp_path / "shim_test")
    compile_shim(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Krylov iterations" in r.stdout
