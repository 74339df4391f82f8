"""The C++ SparseMatrixSolver plugin: compiles against the stand-in Phase
headers (CPU) and solves through libphase_gb300 (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "phase_gb300", "cpp")


def compile_shim(out, main="shim_test.cpp"):
    import __graft_entry__
    __graft_entry__.build()
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(CPP, "standin"),
           "-I", CPP, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", main),
           os.path.join(CPP, "Gb300SparseMatrixSolver.cpp"),
           "-L", os.path.join(ROOT, "phase_gb300"), "-lphase_gb300",
           "-Wl,-rpath," + os.path.join(ROOT, "phase_gb300"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_shim_compiles(tmp_path):
    compile_shim(str(tmp_path / "shim_test"))


def test_shim_setup_rejects_unbuilt_options(tmp_path):
    """The plugin's setup accepts the Belos keys' values the library builds
    and throws Phase's Exception for the rest (no silent substitution)."""
    exe = str(tmp_path / "shim_setup_test")
    compile_shim(exe, "shim_setup_test.cpp")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_shim_solves_on_gpu(tmp_path):
    exe = str(tmp_path / "shim_test")
    compile_shim(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Krylov iterations" in r.stdout
