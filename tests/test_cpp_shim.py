"""The C++ drop-in templates (Opm::gpu::IncompFlowSolverHybrid / EulerUpstream) compile
against the reference's concepts and, on a GPU, reproduce a linear pressure field exactly."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "shim_test.cpp")
HOST = os.path.join(ROOT, "opm-porsol_gb300", "host")
INC = os.path.join(ROOT, "include")


def _compile(pkg, out):
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    libdir = os.path.dirname(pkg.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wno-unused-variable", "-I", HOST, "-I", INC, SRC, "-o", out,
           "-L", libdir, "-lporsol_gpu", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_shim_compiles(pkg, tmp_path):
    _compile(pkg, str(tmp_path / "shim_test"))


@pytest.mark.gpu
def test_shim_runs_on_gpu(pkg, gpulib, tmp_path):
    exe = _compile(pkg, str(tmp_path / "shim_test"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
    assert "=== rate=" in r.stdout and ", IT=" in r.stdout   # linsolver_verbosity 1 reports the CG
