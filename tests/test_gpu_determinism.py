"""Reductions and assembly are fixed-order (no floating-point atomics), so repeating a solve
gives bitwise identical results, also across solver handles."""
import numpy as np
import pytest

from parity import gpu_solve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ltype,precision", [(0, 0), (1, 0), (1, 1)])
def test_repeated_solves_are_bitwise_identical(pkg, gpulib, workloads, ltype, precision):
    prob = workloads.anisotropic_corey(dims=(20, 16, 10))
    a = gpu_solve(pkg, prob, ltype=ltype, tol=1e-11, precision=precision, post=True)
    b = gpu_solve(pkg, prob, ltype=ltype, tol=1e-11, precision=precision, post=True)
    for k in ("pi", "p", "v"):
        assert np.array_equal(a[k], b[k]), k
    assert a["stats"].iterations == b["stats"].iterations
