"""The finest-level smoother step of FP32 hierarchies that stages each slice of the SELL-32x4 matrix
copy in shared memory by bulk copy (k_cheb_step_bulk): parity on a system large enough to use it, and
its bounded wait.  The step engages when the finest level has one thread per row (at least 20,000
rows), so the grids here have about 60,000 face unknowns."""
import numpy as np
import pytest

from parity import gpu_solve, oracle_solve, rel

pytestmark = pytest.mark.gpu


def _expected():
    """The self-test system: row i holds 1/4, 1/2, 3/4, 1 at columns i, i+1, i+5, i+17 (mod 64);
    d_j = 1 + j/64, r = 2, x = 0, c1 = 1/2, c2 = 1/4 (every operation exact in FP32)."""
    n = 64
    d = (1.0 + np.arange(n) / 64.0).astype(np.float32)
    acc = np.zeros(n, np.float32)
    for t, off in enumerate((0, 1, 5, 17)):
        acc += np.float32(0.25 * (t + 1)) * d[(np.arange(n) + off) % n]
    r = np.float32(2.0) - acc
    dn = np.float32(0.5) * d + np.float32(0.25) * r
    return r, dn, d + dn


def test_selftest_step_values(pkg, gpulib):
    rc, r, d, x = pkg.selftest_bulk_wait(False)
    assert rc == 0
    er, ed, ex = _expected()
    assert np.array_equal(r, er) and np.array_equal(d, ed) and np.array_equal(x, ex)


def test_selftest_wait_runs_out_and_context_stays_usable(pkg, gpulib):
    rc, r, _, _ = pkg.selftest_bulk_wait(True)
    assert rc == 6  # PORSOL_ERR_TIMEOUT
    assert np.all(r == 2.0)  # the step wrote nothing
    rc, r, d, x = pkg.selftest_bulk_wait(False)
    assert rc == 0
    er, ed, ex = _expected()
    assert np.array_equal(r, er) and np.array_equal(d, ed) and np.array_equal(x, ex)


def test_mixed_precision_with_bulk_staged_level(pkg, gpulib, orc, workloads):
    """Mixed precision at 19,200 cells (59,800 face unknowns, finest level bulk-staged) reaches 1e-8
    relative flux error against the FP64 oracle, and repeating the solve is bitwise identical."""
    prob = workloads.anisotropic_corey(dims=(32, 30, 20))
    o = oracle_solve(orc, prob, tol=1e-13, dirichlet_guess=True)
    a = gpu_solve(pkg, prob, ltype=1, tol=1e-11, precision=pkg.MIXED)
    rows, _ = a["solver"].amg_info()
    assert len(rows) >= 3 and rows[0] >= 20000
    assert rel(a["v"], o["v"]) < 1e-8
    assert rel(a["p"], o["p"]) < 1e-8
    b = gpu_solve(pkg, prob, ltype=1, tol=1e-11, precision=pkg.MIXED)
    for k in ("pi", "p", "v"):
        assert np.array_equal(a[k], b[k]), k
    assert a["stats"].iterations == b["stats"].iterations
