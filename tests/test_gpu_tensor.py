"""Tensor mobilities (PORSOL_FLUID_TENSOR, the MimeticIPAnisoRelpermEvaluator inner product)
on the GPU against the FP64 oracle; the scalar special case against the scalar model."""
import numpy as np
import pytest

from parity import rel
from tensor_mobility import tensor_problem

pytestmark = pytest.mark.gpu
GRAV = (0.0, 0.0, -9.81)


def _gpu(pkg, g, K, lam, rlam, bct, bcv, src, grav=GRAV, **opt):
    s = pkg.PressureSolver()
    s.init(g, K.ravel(), grav, bct)
    o = pkg.default_solve_opts(residual_tolerance=1e-13, **opt)
    s.solve(pkg.Fluid(pkg.FLUID_TENSOR, 1.0, 1.0, 0.0, 0.0), lam.ravel(), bct, bcv, src,
            mobdens=None if rlam is None else rlam.ravel(), opts=o)
    return s


@pytest.mark.parametrize("ltype,precision", [(0, 0), (1, 0), (1, 1)])
def test_tensor_mobility_matches_oracle(pkg, gpulib, orc, workloads, cart, ltype, precision):
    g, K, lam, rlam, bct, bcv, src = tensor_problem(workloads, cart)
    s = _gpu(pkg, g, K, lam, rlam, bct, bcv, src, linsolver_type=ltype, precision=precision)
    p, v, _ = s.solution()
    o = orc.OraclePressure(g, bct)
    o.compute_inner_products(K.ravel(), GRAV)
    assert o.solve_tensor(lam, rlam, bct, bcv, src, tol=1e-13) == 0
    po, vo, _ = o.solution()
    tol = 1e-10 if precision == 0 else 1e-8
    assert rel(p, po) < tol and rel(v, vo) < tol, (rel(p, po), rel(v, vo))


def test_scalar_tensor_equals_scalar_model(pkg, gpulib, workloads, cart):
    g, K, lam, rlam, bct, bcv, src = tensor_problem(workloads, cart)
    m = np.random.default_rng(2).uniform(0.5, 2.0, g.num_cells)
    md = 900.0 * m
    s = _gpu(pkg, g, K, (m[:, None] * np.eye(3).ravel()[None]), md[:, None] * np.eye(3).ravel()[None], bct, bcv,
             src)
    p1, v1, _ = s.solution()
    s2 = pkg.PressureSolver()
    s2.init(g, K.ravel(), GRAV, bct)
    s2.solve(pkg.Fluid(pkg.FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0), m, bct, bcv, src, mobdens=md,
             opts=pkg.default_solve_opts(residual_tolerance=1e-13))
    p2, v2, _ = s2.solution()
    assert rel(p1, p2) < 1e-11 and rel(v1, v2) < 1e-11


def test_non_symmetric_lambda_k_is_rejected(pkg, gpulib, workloads, cart):
    g, K, lam, rlam, bct, bcv, src = tensor_problem(workloads, cart)
    lam = lam.reshape(-1, 3, 3).copy()
    lam[:, 0, 1] += 0.3                      # no longer commutes with K
    lam[:, 1, 0] += 0.3
    with pytest.raises(pkg.PorsolError):
        _gpu(pkg, g, K, lam.reshape(-1, 9), None, bct, bcv, src)
