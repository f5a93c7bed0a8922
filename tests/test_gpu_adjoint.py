"""Adjoint permeability gradient on the GPU (porsol_objective_value / porsol_adjoint_gradient)
against the FP64 CPU adjoint of the oracle and central finite differences.

Tolerances: FP64 gradients agree with the oracle's to 1e-9 (normwise) when both solves run to
1e-13; the mixed-precision forward + adjoint pair to 1e-8.

Finite differences: J is about 5 and is evaluated in FP64, so a central difference with ln-k step
h resolves the derivative only to about eps |J| / h (5e-10 at h = 1e-6), while the gradient at
random cells of the 64x64x32 grid is about 1e-5.  The h = 1e-6 differences are therefore
checked to 1e-6 relative plus that round-off floor, and the 1e-6 relative agreement itself is
checked against Richardson-extrapolated central differences with h = 1e-3 and 5e-4 (truncation
O(h^4) ~ 1e-12, round-off ~ 2e-12, which only matters for the rare cell whose gradient is far
below 1e-5)."""
import numpy as np
import pytest

from adjoint import adjoint_problem, central_differences, objective
from parity import rel

pytestmark = pytest.mark.gpu


def _gpu(pkg, prob, ltype=1, precision=0, tol=1e-13):
    s = pkg.PressureSolver()
    s.init(prob.grid, prob.perm.ravel(), (0.0, 0.0, 0.0), prob.bc_type)
    o = pkg.default_solve_opts(linsolver_type=ltype, residual_tolerance=tol, precision=precision)
    fl = pkg.Fluid(pkg.FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0)
    s.solve(fl, prob.totmob, prob.bc_type, prob.bc_value, prob.src, mobdens=prob.mobdens, opts=o)
    return s, fl, o


def _oracle(orc, prob, w, target, u, mode=0, tol=1e-13):
    o = orc.OraclePressure(prob.grid, prob.bc_type)
    o.compute_inner_products(prob.perm.ravel())
    assert o.solve(prob.totmob, prob.mobdens, prob.bc_type, prob.bc_value, prob.src, tol=tol) == 0
    rc, J, g = o.adjoint_gradient(w, target, u, mode=mode, tol=tol)
    assert rc == 0
    return J, g


@pytest.mark.parametrize("ltype,precision,mode", [(0, 0, 0), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)])
def test_adjoint_matches_oracle(pkg, gpulib, orc, workloads, cart, ltype, precision, mode):
    prob, w, target, u = adjoint_problem(workloads, cart, dims=(12, 10, 8), diagonal=(mode == 1))
    s, _, _ = _gpu(pkg, prob, ltype, precision)
    J, g, st = s.adjoint_gradient(w, target, u, mode=mode)
    Jo, go = _oracle(orc, prob, w, target, u, mode)
    tol = 1e-9 if precision == 0 else 1e-8
    assert abs(J - Jo) < tol * abs(Jo)
    assert rel(g, go) < tol, rel(g, go)
    assert st.iterations > 0


def test_objective_value_matches_solution(pkg, gpulib, workloads, cart):
    prob, w, target, u = adjoint_problem(workloads, cart, dims=(9, 7, 5))
    s, _, _ = _gpu(pkg, prob)
    p, v, _ = s.solution()
    J = s.objective(w, target, u)
    assert abs(J - objective(p, v, w, target, u)) < 1e-12 * abs(J)
    assert s.objective(None, None, None) == 0.0


def test_adjoint_rejects_unsupported(pkg, gpulib, cart):
    g = cart.CartesianGrid(4, 4, 4)
    s = pkg.PressureSolver()
    bct = np.full(g.num_half_faces, pkg.BC_NEUMANN, np.int32)   # pure Neumann: regularised
    s.init(g, np.tile(np.eye(3).ravel(), g.num_cells), (0.0, 0.0, 0.0), bct)
    src = np.zeros(g.num_cells)
    src[0], src[-1] = 1.0, -1.0
    fl = pkg.Fluid(pkg.FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0)
    s.solve(fl, np.ones(g.num_cells), bct, np.zeros(g.num_half_faces), src,
            opts=pkg.default_solve_opts(linsolver_type=0, residual_tolerance=1e-10))
    with pytest.raises(pkg.PorsolError):
        s.adjoint_gradient(np.ones(g.num_cells))


def test_adjoint_config4_against_oracle_and_fd(pkg, gpulib, orc, workloads):
    """64x64x32 correlated log-normal field: 50 pressure observations + outflux through x+.
    FP64 AMG-CG forward and adjoint; FD at 20 seeded cells with ln-k step 1e-6."""
    prob = workloads.correlated_lognormal()
    w, target, u, cells = workloads.pressure_mismatch_objective(prob)
    s, fl, o = _gpu(pkg, prob, tol=1e-13)
    J, g, _ = s.adjoint_gradient(w, target, u)
    Jo, go = _oracle(orc, prob, w, target, u, tol=1e-13)
    assert abs(J - Jo) < 1e-10 * abs(Jo)
    assert rel(g, go) < 1e-8, rel(g, go)
    # scale identity: the pressure part of J does not change when every k is scaled
    assert abs(g.sum() - float(np.sum(u * s.solution()[1]))) < 1e-9 * np.abs(g).sum()

    # The perturbed solves keep the AMG hierarchy of the base solve (same_matrix): with a fixed
    # preconditioner the truncation error of CG varies smoothly with k, so it does not add noise
    # to the differences.
    o14 = pkg.default_solve_opts(linsolver_type=1, residual_tolerance=1e-14, same_matrix=1)

    def J_of(K):
        s.compute_inner_products(K.ravel())
        s.solve(fl, prob.totmob, prob.bc_type, prob.bc_value, prob.src, mobdens=prob.mobdens, opts=o14)
        return s.objective(w, target, u)

    ga = g[cells]
    fd = central_differences(J_of, prob.perm, cells, [None], h=1e-6)
    floor = 10.0 * np.finfo(float).eps * abs(J) / 1e-6
    assert np.all(np.abs(ga - fd) <= 1e-6 * np.abs(fd) + floor), np.c_[ga, fd]
    f1 = central_differences(J_of, prob.perm, cells, [None], h=1e-3)
    f2 = central_differences(J_of, prob.perm, cells, [None], h=5e-4)
    rich = (4.0 * f2 - f1) / 3.0
    err = np.abs(ga - rich) / np.abs(rich)
    # round-off of the h = 5e-4 differences, about 2e-12: it only matters for the rare cell
    # whose gradient is far below the typical 1e-5
    floor_r = 4.0 * np.finfo(float).eps * abs(J) / 5e-4
    assert np.all(np.abs(ga - rich) <= 1e-6 * np.abs(rich) + floor_r), np.c_[ga, rich, err]
    assert np.median(err) < 1e-7, np.c_[ga, rich, err]


def test_adjoint_flux_gradient_sums_to_flux(pkg, gpulib, workloads):
    """d Q / d ln s for K -> s K summed over cells equals Q (the outflux scales with k)."""
    prob = workloads.correlated_lognormal(dims=(32, 32, 16))
    s, _, _ = _gpu(pkg, prob, tol=1e-13)
    u = np.where(prob.grid.side == 2, 1.0, 0.0)
    Q, g, _ = s.adjoint_gradient(None, None, u)
    assert abs(g.sum() - Q) < 1e-9 * abs(Q)
    g3 = s.adjoint_gradient(None, None, u, mode=pkg.GRAD_LOGK_AXES)[1]
    assert np.abs(g3.sum(axis=1) - g).max() < 1e-10 * np.abs(g).max()
