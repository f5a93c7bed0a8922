"""The FP64 CPU adjoint of the oracle against central finite differences of the oracle's own
forward solve, and the scale identities of the gradient (CPU only)."""
import numpy as np
import pytest

from adjoint import adjoint_problem, central_differences, objective


def _oracle_J(orc, prob, w, target, u):
    def J_of(K):
        o = orc.OraclePressure(prob.grid, prob.bc_type)
        o.compute_inner_products(K.ravel())
        assert o.solve(prob.totmob, prob.mobdens, prob.bc_type, prob.bc_value, prob.src, tol=1e-15) == 0
        p, v, _ = o.solution()
        return objective(p, v, w, target, u)
    return J_of


@pytest.mark.parametrize("mode", [0, 1])
def test_oracle_adjoint_matches_finite_differences(orc, workloads, cart, mode):
    prob, w, target, u = adjoint_problem(workloads, cart, diagonal=(mode == 1))
    o = orc.OraclePressure(prob.grid, prob.bc_type)
    o.compute_inner_products(prob.perm.ravel())
    assert o.solve(prob.totmob, prob.mobdens, prob.bc_type, prob.bc_value, prob.src, tol=1e-15) == 0
    rc, J, grad = o.adjoint_gradient(w, target, u, mode=mode, tol=1e-15)
    assert rc == 0
    J_of = _oracle_J(orc, prob, w, target, u)
    assert abs(J - J_of(prob.perm)) < 1e-13 * abs(J)
    cells = np.random.default_rng(5).choice(prob.grid.num_cells, 8, replace=False)
    axes = [None] if mode == 0 else [0, 1, 2]
    fd = central_differences(J_of, prob.perm, cells, axes)
    ad = grad[cells] if mode == 0 else grad[cells].ravel()
    # central differences with step 1e-6 resolve about 1e-9 absolute here (round-off of J)
    assert np.linalg.norm(ad - fd) / np.linalg.norm(fd) < 1e-6
    if mode == 1:
        rc0, _, g0 = o.adjoint_gradient(w, target, u, mode=0, tol=1e-15)
        assert rc0 == 0 and np.abs(grad.sum(axis=1) - g0).max() < 1e-12 * np.abs(g0).max()


def test_oracle_adjoint_scale_identities(orc, workloads, cart):
    """Scaling every k by s leaves p unchanged and scales v by s, so without sources the
    pressure-mismatch gradient sums to 0 and the outflux gradient sums to the outflux."""
    prob, w, target, _ = adjoint_problem(workloads, cart, dims=(8, 6, 5))
    prob.src[:] = 0.0
    prob.bc_value[prob.grid.side == 3] = 0.0
    o = orc.OraclePressure(prob.grid, prob.bc_type)
    o.compute_inner_products(prob.perm.ravel())
    assert o.solve(prob.totmob, prob.mobdens, prob.bc_type, prob.bc_value, prob.src, tol=1e-14) == 0
    rc, J, g = o.adjoint_gradient(w, target, None, tol=1e-14)
    assert rc == 0 and abs(g.sum()) < 1e-10 * np.abs(g).sum()
    u = np.where(prob.grid.side == 2, 1.0, 0.0)
    rc, Q, g = o.adjoint_gradient(None, None, u, tol=1e-14)
    assert rc == 0 and abs(g.sum() - Q) < 1e-10 * abs(Q)


def test_oracle_adjoint_rejects_unsupported(orc, cart):
    """Pure Neumann/periodic problems have no adjoint here (rc 2)."""
    g = cart.CartesianGrid(3, 3, 3, unique_bids=True)
    bct = np.where(g.boundary, orc.BC_PERIODIC, orc.BC_NEUMANN).astype(np.int32)
    o = orc.OraclePressure(g, bct, g.periodic_partner_bids())
    o.compute_inner_products(np.tile(np.eye(3).ravel(), g.num_cells))
    bcv = np.where(g.side == 1, 1.0, np.where(g.side == 2, -1.0, 0.0))
    assert o.solve(np.ones(g.num_cells), np.zeros(g.num_cells), bct, bcv, np.zeros(g.num_cells), tol=1e-12) == 0
    rc, _, _ = o.adjoint_gradient(np.ones(g.num_cells), None, None)
    assert rc == 2
