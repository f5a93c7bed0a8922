"""The GPU path on non-Cartesian hexahedra (sheared and distorted grids) against the oracle."""
import numpy as np
import pytest

from hexgrids import distorted, linear_field_problem, refined_top, sheared
from parity import gpu_solve, oracle_solve, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [sheared, distorted])
@pytest.mark.parametrize("ltype", [0, 1])
def test_hexgrid_matches_oracle(pkg, gpulib, orc, workloads, cart, make, ltype):
    g = make(cart)
    rng = np.random.default_rng(3)
    nc = g.num_cells
    k = np.exp(rng.normal(0.0, 1.0, nc))
    K = workloads.diag_perm(k, 0.5 * k, 2.0 * k)
    K[:, 1] = K[:, 3] = 0.1 * k
    bct, bcv = workloads.x_dirichlet_bc(g)
    prob = workloads.Problem("hex", g, K, np.full(nc, 0.2), bct, bcv, rng.normal(0, 0.01, nc), np.zeros(nc),
                             (0, 1.0, 1.0, 0.0, 0.0), totmob=np.exp(rng.normal(0, 0.3, nc)), mobdens=np.zeros(nc))
    r = gpu_solve(pkg, prob, ltype=ltype, tol=1e-13)
    o = oracle_solve(orc, prob, tol=1e-13)
    Wg, gg = r["solver"].inner_products()
    Wo, go = o["oracle"].inner_products()
    assert rel(Wg, Wo) < 1e-13
    assert rel(r["pi"], o["pi"]) < 1e-10 and rel(r["p"], o["p"]) < 1e-10 and rel(r["v"], o["v"]) < 1e-10


def test_linear_field_on_sheared_grid(pkg, gpulib, workloads, cart):
    g = sheared(cart)
    prob = linear_field_problem(workloads, g)
    r = gpu_solve(pkg, prob, ltype=1, tol=1e-14)
    assert np.abs(r["p"] - g.ccentroid @ np.array([1.5, -0.7, 0.4])).max() < 1e-9


def _refined_problem(workloads):
    g = refined_top(5, 4, 3, 2)
    rng = np.random.default_rng(9)
    nc = g.num_cells
    k = np.exp(rng.normal(0.0, 1.0, nc))
    bct, bcv = workloads.x_dirichlet_bc(g)
    return workloads.Problem("refined", g, workloads.iso_perm(k), np.full(nc, 0.2), bct, bcv,
                             rng.normal(0, 0.01, nc), np.zeros(nc), (0, 1.0, 1.0, 0.0, 0.0),
                             totmob=np.exp(rng.normal(0, 0.3, nc)), mobdens=np.zeros(nc))


@pytest.mark.parametrize("ltype", [0, 1])
def test_nine_face_cells_match_oracle(pkg, gpulib, orc, workloads, ltype):
    """Cells with up to 12 faces take the MAXNF = 12 kernels (static IP, assembly, recovery)."""
    prob = _refined_problem(workloads)
    r = gpu_solve(pkg, prob, ltype=ltype, tol=1e-13, post=True)
    o = oracle_solve(orc, prob, tol=1e-13, post=True)
    assert rel(r["solver"].inner_products()[0], o["oracle"].inner_products()[0]) < 1e-13
    assert rel(r["pi"], o["pi"]) < 1e-10 and rel(r["p"], o["p"]) < 1e-10 and rel(r["v"], o["v"]) < 1e-10


def test_nine_face_cells_adjoint(pkg, gpulib, orc, workloads):
    prob = _refined_problem(workloads)
    r = gpu_solve(pkg, prob, ltype=1, tol=1e-13)
    nc = prob.grid.num_cells
    w = np.zeros(nc)
    w[::7] = 1.0
    t = np.full(nc, 0.4)
    J, g, _ = r["solver"].adjoint_gradient(w, t, None)
    o = oracle_solve(orc, prob, tol=1e-13)["oracle"]
    rc, Jo, go = o.adjoint_gradient(w, t, None, tol=1e-13)
    assert rc == 0 and abs(J - Jo) < 1e-10 * abs(Jo) and rel(g, go) < 1e-9
