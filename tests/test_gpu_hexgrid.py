"""The GPU path on non-Cartesian hexahedra (sheared and distorted grids) against the oracle."""
import numpy as np
import pytest

from hexgrids import distorted, linear_field_problem, sheared
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
