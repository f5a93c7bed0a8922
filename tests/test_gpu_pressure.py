"""GPU pressure path (IncompFlowSolverHybrid on sm_103a) against the FP64 CPU oracle.

Tolerances: FP64 results are compared at 1e-10 relative (both solvers run to a 1e-12
residual reduction, so the remaining differences are summation order and iteration
count); integer structure is compared exactly; the mixed-precision path must reach
1e-8 relative flux error against the FP64 oracle.
"""
import numpy as np
import pytest

from parity import gpu_solve, oracle_solve, rel, relmax

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-10


def _problem_small(workloads, cart, dims=(7, 6, 5), aniso=True, seed=11):
    rng = np.random.default_rng(seed)
    g = cart.CartesianGrid(*dims)
    nc = g.num_cells
    k = np.exp(rng.normal(np.log(100 * workloads.MILLIDARCY), 1.5, nc))
    K = workloads.diag_perm(k, 0.7 * k, (0.1 if aniso else 1.0) * k)
    bct, bcv = workloads.x_dirichlet_bc(g)
    sat = rng.uniform(0, 1, nc)
    return workloads.Problem("small", g, K, np.full(nc, 0.2), bct, bcv, np.zeros(nc), sat,
                             (1, 1e-3, 5e-3, 1000.0, 850.0))


def test_structure_matches_oracle(pkg, gpulib, orc, workloads, cart):
    prob = _problem_small(workloads, cart)
    g = gpu_solve(pkg, prob, ltype=0)
    o = orc.OraclePressure(prob.grid, prob.bc_type)
    for a, b in zip(g["solver"].structure(), o.structure()):
        assert np.array_equal(a, b)


def test_periodic_structure_matches_oracle(pkg, gpulib, orc, cart):
    grid = cart.CartesianGrid(5, 4, 3, unique_bids=True)
    pb = grid.periodic_partner_bids()
    bct = np.where(grid.boundary, pkg.BC_PERIODIC, pkg.BC_NEUMANN).astype(np.int32)
    s = pkg.PressureSolver()
    K = np.tile(np.eye(3).ravel(), grid.num_cells)
    s.init(grid, K, (0, 0, 0), bct, pb)
    o = orc.OraclePressure(grid, bct, pb)
    for a, b in zip(s.structure(), o.structure()):
        assert np.array_equal(a, b)


def test_static_inner_products(pkg, gpulib, orc, workloads, cart):
    """computeInnerProducts: W and gravity flux per cell, full tensors and gravity on."""
    rng = np.random.default_rng(5)
    grid = cart.CartesianGrid(5, 4, 3, 0.3, 0.2, 0.7)
    nc = grid.num_cells
    A = rng.normal(size=(nc, 3, 3))
    K = np.einsum("cij,ckj->cik", A, A) + 0.5 * np.eye(3)
    bct, bcv = workloads.x_dirichlet_bc(grid)
    s = pkg.PressureSolver()
    grav = (0.0, 0.3, -9.81)
    s.init(grid, K.reshape(nc, 9).ravel(), grav, bct)
    o = orc.OraclePressure(grid, bct)
    o.compute_inner_products(K.reshape(nc, 9).ravel(), grav)
    Wg, gg = s.inner_products()
    Wo, go = o.inner_products()
    assert relmax(Wg, Wo) < 1e-13
    assert relmax(gg, go) < 1e-13


@pytest.mark.parametrize("n", [1, 2, 4])
def test_ipeval_fixture_on_gpu(pkg, gpulib, cart, n):
    """The static inverse inner products of the attic/mimetic/mimetic_ipeval_test.cpp fixture
    (K = diag(10, 1, 0.1), unit cube in 1, 8, 64 cells) equal the recorded copy
    (tests/golden/ipeval_binv.json)."""
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ipeval_binv.json")))["grids"][str(n)]
    g = cart.CartesianGrid(n, n, n, 1.0 / n, 1.0 / n, 1.0 / n)
    K = np.zeros((g.num_cells, 9))
    K[:, 0], K[:, 4], K[:, 8] = 10.0, 1.0, 0.1
    s = pkg.PressureSolver()
    s.init(g, K.ravel(), (0.0, 0.0, 0.0), np.full(g.num_half_faces, pkg.BC_NEUMANN, np.int32))
    B, _ = s.inner_products()
    B = B.reshape(g.num_cells, 36)
    np.testing.assert_allclose(B[0], gold["first_cell"], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(B[-1], gold["last_cell"], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(np.linalg.norm(B, axis=1), gold["cell_norms"], rtol=1e-13)


@pytest.mark.parametrize("fluid", ["corey", "cellwise_gravity"])
def test_assembled_system(pkg, gpulib, orc, workloads, cart, fluid):
    """assembleDynamic: the global matrix and right-hand side entry by entry."""
    prob = _problem_small(workloads, cart)
    nc = prob.grid.num_cells
    grav = (0.0, 0.0, 0.0)
    if fluid == "cellwise_gravity":
        rng = np.random.default_rng(2)
        prob.fluid = (0, 1.0, 1.0, 0.0, 0.0)
        prob.totmob = rng.uniform(0.5, 2.0, nc)
        prob.mobdens = rng.uniform(100, 900, nc)
        grav = (0.0, 0.0, 9.81)
        prob.src = rng.normal(size=nc) * 1e-3
        prob.src -= prob.src.mean()
    s = pkg.PressureSolver()
    s.init(prob.grid, prob.perm.ravel(), grav, prob.bc_type)
    model, mu1, mu2, r1, r2 = prob.fluid
    fl = pkg.Fluid(model, mu1, mu2, r1, r2)
    sat = prob.totmob if model == 0 else prob.sat
    s.solve(fl, sat, prob.bc_type, prob.bc_value, prob.src, mobdens=prob.mobdens if model == 0 else None,
            opts=pkg.default_solve_opts(linsolver_type=0, residual_tolerance=1e-12))
    S, rhs = s.system()
    o = orc.OraclePressure(prob.grid, prob.bc_type)
    o.compute_inner_products(prob.perm.ravel(), grav)
    tm, md = prob.mobilities()
    o.assemble(tm, md, prob.bc_type, prob.bc_value, prob.src)
    so = o.system()
    assert relmax(S, so["S"]) < 1e-12
    assert relmax(rhs, so["rhs"]) < 1e-12


@pytest.mark.parametrize("ltype", [0, 1])
def test_solve_matches_oracle(pkg, gpulib, orc, workloads, cart, ltype):
    prob = _problem_small(workloads, cart)
    g = gpu_solve(pkg, prob, ltype=ltype)
    o = oracle_solve(orc, prob, dirichlet_guess=(ltype != 0))
    assert rel(g["pi"], o["pi"]) < FP64_TOL
    assert rel(g["p"], o["p"]) < FP64_TOL
    assert rel(g["v"], o["v"]) < FP64_TOL
    if ltype == 0:
        # identical ILU0-CG algorithm: iteration counts agree
        assert abs(g["stats"].iterations - o["iterations"]) <= 1
    assert g["stats"].mass_balance < 1e-9


@pytest.mark.parametrize("precision,tol,bound", [(0, 1e-12, FP64_TOL), (1, 1e-11, 1e-8)])
def test_kcycle_type2_matches_oracle(pkg, gpulib, orc, workloads, precision, tol, bound):
    """linsolver_type 2 (the reference's KAMG, solveLinearSystemKAMG :1609-1666) runs the K-cycle:
    the same converged answer as the oracle, and no more CG iterations than the V-cycle of type 1
    on a system deep enough for a K-level (several AMG levels)."""
    prob = workloads.anisotropic_corey(dims=(40, 30, 20))
    o = oracle_solve(orc, prob, tol=1e-13, dirichlet_guess=True)
    k = gpu_solve(pkg, prob, ltype=2, tol=tol, precision=precision)
    v = gpu_solve(pkg, prob, ltype=1, tol=tol, precision=precision)
    assert k["stats"].amg_levels >= 3
    assert rel(k["v"], o["v"]) < bound and rel(k["p"], o["p"]) < bound
    assert k["stats"].iterations <= v["stats"].iterations, (k["stats"].iterations, v["stats"].iterations)


def test_unit_cube_ilu0(pkg, gpulib, orc, workloads):
    """10^3 cells, CG + ILU0 to 1e-10, plain FP64."""
    prob = workloads.unit_cube_lognormal()
    g = gpu_solve(pkg, prob, ltype=0, tol=1e-10)
    o = oracle_solve(orc, prob, tol=1e-10)
    assert g["stats"].iterations == o["iterations"]
    assert rel(g["v"], o["v"]) < 1e-9
    assert rel(g["p"], o["p"]) < 1e-9


def test_pure_neumann_regularised(pkg, gpulib, orc, workloads, cart):
    """No Dirichlet face: S[0][0] *= 2 (IncompFlowSolverHybrid.hpp:1398-1400), sources drive flow."""
    prob = _problem_small(workloads, cart, dims=(5, 5, 4))
    nc = prob.grid.num_cells
    prob.bc_type[:] = pkg.BC_NEUMANN
    prob.bc_value[:] = 0.0
    prob.src = np.zeros(nc)
    prob.src[0] = 1e-6
    prob.src[-1] = -1e-6
    for ltype in (0, 1):
        g = gpu_solve(pkg, prob, ltype=ltype)
        o = oracle_solve(orc, prob, dirichlet_guess=(ltype != 0))
        assert rel(g["v"], o["v"]) < FP64_TOL
        assert rel(g["p"], o["p"]) < FP64_TOL


def test_neumann_inflow(pkg, gpulib, orc, workloads, cart):
    """Neumann outflux on x- plus Dirichlet on x+."""
    prob = _problem_small(workloads, cart)
    grid = prob.grid
    prob.bc_type[grid.side == 1] = pkg.BC_NEUMANN
    prob.bc_value[grid.side == 1] = -1e-9
    g = gpu_solve(pkg, prob, ltype=1)
    o = oracle_solve(orc, prob, dirichlet_guess=True)
    assert rel(g["v"], o["v"]) < FP64_TOL


def test_periodic_solve_and_post_process(pkg, gpulib, orc, workloads, cart):
    """Fully periodic unit-drop problem (setupUpscalingConditions Periodic,
    setupBoundaryConditions.hpp:136-157), then postProcessFluxes."""
    grid = cart.CartesianGrid(6, 5, 4, unique_bids=True)
    pb = grid.periodic_partner_bids()
    nc = grid.num_cells
    rng = np.random.default_rng(9)
    A = rng.normal(size=(nc, 3, 3)) * 0.3
    K = (np.einsum("cij,ckj->cik", A, A) + np.eye(3)).reshape(nc, 9)
    bct = np.where(grid.boundary, pkg.BC_PERIODIC, pkg.BC_NEUMANN).astype(np.int32)
    bcv = np.zeros(grid.num_half_faces)
    bcv[grid.side == 3] = 1.0
    bcv[grid.side == 4] = -1.0
    prob = workloads.Problem("per", grid, K, np.full(nc, 0.2), bct, bcv, np.zeros(nc), np.zeros(nc),
                             (0, 1.0, 1.0, 0.0, 0.0), totmob=np.ones(nc), mobdens=np.zeros(nc))
    for ltype in (0, 1):
        g = gpu_solve(pkg, prob, ltype=ltype, post=True, partner=pb)
        o = oracle_solve(orc, prob, dirichlet_guess=(ltype != 0), post=True, partner=pb)
        assert rel(g["pi"], o["pi"]) < FP64_TOL
        assert rel(g["v"], o["v"]) < FP64_TOL
        assert abs(g["maxmod"] - o["maxmod"]) <= 1e-10 * np.abs(o["v"]).max()


def test_post_process_antisymmetric(pkg, gpulib, workloads, cart):
    prob = _problem_small(workloads, cart)
    g = gpu_solve(pkg, prob, ltype=1, post=True, tol=1e-6)
    cf = g["solver"].structure()[0]
    v = g["v"]
    grid = prob.grid
    interior = ~grid.boundary
    # twin half-faces carry opposite fluxes after post-processing
    order = np.argsort(cf[interior], kind="stable")
    vi = v[interior][order].reshape(-1, 2)
    assert np.abs(vi[:, 0] + vi[:, 1]).max() <= 1e-15 * np.abs(v).max()


def test_mixed_precision_flux_error(pkg, gpulib, orc, workloads):
    """Mixed precision (FP32 CG recurrences and AMG, FP64 solution with residual replacements) reaches
    1e-8 relative flux error (sigma=2 field)."""
    prob = workloads.anisotropic_corey(dims=(24, 20, 10))
    o = oracle_solve(orc, prob, tol=1e-13, dirichlet_guess=True)
    g = gpu_solve(pkg, prob, ltype=1, tol=1e-11, precision=pkg.MIXED)
    assert rel(g["v"], o["v"]) < 1e-8
    assert rel(g["p"], o["p"]) < 1e-8
    assert g["stats"].outer_iterations >= 2


@pytest.mark.parametrize("n", [50, 60])
def test_known_answer_on_gpu(pkg, gpulib, workloads, n):
    """The reference's recorded known-answer errors (timing_results.txt) from the GPU AMG-CG path."""
    import json, os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answer.json")))["cases"][str(n)]
    prob = workloads.known_answer(n)
    g = gpu_solve(pkg, prob, ltype=1, tol=1e-10)
    l1, l2, li = workloads.error_norms(prob, g["p"])
    assert abs(l1 - gold["L1"]) <= 6e-6 * gold["L1"] + 1e-9
    assert abs(l2 - gold["L2"]) <= 6e-6 * gold["L2"] + 1e-9
    assert abs(li - gold["Linf"]) <= 3e-8


def test_errors_are_reported(pkg, gpulib, workloads, cart):
    prob = _problem_small(workloads, cart)
    s = pkg.PressureSolver()
    s.init(prob.grid, prob.perm.ravel(), (0, 0, 0), prob.bc_type)
    fl = pkg.Fluid(*prob.fluid)
    with pytest.raises(pkg.PorsolError) as e:
        s.solve(fl, prob.sat, prob.bc_type, prob.bc_value, prob.src, opts=pkg.default_solve_opts(linsolver_type=7))
    assert e.value.code == 8
    with pytest.raises(pkg.PorsolError) as e:
        s.solve(fl, prob.sat, prob.bc_type, prob.bc_value, prob.src,
                opts=pkg.default_solve_opts(linsolver_type=0, linsolver_maxit=2, residual_tolerance=1e-14))
    assert e.value.code == 1 and "failed to converge in 2 iterations" in str(e.value)
    bad = prob.sat.copy()
    bad[3] = np.nan
    with pytest.raises(pkg.PorsolError) as e:
        s.solve(fl, bad, prob.bc_type, prob.bc_value, prob.src)
    assert e.value.code == 3
    # the handle stays usable after errors
    s.solve(fl, prob.sat, prob.bc_type, prob.bc_value, prob.src)
    # an empty grid is rejected up front (the reference's init skips it)
    empty = cart.CartesianGrid(1, 1, 1)
    empty.num_cells = 0
    empty.facepos = np.zeros(1, np.int32)
    for k in ("neighbour", "bid", "area"):
        setattr(empty, k, getattr(empty, k)[:0])
    for k in ("fcentroid", "fnormal", "ccentroid"):
        setattr(empty, k, getattr(empty, k)[:0])
    empty.volume = empty.volume[:0]
    e2 = pkg.PressureSolver()
    with pytest.raises(pkg.PorsolError) as e:
        e2.init(empty, np.zeros(0), (0, 0, 0), np.zeros(0, np.int32))
    assert e.value.code == 2 and "no cells" in str(e.value)
