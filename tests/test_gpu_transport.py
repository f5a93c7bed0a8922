"""GPU explicit upstream transport (EulerUpstream::transportSolve) against the CPU oracle."""
import numpy as np
import pytest

from parity import gpu_solve, relmax

pytestmark = pytest.mark.gpu


def _setup(pkg, orc, workloads, cart, dims=(10, 8, 4), grav=(0.0, 0.0, 0.0), capillary=False, seed=3):
    rng = np.random.default_rng(seed)
    prob = workloads.layered_lognormal(dims=dims, seed=seed, sat=rng.uniform(0.0, 0.4, int(np.prod(dims))))
    if capillary:
        # The no-rock capillary pressure is 1e5 (1 - s) Pa; with a 1 Pa drop it swamps the
        # viscous flux and the explicit scheme (which has no capillary CFL bound without rock
        # tables) leaves [0, 1].  A 1000 bar drop keeps capillarity a perturbation.
        prob.bc_value = prob.bc_value * 1e8
    g = gpu_solve(pkg, prob, ltype=1, tol=1e-12, post=True)
    flux = g["v"]
    nc = prob.grid.num_cells
    _, mu1, mu2, r1, r2 = prob.fluid
    topt = dict(method_capillary=int(capillary))
    T = pkg.TransportSolver()
    T.init(prob.grid, prob.perm.ravel(), prob.poro, pkg.Fluid(pkg.FLUID_COREY2, mu1, mu2, r1, r2), prob.sat_type,
           prob.sat_value, opts=pkg.default_transport_opts(**topt))
    O = orc.OracleTransport(prob.grid, prob.perm.ravel(), prob.poro, orc.Fluid(mu1, mu2, r1, r2), prob.sat_type,
                            prob.sat_value, opts=orc.TransportOpts.defaults(**topt))
    return prob, flux, T, O


@pytest.mark.parametrize("capillary", [False, True])
def test_transport_matches_oracle(pkg, gpulib, orc, workloads, cart, capillary):
    prob, flux, T, O = _setup(pkg, orc, workloads, cart, capillary=capillary)
    pv = (prob.poro * prob.grid.volume).sum()
    qin = -flux[prob.grid.side == 1].sum()
    t = 0.05 * pv / qin
    s_gpu, st = T.solve(prob.sat, t, flux)
    rc, s_orc, ns, rep = O.solve(prob.sat, t, flux)
    assert rc == 0
    assert st.small_steps == ns and st.repeats == rep
    assert relmax(s_gpu, s_orc) < 1e-11
    assert s_gpu.min() > -1e-3 and s_gpu.max() < 1 + 1e-3


def test_transport_gravity(pkg, gpulib, orc, workloads, cart):
    prob, flux, T, O = _setup(pkg, orc, workloads, cart, dims=(6, 5, 6))
    grav = (0.0, 0.0, 9.81 * 1e-12)   # small so that the CFL stays viscous-dominated
    pv = (prob.poro * prob.grid.volume).sum()
    qin = -flux[prob.grid.side == 1].sum()
    t = 0.02 * pv / qin
    s_gpu, st = T.solve(prob.sat, t, flux, grav=grav)
    rc, s_orc, ns, rep = O.solve(prob.sat, t, flux, grav=grav)
    assert rc == 0 and st.small_steps == ns
    assert relmax(s_gpu, s_orc) < 1e-11


def test_transport_retry_and_failure(pkg, gpulib, orc, workloads, cart):
    """A step count too small for the flux (maximum_small_steps = 1) makes the saturation leave
    [-0.001, 1.001]; the retry loop doubles the steps (EulerUpstream_impl.hpp:181-213) exactly as
    the oracle does."""
    prob, flux, T, O = _setup(pkg, orc, workloads, cart)
    _, mu1, mu2, r1, r2 = prob.fluid
    opt = dict(method_capillary=0, maximum_small_steps=1, minimum_small_steps=1)
    T2 = pkg.TransportSolver()
    T2.init(prob.grid, prob.perm.ravel(), prob.poro, pkg.Fluid(pkg.FLUID_COREY2, mu1, mu2, r1, r2), prob.sat_type,
            prob.sat_value, opts=pkg.default_transport_opts(**opt))
    O2 = orc.OracleTransport(prob.grid, prob.perm.ravel(), prob.poro, orc.Fluid(mu1, mu2, r1, r2), prob.sat_type,
                             prob.sat_value, opts=orc.TransportOpts.defaults(**opt))
    pv = (prob.poro * prob.grid.volume).sum()
    qin = -flux[prob.grid.side == 1].sum()
    t = 0.05 * pv / qin
    s_gpu, st = T2.solve(prob.sat, t, flux)
    rc, s_orc, ns, rep = O2.solve(prob.sat, t, flux)
    assert rc == 0 and rep >= 1
    assert st.repeats == rep and st.small_steps == ns
    assert relmax(s_gpu, s_orc) < 1e-11
    # far too long a step with retries exhausted: error status, saturation restored
    with pytest.raises(pkg.PorsolError) as e:
        T2.solve(prob.sat, 1e4 * t, flux)
    assert e.value.code == 4


def test_transport_periodic_and_wells(pkg, gpulib, orc, workloads, cart):
    """Periodic in y (pressure and saturation), Dirichlet x-/x+, plus an injector and a producer
    (injection rates: positive injects water, negative produces with the cell's fractional flow)."""
    g = cart.CartesianGrid(8, 6, 3, unique_bids=True)
    nc = g.num_cells
    rng = np.random.default_rng(12)
    K = workloads.iso_perm(np.exp(rng.normal(np.log(100 * workloads.MILLIDARCY), 1.0, nc)))
    poro = np.full(nc, 0.2)
    pb = g.periodic_partner_bids()
    ybnd = (g.side == 3) | (g.side == 4)
    bct, bcv = workloads.x_dirichlet_bc(g)
    bct[ybnd] = workloads.BC_PERIODIC
    bcv[ybnd] = 0.0
    partner = np.where(ybnd, pb, 0).astype(np.int32)
    src = np.zeros(nc)
    src[5], src[nc - 7] = 2e-14, -2e-14
    sat = rng.uniform(0.0, 0.3, nc)
    prob = workloads.Problem("per", g, K, poro, bct, bcv, src, sat, (1, 1e-3, 1e-2, 1000.0, 850.0))
    r = gpu_solve(pkg, prob, ltype=1, tol=1e-13, post=True, partner=partner)
    flux = r["v"]
    st_t = np.where(ybnd, workloads.BC_PERIODIC, workloads.BC_DIRICHLET).astype(np.int32)
    sv = np.ones(g.num_half_faces)
    fl = pkg.Fluid(pkg.FLUID_COREY2, 1e-3, 1e-2, 1000.0, 850.0)
    T = pkg.TransportSolver()
    T.init(g, K.ravel(), poro, fl, st_t, sv, partner_bid=partner, opts=pkg.default_transport_opts(method_capillary=0))
    O = orc.OracleTransport(g, K.ravel(), poro, orc.Fluid(1e-3, 1e-2, 1000.0, 850.0), st_t, sv, partner_bid=partner,
                            opts=orc.TransportOpts.defaults(method_capillary=0))
    pv = (poro * g.volume).sum()
    t = 0.02 * pv / np.abs(flux[g.side == 1]).sum()
    s_gpu, st = T.solve(sat, t, flux, injection=src)
    rc, s_orc, ns, rep = O.solve(sat, t, flux, injection=src)
    assert rc == 0 and st.small_steps == ns and st.repeats == rep
    assert relmax(s_gpu, s_orc) < 1e-11


def test_transport_slug_constant_velocity(pkg, gpulib, orc, cart):
    """The fixture of attic/euler/EulerSolverTester.hpp:69-100,155-180 on the GPU: a constant velocity
    v = (1, 0, 0) (flux = (v . n) A), a slug of water in the middle third, water entering through x-.
    GPU = oracle, and the water volume grows by exactly the injected amount while the front has not
    reached x+."""
    g = cart.CartesianGrid(12, 3, 2)
    nc = g.num_cells
    q = (g.fnormal[:, 0] * 1.0) * g.area
    K = np.zeros((nc, 9))
    K[:, 0] = K[:, 4] = K[:, 8] = 1.0
    poro = np.full(nc, 0.25)
    st = np.full(g.num_half_faces, pkg.BC_DIRICHLET, np.int32)
    sv = np.ones(g.num_half_faces)
    T = pkg.TransportSolver()
    T.init(g, K.ravel(), poro, pkg.Fluid(pkg.FLUID_COREY2, 1.0, 2.0, 1000.0, 800.0), st, sv,
           opts=pkg.default_transport_opts(method_capillary=0))
    O = orc.OracleTransport(g, K.ravel(), poro, orc.Fluid(1.0, 2.0, 1000.0, 800.0), st, sv,
                            opts=orc.TransportOpts.defaults(method_capillary=0))
    s0 = np.zeros(nc)
    s0[(g.ccentroid[:, 0] > 1 / 3) & (g.ccentroid[:, 0] < 2 / 3)] = 1.0
    s_gpu, stats = T.solve(s0, 0.005, q)
    rc, s_orc, ns, rep = O.solve(s0, 0.005, q)
    assert rc == 0 and stats.small_steps == ns and stats.repeats == rep
    assert relmax(s_gpu, s_orc) < 1e-12
    inflow = -q[g.side == 1].sum()
    assert s_gpu[g.ccentroid[:, 0] > 0.9].max() == 0.0
    assert abs(((s_gpu - s0) * poro * g.volume).sum() - inflow * 0.005) < 1e-12
