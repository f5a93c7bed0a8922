"""GPU explicit upstream transport (EulerUpstream::transportSolve) against the CPU oracle."""
import numpy as np
import pytest

from parity import gpu_solve, relmax

pytestmark = pytest.mark.gpu


def _setup(pkg, orc, workloads, cart, dims=(10, 8, 4), grav=(0.0, 0.0, 0.0), capillary=False, seed=3):
    rng = np.random.default_rng(seed)
    prob = workloads.case5(dims=dims, seed=seed, sat=rng.uniform(0.0, 0.4, int(np.prod(dims))))
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
