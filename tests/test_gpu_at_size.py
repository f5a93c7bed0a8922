"""Parity at the workload sizes: the GPU path against the FP64 CPU oracle on the full-size
two-phase pressure problem (100x100x50 anisotropic Corey-2, 500k cells), on two IMPES steps
(pressure solve + EulerUpstream::transportSolve) of the layered workload at 100x100x25, and on
periodic upscaling sub-grids whose sides span 8..32.  The reference path restated by the oracle:
IncompFlowSolverHybrid.hpp:1387-1420 (ILU0-CG), :1672-1730 (recovery), :707-807
(postProcessFluxes), EulerUpstream_impl.hpp:153-385 (transport).  Tolerances: relative 2-norm
flux and pressure error <= 1e-10 for the FP64 path, <= 1e-8 for mixed precision."""
import numpy as np
import pytest

from parity import gpu_solve, oracle_solve, rel
from upscaling import oracle_keff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def config2(orc, workloads):
    prob = workloads.anisotropic_corey()          # 100 x 100 x 50, sigma 2, kz = 0.1 kx, s ~ U[0, 1]
    assert prob.grid.num_cells == 500_000
    o = oracle_solve(orc, prob, tol=1e-13, dirichlet_guess=True, post=True)
    return prob, o


@pytest.mark.parametrize("precision,tol,bound", [(0, 1e-12, 1e-10), (1, 1e-11, 1e-8)])
def test_config2_full_size_against_oracle(pkg, gpulib, config2, precision, tol, bound):
    prob, o = config2
    g = gpu_solve(pkg, prob, ltype=1, tol=tol, precision=precision, post=True)
    ev, ep = rel(g["v"], o["v"]), rel(g["p"], o["p"])
    assert ev <= bound and ep <= bound, (precision, ev, ep)
    g["solver"].close()


def _impes_steps(run_pressure, run_transport, prob, nsteps, step_pv=0.1 / 50):
    """Pressure solve then transport step, nsteps times; the step length injects step_pv pore
    volumes at the inflow of the first pressure solve (the IMPES workload's rule)."""
    g = prob.grid
    pv = float((prob.poro * g.volume).sum())
    sat = prob.sat.copy()
    dt, substeps = None, []
    for _ in range(nsteps):
        v = run_pressure(sat)
        if dt is None:
            dt = step_pv * pv / float(-v[g.side == 1].sum())
        sat, ns = run_transport(sat, dt, v)
        substeps.append(ns)
    return sat, v, substeps


@pytest.mark.parametrize("precision,tol,bound,sat_bound", [(0, 1e-12, 1e-9, 1e-7), (1, 1e-11, 1e-7, 1e-6)])
def test_impes_two_steps_against_oracle(pkg, gpulib, orc, workloads, precision, tol, bound, sat_bound):
    """Relative flux error after the second pressure solve <= bound; saturation after two steps
    within sat_bound, absolute in every cell and relative in the 2-norm (cells at the front amplify
    the flux difference: up to 1.4e-8 absolute at FP64)."""
    prob = workloads.layered_lognormal(dims=(100, 100, 25))
    g = prob.grid
    model, mu1, mu2, r1, r2 = prob.fluid
    fl = pkg.Fluid(model, mu1, mu2, r1, r2)
    topt = dict(method_capillary=0)
    # GPU: one pressure handle and one transport handle, as the IMPES loop of the benchmark
    P = pkg.PressureSolver()
    P.init(g, prob.perm.ravel(), (0.0, 0.0, 0.0), prob.bc_type)
    T = pkg.TransportSolver()
    T.init(g, prob.perm.ravel(), prob.poro, fl, prob.sat_type, prob.sat_value,
           opts=pkg.default_transport_opts(**topt))
    opts = pkg.default_solve_opts(linsolver_type=1, residual_tolerance=tol, precision=precision)

    def gpu_p(sat):
        P.solve(fl, sat, prob.bc_type, prob.bc_value, prob.src, opts=opts)
        P.post_process_fluxes()
        return P.solution()[1]

    def gpu_t(sat, dt, v):
        s, st = T.solve(sat, dt, v)
        return s, st.small_steps

    # oracle: ILU0-CG to 1e-13 and the restated transportSolve
    O = orc.OraclePressure(g, prob.bc_type)
    O.compute_inner_products(prob.perm.ravel())
    OT = orc.OracleTransport(g, prob.perm.ravel(), prob.poro, orc.Fluid(mu1, mu2, r1, r2), prob.sat_type,
                             prob.sat_value, opts=orc.TransportOpts.defaults(**topt))

    def orc_p(sat):
        m1, m2 = sat * sat / mu1, (1 - sat) ** 2 / mu2
        assert O.solve(m1 + m2, r1 * m1 + r2 * m2, prob.bc_type, prob.bc_value, prob.src, tol=1e-13,
                       dirichlet_guess=True) == 0
        O.post_process_fluxes()
        return O.solution()[1]

    def orc_t(sat, dt, v):
        rc, s, ns, _ = OT.solve(sat, dt, v)
        assert rc == 0
        return s, ns

    s_gpu, v_gpu, ns_gpu = _impes_steps(gpu_p, gpu_t, prob, 2)
    s_orc, v_orc, ns_orc = _impes_steps(orc_p, orc_t, prob, 2)
    assert ns_gpu == ns_orc
    assert rel(v_gpu, v_orc) <= bound
    assert np.abs(s_gpu - s_orc).max() <= sat_bound, np.abs(s_gpu - s_orc).max()
    assert rel(s_gpu, s_orc) <= sat_bound
    assert s_gpu.max() > 0.5   # water has entered
    P.close()
    T.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_upscaling_sides_8_to_32_against_oracle(pkg, gpulib, orc, workloads, precision):
    """Sub-grids whose sides span the batched workload's range U{8..32}, in one batch."""
    union, sizes, K = workloads.periodic_subgrids(seed=23, sides=[8, 13, 19, 26, 32])
    s = pkg.PressureSolver()
    keff, st = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                                  pkg.default_solve_opts(residual_tolerance=1e-12, precision=precision))
    for gi in range(len(sizes)):
        c0, c1 = union.cellpos[gi], union.cellpos[gi + 1]
        ref = oracle_keff(orc, union.grids[gi], K[c0:c1])
        err = np.abs(keff[gi] - ref).max() / np.abs(ref).max()
        assert err < (1e-9 if precision == 0 else 1e-8), (int(sizes[gi]), err)
    s.close()
