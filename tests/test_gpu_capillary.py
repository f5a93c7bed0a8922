"""GPU ImplicitCapillarity step and rock-table transport against the CPU oracle.

Rock tables (RockJfunc) change every mobility and the capillary pressure of the transport path;
ImplicitCapillarity::transportSolve (euler/ImplicitCapillarity_impl.hpp:138-226) adds a pressure
solve with fixed capillary mobilities and the volume-matching root search.  Both sides get the same
inputs; the pressure solves run to 1e-12 so the saturations agree to 1e-9."""
import ctypes as C

import numpy as np
import pytest

import capillary as cp
from parity import relmax

pytestmark = pytest.mark.gpu


def _gpu_objects(pkg, c, rocks=True, opts=None):
    g = c["grid"]
    T = pkg.TransportSolver()
    T.init(g, c["K"].ravel(), c["poro"], pkg.Fluid(pkg.FLUID_COREY2, cp.MU1, cp.MU2, cp.RHO1, cp.RHO2),
           c["sat_type"], c["sat_value"], partner_bid=c["partner"], opts=opts)
    if rocks:
        T.set_rock_tables(c["tables"], c["cell_rock"], True, cp.SIGMA_COS_THETA)
    P = pkg.PressureSolver()
    P.init(g, c["K"].ravel(), (0.0, 0.0, 0.0), c["bct"], c["partner"])
    return T, P


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("ltype", [0, 1])
def test_capillary_matches_oracle(pkg, gpulib, orc, workloads, cart, periodic, ltype):
    c = cp.case(orc, workloads, cart, periodic=periodic)
    To, Po = cp.oracle_objects(orc, c)
    rc, s_orc, shift_o, rit_o, _ = orc.capillary_solve(
        Po, To, c["sat"], c["flux"], c["bct"], c["bcv"],
        opts=orc.CapillaryOpts.defaults(residual_tolerance=1e-13, linsolver_type=ltype))
    assert rc == 0
    T, P = _gpu_objects(pkg, c)
    s_gpu, st = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"],
                                  opts=pkg.default_capillary_opts(residual_tolerance=1e-13, linsolver_type=ltype))
    assert relmax(s_gpu, s_orc) < 1e-9
    assert abs(st.shift - shift_o) <= 1e-9 * max(1.0, abs(shift_o))
    assert abs(st.root_iterations - rit_o) <= 1
    pv = c["poro"] * c["grid"].volume
    assert abs((pv * s_gpu).sum() - (pv * c["sat"]).sum()) / pv.sum() <= 2e-12


def test_capillary_mixed_precision_and_relaxation(pkg, gpulib, orc, workloads, cart):
    c = cp.case(orc, workloads, cart, dims=(12, 10, 6))
    T, P = _gpu_objects(pkg, c)
    s64, st64 = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"],
                                  opts=pkg.default_capillary_opts(residual_tolerance=1e-12))
    s32, st32 = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"],
                                  opts=pkg.default_capillary_opts(residual_tolerance=1e-12, precision=pkg.MIXED))
    assert relmax(s32, s64) < 1e-8
    sr, _ = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"],
                              opts=pkg.default_capillary_opts(residual_tolerance=1e-12, update_relaxation=0.5))
    np.testing.assert_allclose(sr, 0.5 * c["sat"] + 0.5 * s64, rtol=0, atol=1e-14)


def test_capillary_device_entry_point(pkg, gpulib, orc, workloads, cart):
    import torch
    c = cp.case(orc, workloads, cart)
    T, P = _gpu_objects(pkg, c)
    o = pkg.default_capillary_opts(residual_tolerance=1e-12)
    s_host, st_h = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"], opts=o)
    dev = torch.device("cuda:0")
    d_sat = torch.tensor(c["sat"], dtype=torch.float64, device=dev)
    d_flux = torch.tensor(c["flux"], dtype=torch.float64, device=dev)
    d_bct = torch.tensor(c["bct"], dtype=torch.int32, device=dev)
    d_bcv = torch.tensor(c["bcv"], dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    st = pkg.CapillaryStats()
    g = np.zeros(3)
    rc = pkg.lib().porsol_capillary_solve_device(T.h, P.h, C.c_void_p(d_sat.data_ptr()), g.ctypes.data,
                                                 C.c_void_p(d_flux.data_ptr()), None, C.c_void_p(d_bct.data_ptr()),
                                                 C.c_void_p(d_bcv.data_ptr()), C.byref(o), C.byref(st))
    assert rc == 0, pkg.lib().porsol_transport_last_error(T.h)
    assert np.array_equal(d_sat.cpu().numpy(), s_host)
    assert st.shift == st_h.shift


@pytest.mark.parametrize("capillary", [False, True])
def test_transport_with_rock_tables_matches_oracle(pkg, gpulib, orc, workloads, cart, capillary):
    """EulerUpstream with rock tables: table mobilities (upstream cell's rock), J-scaled capillary
    pressure, averaged mean-saturation mobilities of both rocks, and the per-rock CFL factors
    including the capillary bound (ReservoirPropertyCapillary_impl.hpp:213-282)."""
    c = cp.case(orc, workloads, cart, dims=(10, 8, 4), seed=5)
    topt = dict(method_capillary=int(capillary))
    T, _ = _gpu_objects(pkg, c, opts=pkg.default_transport_opts(**topt))
    To, _ = cp.oracle_objects(orc, c)
    To.opts = orc.TransportOpts.defaults(**topt)
    pv = (c["poro"] * c["grid"].volume).sum()
    # The capillary CFL bound of the tables is far below the viscous one, and the centred
    # mean-saturation mobilities of the capillary term (EulerUpstreamResidual_impl.hpp:226-236)
    # keep drawing water from cells at s_min, so the explicit scheme leaves [0, 1] over long
    # spans; 8 capillary CFL steps move the saturation by up to 0.19 and stay in range.
    if capillary:
        t = 8 * To.cfl(c["flux"])
    else:
        t = 0.05 * pv / np.abs(c["flux"][c["grid"].side == 1]).sum()
    s_gpu, st = T.solve(c["sat"], t, c["flux"])
    rc, s_orc, ns, rep = To.solve(c["sat"], t, c["flux"])
    assert rc == 0
    assert st.small_steps == ns and st.repeats == rep
    assert relmax(s_gpu, s_orc) < 1e-11
    assert abs(st.cfl_dt - To.cfl(c["flux"])) <= 1e-12 * st.cfl_dt


def test_rock_table_errors(pkg, gpulib, orc, workloads, cart):
    c = cp.case(orc, workloads, cart)
    T, P = _gpu_objects(pkg, c, rocks=False)
    bad = [np.array(t) for t in c["tables"]]
    bad[0][3, 3] = bad[0][2, 3] + 1.0   # J not monotone
    with pytest.raises(pkg.PorsolError) as e:
        T.set_rock_tables(bad, c["cell_rock"])
    assert e.value.code == 2
    with pytest.raises(pkg.PorsolError) as e:
        T.set_rock_tables(c["tables"], np.full(c["grid"].num_cells, 2, np.int32))   # rock 2 does not exist
    assert e.value.code == 2
    # without rock tables the inverse capillary-pressure curve is 0: no shift can be bracketed
    with pytest.raises(pkg.PorsolError) as e:
        T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"])
    assert e.value.code == 1
    # the saturation is left unchanged on failure, and the handle stays usable
    T.set_rock_tables(c["tables"], c["cell_rock"], True, cp.SIGMA_COS_THETA)
    s, st = T.capillary_solve(P, c["sat"], c["flux"], c["bct"], c["bcv"])
    assert st.root_iterations > 0 and np.isfinite(s).all()
