"""The oracle's ImplicitCapillarity step and rock tables (CPU only).

ImplicitCapillarity::transportSolve (euler/ImplicitCapillarity_impl.hpp:138-226) moves the
capillary pressure by the constant that keeps the pore-volume-weighted saturation
(MatchSaturatedVolumeFunctor.hpp:49-112), so the saturation volume is conserved to the root
tolerance 1e-12; relaxation mixes old and new saturations linearly; without rock tables the inverse
capillary-pressure curve is 0 and no shift can be bracketed.  The table path of the transport
residual reduces to the closed-form Corey-2 path for tables that sample s^2 and (1-s)^2."""
import numpy as np
import pytest

import capillary as cp


@pytest.mark.parametrize("periodic", [False, True])
def test_capillary_conserves_saturation_volume(orc, workloads, cart, periodic):
    c = cp.case(orc, workloads, cart, periodic=periodic)
    T, P = cp.oracle_objects(orc, c)
    rc, s, shift, rit, _ = orc.capillary_solve(P, T, c["sat"], c["flux"], c["bct"], c["bcv"],
                                               opts=orc.CapillaryOpts.defaults(residual_tolerance=1e-12))
    assert rc == 0 and 0 < rit <= 40
    pv = c["poro"] * c["grid"].volume
    assert abs((pv * s).sum() - (pv * c["sat"]).sum()) / pv.sum() <= 1.01e-12
    lo = np.where(c["cell_rock"] == 0, 0.1, 0.15)
    hi = np.where(c["cell_rock"] == 0, 0.9, 0.85)
    assert (s >= lo).all() and (s <= hi).all()   # satFromCapPress clamps to [s_min, s_max]
    assert np.ptp(s) > 0.3                        # the J scaling spreads the saturations


def test_capillary_relaxation(orc, workloads, cart):
    c = cp.case(orc, workloads, cart)
    T, P = cp.oracle_objects(orc, c)
    o1 = orc.CapillaryOpts.defaults(residual_tolerance=1e-12)
    o2 = orc.CapillaryOpts.defaults(residual_tolerance=1e-12, update_relaxation=0.25)
    rc1, s1, sh1, _, _ = orc.capillary_solve(P, T, c["sat"], c["flux"], c["bct"], c["bcv"], opts=o1)
    rc2, s2, sh2, _, _ = orc.capillary_solve(P, T, c["sat"], c["flux"], c["bct"], c["bcv"], opts=o2)
    assert rc1 == rc2 == 0 and sh1 == sh2
    np.testing.assert_allclose(s2, 0.75 * c["sat"] + 0.25 * s1, rtol=0, atol=1e-15)


def test_capillary_without_rock_tables_fails(orc, workloads, cart):
    c = cp.case(orc, workloads, cart)
    T, P = cp.oracle_objects(orc, c)
    T.fluid = orc.Fluid(cp.MU1, cp.MU2, cp.RHO1, cp.RHO2)
    rc, *_ = orc.capillary_solve(P, T, c["sat"], c["flux"], c["bct"], c["bcv"])
    assert rc == 4


def _corey_table(n=2001):
    s = np.linspace(0.0, 1.0, n)
    return np.column_stack([s, s * s, (1 - s) ** 2, 1.0 - s])


def test_table_residual_reduces_to_corey(orc, workloads, cart):
    c = cp.case(orc, workloads, cart)
    g = c["grid"]
    rt = orc.RockTables([_corey_table()], np.zeros(g.num_cells, np.int32), False)
    opts = orc.TransportOpts.defaults(method_capillary=0)
    args = (g, c["K"].ravel(), c["poro"])
    Tt = orc.OracleTransport(*args, rt.fluid(cp.MU1, cp.MU2, cp.RHO1, cp.RHO2), c["sat_type"], c["sat_value"],
                             opts=opts)
    Tc = orc.OracleTransport(*args, orc.Fluid(cp.MU1, cp.MU2, cp.RHO1, cp.RHO2), c["sat_type"], c["sat_value"],
                             opts=opts)
    grav = (0.0, 0.0, 9.81e-6)
    rt_ = Tt.residual(c["sat"], c["flux"], grav=grav)
    rc_ = Tc.residual(c["sat"], c["flux"], grav=grav)
    assert np.abs(rt_ - rc_).max() <= 1e-5 * np.abs(rc_).max()
    f_tab = orc.cfl_factors(rt.fluid(cp.MU1, cp.MU2), c["K"].ravel(), c["poro"])
    f_cor = orc.cfl_factors(orc.Fluid(cp.MU1, cp.MU2, 0.0, 0.0))
    np.testing.assert_allclose(f_tab[:2], f_cor[:2], rtol=1e-3)
    assert f_cor[2] == 0.0 and f_tab[2] > 0.0   # J = 1 - s has slope -1: a capillary CFL bound appears
