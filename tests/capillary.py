"""ImplicitCapillarity cases shared by the CPU (oracle) and GPU tests.

A layered log-normal box (or a y-periodic one) with two J-function rocks assigned by layer
parity, a heterogeneous initial saturation and the half-face fluxes of a pressure solve with the
tables' mobilities.  The rock tables are RockJfunc tables (columns s, krw, kro, J); the flux is
computed once by the oracle, so GPU and oracle runs get identical inputs."""
import numpy as np

MU1, MU2, RHO1, RHO2 = 1e-3, 1e-2, 1000.0, 850.0
SIGMA_COS_THETA = 1e-6   # J scaling that puts the capillary pressure near the 1 Pa pressure drop


def rock_table(smin, smax, n=17, jmax=2.0, ew=2.0, eo=2.0):
    s = np.linspace(smin, smax, n)
    se = (s - smin) / (smax - smin)
    krw = se ** ew
    kro = (1.0 - se) ** eo
    J = jmax * (1.0 - se) ** 2 + 0.05 * (1.0 - se)   # decreasing, 0 at s_max
    return np.column_stack([s, krw, kro, J])


def tables():
    return [rock_table(0.1, 0.9), rock_table(0.15, 0.85, n=11, jmax=3.0, ew=3.0, eo=1.5)]


def table_mobilities(tabs, cell_rock, s):
    """kr/mu per cell by piecewise-linear interpolation with the end values outside the table
    (the reader's fix-ups krw[0] = 0, kro[-1] = 0 hold for these tables already)."""
    m1 = np.empty_like(s)
    m2 = np.empty_like(s)
    for r, t in enumerate(tabs):
        c = cell_rock == r
        m1[c] = np.interp(s[c], t[:, 0], t[:, 1]) / MU1
        m2[c] = np.interp(s[c], t[:, 0], t[:, 2]) / MU2
    return m1, m2


def case(orc, workloads, cart, dims=(8, 6, 4), seed=11, periodic=False):
    rng = np.random.default_rng(seed)
    if periodic:
        g = cart.CartesianGrid(*dims, unique_bids=True)
        nc = g.num_cells
        K = workloads.iso_perm(np.exp(rng.normal(np.log(100 * workloads.MILLIDARCY), 1.0, nc)))
        ybnd = (g.side == 3) | (g.side == 4)
        bct, bcv = workloads.x_dirichlet_bc(g)
        bct[ybnd] = workloads.BC_PERIODIC
        bcv[ybnd] = 0.0
        partner = np.where(ybnd, g.periodic_partner_bids(), 0).astype(np.int32)
        sat_type = np.where(ybnd, workloads.BC_PERIODIC, workloads.BC_DIRICHLET).astype(np.int32)
    else:
        prob = workloads.layered_lognormal(dims=dims, seed=seed)
        g, K, bct, bcv = prob.grid, prob.perm, prob.bc_type, prob.bc_value
        nc = g.num_cells
        partner = None
        sat_type = np.full(g.num_half_faces, workloads.BC_DIRICHLET, np.int32)
    poro = rng.uniform(0.15, 0.3, nc)
    sat_value = np.full(g.num_half_faces, 0.85)
    layer = np.arange(nc) // (dims[0] * dims[1])
    cell_rock = (layer % 2).astype(np.int32)
    tabs = tables()
    sat = rng.uniform(0.3, 0.6, nc)
    # pressure solution at the initial saturation with the tables' mobilities
    m1, m2 = table_mobilities(tabs, cell_rock, sat)
    o = orc.OraclePressure(g, bct, partner)
    o.compute_inner_products(K.ravel())
    assert o.solve(m1 + m2, RHO1 * m1 + RHO2 * m2, bct, bcv, np.zeros(nc), tol=1e-13) == 0
    o.post_process_fluxes()
    _, flux, _ = o.solution()
    return dict(grid=g, K=K, poro=poro, bct=bct, bcv=bcv, partner=partner, sat_type=sat_type, sat_value=sat_value,
                cell_rock=cell_rock, tables=tabs, sat=sat, flux=flux)


def oracle_objects(orc, c):
    """The oracle's transport (with the rock tables) and its zero-gravity pressure handle."""
    rt = orc.RockTables(c["tables"], c["cell_rock"], True, SIGMA_COS_THETA)
    T = orc.OracleTransport(c["grid"], c["K"].ravel(), c["poro"], rt.fluid(MU1, MU2, RHO1, RHO2), c["sat_type"],
                            c["sat_value"], partner_bid=c["partner"])
    P = orc.OraclePressure(c["grid"], c["bct"], c["partner"])
    P.compute_inner_products(c["K"].ravel())
    return T, P
