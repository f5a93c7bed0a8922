"""porsol_transport_cfl_noalloc: the viscous CFL step for callers that cannot allocate device
memory (their device memory belongs to their own pool allocator).  It must agree with the CFL
step that the allocating transport entry point (porsol_transport_solve) computes with the same
kernel arithmetic, on two calls in a row (the fixed scratch array keeps the previous call's
contents), and report a zero step as findCFLtimeVelocity's zero-step error
(CflCalculator.hpp:75-77).  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_cfl_matches_transport_entry_point(pkg, gpulib, orc, workloads):
    import torch
    from parity import gpu_solve
    prob = workloads.layered_lognormal(dims=(12, 9, 5), seed=17)
    flux = gpu_solve(pkg, prob, ltype=1, tol=1e-12, post=True)["v"]
    g = prob.grid
    _, mu1, mu2, r1, r2 = prob.fluid
    opts = pkg.default_transport_opts(method_gravity=0, method_capillary=0)
    T = pkg.TransportSolver()
    T.init(g, prob.perm.ravel(), prob.poro, pkg.Fluid(pkg.FLUID_COREY2, mu1, mu2, r1, r2), prob.sat_type,
           prob.sat_value, opts=opts)
    _, st = T.solve(prob.sat, 1e-30, flux)            # a tiny step: only the CFL bound matters
    ref = st.cfl_dt / opts.courant_number            # velocity bound of the allocating path
    fac = orc.cfl_factors(orc.Fluid(mu1, mu2, r1, r2))[0]
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in
         dict(fp=g.facepos.astype(np.int32), q=flux, vol=g.volume, phi=prob.poro).items()}
    torch.cuda.synchronize()
    for call in range(2):
        dt = C.c_double(-1.0)
        rc = pkg.lib().porsol_transport_cfl_noalloc(g.num_cells, d["fp"].data_ptr(), d["q"].data_ptr(),
                                                    d["vol"].data_ptr(), d["phi"].data_ptr(), fac, C.byref(dt),
                                                    None)
        assert rc == 0, f"call {call}: status {rc}"
        assert abs(dt.value - ref) <= 1e-12 * ref, (call, dt.value, ref)
    # sizes beyond the fixed scratch are rejected before any work
    dt = C.c_double(0.0)
    rc = pkg.lib().porsol_transport_cfl_noalloc(4194305, d["fp"].data_ptr(), d["q"].data_ptr(),
                                                d["vol"].data_ptr(), d["phi"].data_ptr(), fac, C.byref(dt), None)
    assert rc == 2   # PORSOL_ERR_BAD_ARG

    # a cell with zero porosity and non-zero flux has a zero step: PORSOL_ERR_CFL with *dt = 0,
    # after a call that left a non-zero result in the shared scratch array
    phi0 = prob.poro.copy()
    fp = g.facepos
    busy = int(np.argmax([np.abs(flux[fp[c]:fp[c + 1]]).sum() for c in range(g.num_cells)]))
    phi0[busy] = 0.0
    d_phi0 = torch.from_numpy(phi0).to(dev)
    torch.cuda.synchronize()
    dt = C.c_double(-1.0)
    rc = pkg.lib().porsol_transport_cfl_noalloc(g.num_cells, d["fp"].data_ptr(), d["q"].data_ptr(),
                                                d["vol"].data_ptr(), d_phi0.data_ptr(), fac, C.byref(dt), None)
    assert rc == 9, f"status {rc}"   # PORSOL_ERR_CFL
    assert dt.value == 0.0
    # and the next ordinary call is exact again
    dt = C.c_double(-1.0)
    rc = pkg.lib().porsol_transport_cfl_noalloc(g.num_cells, d["fp"].data_ptr(), d["q"].data_ptr(),
                                                d["vol"].data_ptr(), d["phi"].data_ptr(), fac, C.byref(dt), None)
    assert rc == 0 and abs(dt.value - ref) <= 1e-12 * ref
