"""Helpers shared by the GPU parity tests: run one problem through the C ABI and through
the FP64 CPU oracle on identical inputs."""
import numpy as np


def gpu_solve(pkg, prob, ltype=1, tol=1e-12, precision=0, post=False, partner=None, **opt):
    s = pkg.PressureSolver()
    s.init(prob.grid, prob.perm.ravel(), (0.0, 0.0, 0.0), prob.bc_type, partner)
    model, mu1, mu2, r1, r2 = prob.fluid
    fl = pkg.Fluid(model, mu1, mu2, r1, r2)
    sat = prob.totmob if model == 0 else prob.sat
    md = prob.mobdens if model == 0 else None
    o = pkg.default_solve_opts(linsolver_type=ltype, residual_tolerance=tol, precision=precision, **opt)
    st = s.solve(fl, sat, prob.bc_type, prob.bc_value, prob.src, mobdens=md, opts=o)
    mm = s.post_process_fluxes() if post else None
    p, v, pi = s.solution()
    return dict(solver=s, stats=st, p=p, v=v, pi=pi, maxmod=mm)


def oracle_solve(orc, prob, tol=1e-12, dirichlet_guess=False, post=False, partner=None):
    o = orc.OraclePressure(prob.grid, prob.bc_type, partner)
    o.compute_inner_products(prob.perm.ravel())
    tm, md = prob.mobilities()
    rc = o.solve(tm, md, prob.bc_type, prob.bc_value, prob.src, tol=tol, dirichlet_guess=dirichlet_guess)
    assert rc == 0, "oracle did not converge"
    mm = o.post_process_fluxes() if post else None
    p, v, pi = o.solution()
    return dict(oracle=o, p=p, v=v, pi=pi, maxmod=mm, iterations=o.iterations)


def rel(a, b):
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def relmax(a, b):
    d = np.abs(b).max()
    return np.abs(a - b).max() / (d if d > 0 else 1.0)
