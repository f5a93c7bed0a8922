"""Record how many ILU0-CG iterations the FP64 CPU oracle needs for the full-size
pressure solve of the 200x200x25 layered case (first IMPES step, s = 0) at the
reference's default tolerance (1e-8), at the benchmark's GPU tolerance (1e-11, the
residual reduction that reaches 1e-8 relative flux error) and at 1e-13 (the tolerance of
the full-size oracle solve the benchmark compares against).  The CPU baseline of bench.py
times a bounded sample of that solve (assembly, ILU0 factorisation, a few CG iterations,
recovery) and scales the per-iteration cost by the 1e-11 count.
Run: python tests/golden/make_oracle_iterations.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402
import oracle  # noqa: E402

wl = ge.load_module("workloads")
out = {}
for tol in (1e-8, 1e-11, 1e-13):
    p = wl.layered_lognormal()
    o = oracle.OraclePressure(p.grid, p.bc_type)
    o.compute_inner_products(p.perm.ravel())
    tm, md = p.mobilities()
    t = time.time()
    rc = o.solve(tm, md, p.bc_type, p.bc_value, p.src, tol=tol, dirichlet_guess=True)
    out[f"{tol:g}"] = dict(iterations=o.iterations, reduction=o.reduction, converged=(rc == 0),
                           seconds_here=round(time.time() - t, 1))
    print(tol, out[f"{tol:g}"], flush=True)
json.dump(dict(case="200x200x25 layered log-normal (seed 20261208), s=0, Dirichlet p=1/p=0 on x-/x+",
               solver="oracle ILU0-CG with the Dirichlet-row initial guess", results=out),
          open(os.path.join(HERE, "oracle_layered_1m_ilu0.json"), "w"), indent=2)
