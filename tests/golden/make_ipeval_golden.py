"""Record the oracle's static inverse inner products for the fixture of the reference's
attic/mimetic/mimetic_ipeval_test.cpp:56-101,134-154: K = diag(10, 1, 0.1) on unit-cube grids of
1, 2x2x2 and 4x4x4 cells.  The reference prints these matrices but stores no output, so the oracle's
values (column-major per cell, as Binv_) are the golden copy the CPU and GPU tests compare with.
Run: python tests/golden/make_ipeval_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402
import oracle  # noqa: E402

cart = ge.load_module("cartesian")
out = {"K": [10.0, 1.0, 0.1], "grids": {}}
for n in (1, 2, 4):
    g = cart.CartesianGrid(n, n, n, 1.0 / n, 1.0 / n, 1.0 / n)
    nc = g.num_cells
    K = np.zeros((nc, 9))
    K[:, 0], K[:, 4], K[:, 8] = 10.0, 1.0, 0.1
    o = oracle.OraclePressure(g, np.full(g.num_half_faces, oracle.BC_NEUMANN, np.int32))
    o.compute_inner_products(K.ravel())
    B, _ = o.inner_products()
    B = B.reshape(nc, 36)
    out["grids"][str(n)] = {
        "cells": nc,
        "first_cell": B[0].tolist(),
        "last_cell": B[-1].tolist(),
        "cell_norms": np.linalg.norm(B, axis=1).tolist(),
    }
with open(os.path.join(HERE, "ipeval_binv.json"), "w") as f:
    json.dump(out, f, indent=1)
print("written", {k: v["cells"] for k, v in out["grids"].items()})
