"""Helpers for the periodic-upscaling tests."""
import numpy as np


def oracle_keff(orc, grid, K9, tol=1e-13):
    return orc.upscale_periodic(grid, K9, tol)[0]


def layered_perm(cart, n, kz_values):
    """n x n x len(kz_values) unit cube, isotropic k varying with the z layer only."""
    g = cart.CartesianGrid(n, n, len(kz_values), unique_bids=True)
    k = np.repeat(np.asarray(kz_values, float), n * n)
    K = np.zeros((g.num_cells, 9))
    K[:, 0] = K[:, 4] = K[:, 8] = k
    return g, K
