"""A problem for the tensor-mobility evaluator (MimeticIPAnisoRelpermEvaluator): full SPD
permeability tensors and total mobility tensors lambda_t = a I + b K (which commute with K, so
lambda_t K is symmetric), gravity along z, Dirichlet x-, x+ and no-flow elsewhere."""
import numpy as np


def tensor_problem(workloads, cart, dims=(7, 6, 5), seed=8):
    rng = np.random.default_rng(seed)
    g = cart.CartesianGrid(*dims)
    nc = g.num_cells
    A = rng.normal(size=(nc, 3, 3)) * 0.4
    K = np.eye(3)[None] + np.einsum("cij,ckj->cik", A, A)
    K *= np.exp(rng.normal(0.0, 1.0, nc))[:, None, None]
    a = rng.uniform(0.5, 2.0, nc)[:, None, None]
    b = rng.uniform(0.0, 0.5, nc)[:, None, None] / np.trace(K, axis1=1, axis2=2)[:, None, None]
    lam = a * np.eye(3)[None] + b * K
    rlam = 1000.0 * a * np.eye(3)[None] + 850.0 * b * K
    bct, bcv = workloads.x_dirichlet_bc(g)
    return g, K.reshape(nc, 9), lam.reshape(nc, 9), rlam.reshape(nc, 9), bct, bcv, np.zeros(nc)
