"""Helpers for the adjoint tests: a small problem that exercises every term of the adjoint
(full or diagonal tensors, cell-wise mobility, Dirichlet + Neumann faces, sources, pressure
and interior/boundary flux weights) and finite differences of the objective."""
import numpy as np


def adjoint_problem(workloads, cart, dims=(6, 5, 4), diagonal=False, seed=3):
    rng = np.random.default_rng(seed)
    g = cart.CartesianGrid(*dims)
    nc = g.num_cells
    k = np.exp(rng.normal(0.0, 1.0, nc))
    if diagonal:
        K = workloads.diag_perm(k, k * np.exp(rng.normal(0, 1, nc)), 0.3 * k)
    else:
        A = rng.normal(size=(nc, 3, 3)) * 0.3
        K = ((np.eye(3)[None] + np.einsum("cij,ckj->cik", A, A)) * k[:, None, None]).reshape(nc, 9)
    bct, bcv = workloads.x_dirichlet_bc(g)
    bcv[g.side == 3] = 0.05                      # Neumann outflux on y-
    tm = np.exp(rng.normal(0.0, 0.5, nc))
    prob = workloads.Problem("adjoint", g, K, np.full(nc, 0.2), bct, bcv, rng.normal(0, 0.01, nc),
                             np.zeros(nc), (0, 1.0, 1.0, 0.0, 0.0), totmob=tm, mobdens=np.zeros(nc))
    w = np.zeros(nc)
    w[rng.choice(nc, max(2, nc // 12), replace=False)] = 1.0
    target = rng.normal(0.5, 0.1, nc)
    u = np.where(g.side == 2, 1.0, 0.0) + np.where(g.neighbour >= 0, rng.normal(0, 0.1, g.num_half_faces), 0.0)
    return prob, w, target, u


def objective(p, v, w, target, u):
    return float(np.sum(w * (p - target) ** 2) + np.sum(u * v))


def perturbed(K, c, axis, h):
    """Copy of K with ln k of cell c moved by h: the whole tensor (axis None) or one axis."""
    Kp = K.copy()
    if axis is None:
        Kp[c] *= np.exp(h)
    else:
        Kp[c, 4 * axis] *= np.exp(h)
    return Kp


def central_differences(J_of, K, cells, axes, h=1e-6):
    out = []
    for c in cells:
        for a in axes:
            out.append((J_of(perturbed(K, c, a, h)) - J_of(perturbed(K, c, a, -h))) / (2 * h))
    return np.array(out)
