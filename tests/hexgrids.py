"""Non-Cartesian hexahedral grids for the parity tests: an affine (sheared) grid, on which the
mimetic method reproduces linear pressure fields exactly, and a smoothly distorted one."""
import numpy as np

SHEAR = np.array([[1.0, 0.35, 0.1], [0.05, 0.8, 0.25], [0.1, -0.1, 1.2]])


def sheared(cart, dims=(6, 5, 4)):
    return cart.HexGrid(*dims, lambda x: x @ SHEAR.T + np.array([0.2, -0.1, 0.3]))


def distorted(cart, dims=(6, 5, 4), amp=0.06):
    def f(x):
        y = x.copy()
        y[:, 0] += amp * np.sin(2 * np.pi * x[:, 1]) * np.sin(np.pi * x[:, 2])
        y[:, 1] += amp * np.sin(2 * np.pi * x[:, 2]) * np.sin(np.pi * x[:, 0])
        y[:, 2] += amp * np.sin(2 * np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1])
        return y
    return cart.HexGrid(*dims, f)


def linear_field_problem(workloads, g, grad=(1.5, -0.7, 0.4)):
    """Constant full tensor K, unit mobility, Dirichlet p = grad . x on every boundary face."""
    nc = g.num_cells
    rng = np.random.default_rng(6)
    A = rng.normal(size=(3, 3)) * 0.3
    K = np.eye(3) + A @ A.T
    bct = np.where(g.boundary, workloads.BC_DIRICHLET, workloads.BC_NEUMANN).astype(np.int32)
    bcv = np.where(g.boundary, g.fcentroid @ np.asarray(grad), 0.0)
    return workloads.Problem("linear", g, np.tile(K.ravel(), (nc, 1)), np.full(nc, 0.2), bct, bcv, np.zeros(nc),
                             np.zeros(nc), (0, 1.0, 1.0, 0.0, 0.0), totmob=np.ones(nc), mobdens=np.zeros(nc))
