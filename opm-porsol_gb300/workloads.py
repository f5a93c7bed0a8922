"""Seeded synthetic workloads for the tests and the benchmark.

There is no public dataset for this path; every input is generated here from a
documented seed (20261203 + k, numpy PCG64).  Units are SI as in the reference
(Opm::unit): permeability in m^2 (1 mD = 9.869233e-16 m^2), viscosity in Pa s,
pressure in Pa (the workloads prescribe p = 1 and p = 0).

  unit_cube_lognormal    10x10x10 unit cube, isotropic ln k ~ N(ln 100 mD, 1) i.i.d.,
                         total mobility 1, Dirichlet p=1 (x-) / p=0 (x+), no-flow elsewhere,
                         ILU0-CG 1e-10 (seed + 1).
  anisotropic_corey      100x100x50, kx=ky log-normal sigma=2 Gaussian-correlated (5 cells),
                         kz = 0.1 kx, Corey-2 mobilities with viscosity ratio 5, s ~ U[0,1]
                         (seed + 2).
  periodic_subgrids      512 periodic unit cubes n^3, n ~ U{8..32}, full log-normal tensors
                         sigma=1.5 with random principal axes (seed + 3).
  correlated_lognormal   64x64x32, isotropic log-normal sigma=1 correlated over 4 cells
                         (seed + 4); pressure_mismatch_objective: squared pressure mismatches
                         at 50 cells + outflux through x+.
  layered_lognormal      200x200x25, 25 layers, layer mean ~ N(ln 100 mD, 1),
                         ln k ~ N(mean, 2^2) i.i.d. within a layer, Corey-2 with viscosity
                         ratio 10, initial s = 0, water (s = 1) enters through x- (seed + 5).
  layered_capillary      the layered_lognormal grid and permeability with two RockJfunc
                         rocks by layer parity (s in [0.1, 0.9] / [0.15, 0.85], power-law
                         relperms, decreasing J), porosity ~ U[0.15, 0.3], s ~ U[0.3, 0.6],
                         J scaling sigma cos(theta) = 1e-6 (seed + 6).
"""
from __future__ import annotations

import os
import sys
from dataclasses import dataclass, field

import numpy as np

_here = os.path.dirname(os.path.abspath(__file__))
if _here not in sys.path:
    sys.path.insert(0, _here)
from cartesian import CartesianGrid, UnionGrid  # noqa: E402

MILLIDARCY = 9.869233e-16
SEED0 = 20261203
BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2


@dataclass
class Problem:
    name: str
    grid: CartesianGrid
    perm: np.ndarray            # (nc, 9) row-major tensors
    poro: np.ndarray
    bc_type: np.ndarray         # FlowBC type per half-face
    bc_value: np.ndarray
    src: np.ndarray
    sat: np.ndarray
    fluid: tuple                # (model, mu1, mu2, rho1, rho2); model 0 = cell-wise, 1 = Corey-2
    totmob: np.ndarray = None   # cell-wise model only
    mobdens: np.ndarray = None
    sat_type: np.ndarray = None
    sat_value: np.ndarray = None
    extra: dict = field(default_factory=dict)

    def mobilities(self):
        """Total mobility and sum(rho_i mob_i) per cell, as the fluid model defines them."""
        model, mu1, mu2, r1, r2 = self.fluid
        if model == 0:
            return self.totmob, (self.mobdens if self.mobdens is not None else np.zeros_like(self.totmob))
        s = self.sat
        m1 = (s * s) / mu1
        m2 = ((1.0 - s) * (1.0 - s)) / mu2
        return m1 + m2, r1 * m1 + r2 * m2


def x_dirichlet_bc(grid: CartesianGrid, p_in=1.0, p_out=0.0):
    """Dirichlet p_in on x- (side 1), p_out on x+ (side 2), no-flow Neumann elsewhere."""
    bct = np.full(grid.num_half_faces, BC_NEUMANN, np.int32)
    bcv = np.zeros(grid.num_half_faces)
    bct[grid.side == 1] = BC_DIRICHLET
    bct[grid.side == 2] = BC_DIRICHLET
    bcv[grid.side == 1] = p_in
    bcv[grid.side == 2] = p_out
    return bct, bcv


def iso_perm(k):
    K = np.zeros((len(k), 9))
    K[:, 0] = K[:, 4] = K[:, 8] = k
    return K


def diag_perm(kx, ky, kz):
    K = np.zeros((len(kx), 9))
    K[:, 0], K[:, 4], K[:, 8] = kx, ky, kz
    return K


def correlated_normal(rng, dims, corr_cells, sigma=1.0):
    """Zero-mean Gaussian field with a Gaussian kernel of std `corr_cells`, rescaled to `sigma`."""
    from scipy.ndimage import gaussian_filter
    nx, ny, nz = dims
    z = rng.standard_normal((nz, ny, nx))
    f = gaussian_filter(z, sigma=corr_cells, mode="wrap")
    f = (f - f.mean()) / f.std() * sigma
    return f.ravel()   # x fastest, matching the grid's cell order


def unit_cube_lognormal(n=10, seed=None):
    rng = np.random.default_rng(SEED0 + 1 if seed is None else seed)
    g = CartesianGrid(n, n, n)
    nc = g.num_cells
    k = np.exp(rng.normal(np.log(100 * MILLIDARCY), 1.0, nc))
    bct, bcv = x_dirichlet_bc(g)
    return Problem("unit_cube_lognormal", g, iso_perm(k), np.full(nc, 0.2), bct, bcv, np.zeros(nc), np.zeros(nc),
                   (0, 1.0, 1.0, 0.0, 0.0), totmob=np.ones(nc), mobdens=np.zeros(nc))


def anisotropic_corey(dims=(100, 100, 50), seed=None, corr=5.0):
    rng = np.random.default_rng(SEED0 + 2 if seed is None else seed)
    g = CartesianGrid(*dims)
    nc = g.num_cells
    lk = np.log(100 * MILLIDARCY) + correlated_normal(rng, dims, corr, 2.0)
    kx = np.exp(lk)
    sat = rng.uniform(0.0, 1.0, nc)
    bct, bcv = x_dirichlet_bc(g)
    return Problem("anisotropic_corey", g, diag_perm(kx, kx, 0.1 * kx), np.full(nc, 0.2), bct, bcv, np.zeros(nc), sat,
                   (1, 1e-3, 5e-3, 1000.0, 850.0))


def random_rotations(rng, n):
    """Uniformly distributed rotation matrices (QR of Gaussian matrices, sign-fixed)."""
    A = rng.standard_normal((n, 3, 3))
    Q, R = np.linalg.qr(A)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    det = np.linalg.det(Q)
    Q[det < 0, :, 0] *= -1.0
    return Q


def periodic_subgrids(num=512, nmin=8, nmax=32, seed=None, sigma=1.5, sides=None):
    """Batched periodic upscaling: `num` unit-cube sub-grids of n^3 cells, n ~ U{nmin..nmax},
    full SPD tensors K = R diag(exp(g)) R^T per cell, g ~ N(ln 100 mD, sigma^2), R uniform.
    `sides` (a list of n) replaces the drawn sides (num is then its length)."""
    rng = np.random.default_rng(SEED0 + 3 if seed is None else seed)
    sizes = rng.integers(nmin, nmax + 1, size=num)
    if sides is not None:
        sizes = np.asarray(sides, dtype=sizes.dtype)
    grids = [CartesianGrid(int(n), int(n), int(n), unique_bids=True) for n in sizes]
    union = UnionGrid(grids)
    nc = union.num_cells
    R = random_rotations(rng, nc)
    lam = np.exp(rng.normal(np.log(100 * MILLIDARCY), sigma, (nc, 3)))
    K = np.einsum("cij,cj,ckj->cik", R, lam, R)
    return union, sizes, K.reshape(nc, 9)


def correlated_lognormal(dims=(64, 64, 32), seed=None, corr=4.0):
    rng = np.random.default_rng(SEED0 + 4 if seed is None else seed)
    g = CartesianGrid(*dims)
    nc = g.num_cells
    lk = np.log(100 * MILLIDARCY) + correlated_normal(rng, dims, corr, 1.0)
    bct, bcv = x_dirichlet_bc(g)
    return Problem("correlated_lognormal", g, iso_perm(np.exp(lk)), np.full(nc, 0.2), bct, bcv, np.zeros(nc), np.zeros(nc),
                   (0, 1.0, 1.0, 0.0, 0.0), totmob=np.ones(nc), mobdens=np.zeros(nc))


def pressure_mismatch_objective(problem, seed=None, n_obs=50, n_fd=20):
    """Objective of the adjoint workload on a correlated_lognormal grid: pressure mismatch at `n_obs`
    seeded cells against targets p* ~ N(0.5, 0.1^2), plus the total outflux through x+ (side 2).
    Returns (cell_weight, cell_target, hf_weight, fd_cells): fd_cells are the `n_fd` seeded cells
    at which finite differences check the gradient."""
    rng = np.random.default_rng(SEED0 + 40 if seed is None else seed)
    g = problem.grid
    nc = g.num_cells
    obs = rng.choice(nc, n_obs, replace=False)
    w = np.zeros(nc)
    w[obs] = 1.0
    target = np.zeros(nc)
    target[obs] = rng.normal(0.5, 0.1, n_obs)
    u = np.where(g.side == 2, 1.0, 0.0)
    fd_cells = rng.choice(nc, n_fd, replace=False)
    return w, target, u, fd_cells


def layered_lognormal(dims=(200, 200, 25), seed=None, sat=None):
    rng = np.random.default_rng(SEED0 + 5 if seed is None else seed)
    nx, ny, nz = dims
    g = CartesianGrid(*dims)
    nc = g.num_cells
    means = rng.normal(np.log(100 * MILLIDARCY), 1.0, nz)
    layer = np.repeat(np.arange(nz), nx * ny)
    lk = rng.normal(means[layer], 2.0)
    bct, bcv = x_dirichlet_bc(g)
    s = np.zeros(nc) if sat is None else sat
    st = np.full(g.num_half_faces, BC_DIRICHLET, np.int32)   # SatBC default: Dirichlet s = 1
    sv = np.ones(g.num_half_faces)
    return Problem("layered_lognormal", g, iso_perm(np.exp(lk)), np.full(nc, 0.2), bct, bcv, np.zeros(nc), s,
                   (1, 1e-3, 1e-2, 1000.0, 850.0), sat_type=st, sat_value=sv)


def known_answer(n):
    """examples/known_answer_test.cpp: u = sin(2 pi x) cos(2 pi y) z on the unit cube,
    source -Lap(u)|c|, Dirichlet u on every boundary face, K = 1, unit mobility."""
    pi = 3.14159265358979323846264338327950288
    g = CartesianGrid(n, n, n)
    nc = g.num_cells

    def u(x):
        return np.sin(2 * pi * x[:, 0]) * np.cos(2 * pi * x[:, 1]) * x[:, 2]

    def lap(x):
        return -2 * 2 * pi * 2 * pi * np.sin(2 * pi * x[:, 0]) * np.cos(2 * pi * x[:, 1]) * x[:, 2]

    bct = np.where(g.boundary, BC_DIRICHLET, BC_NEUMANN).astype(np.int32)
    bcv = np.where(g.boundary, u(g.fcentroid), 0.0)
    src = -lap(g.ccentroid) * g.volume
    p = Problem(f"kat{n}", g, iso_perm(np.ones(nc)), np.ones(nc), bct, bcv, src, np.zeros(nc),
                (0, 1.0, 1.0, 0.0, 0.0), totmob=np.ones(nc), mobdens=np.zeros(nc))
    p.extra["u"] = u
    return p


def error_norms(problem, pressure):
    """Volume-weighted L1/L2 error densities and L-inf error of the cell pressure
    (examples/known_answer_test.cpp:214-238)."""
    g = problem.grid
    diff = problem.extra["u"](g.ccentroid) - pressure
    v = g.volume
    totv = v.sum()
    return (np.sum(np.abs(diff * v)) / totv, np.sqrt(np.sum(diff * diff * v)) / totv, np.abs(diff).max())


def rock_table(smin, smax, n=17, jmax=2.0, ew=2.0, eo=2.0):
    """A RockJfunc table (columns s, krw, kro, J): power-law relative permeabilities in the
    normalised saturation and a decreasing J-function that reaches 0 at s_max."""
    s = np.linspace(smin, smax, n)
    se = (s - smin) / (smax - smin)
    J = jmax * (1.0 - se) ** 2 + 0.05 * (1.0 - se)
    return np.column_stack([s, se ** ew, (1.0 - se) ** eo, J])


def layered_capillary(dims=(200, 200, 25), seed=None):
    """The ImplicitCapillarity workload: layered_lognormal's grid, permeability and x-Dirichlet
    pressure BCs with two rocks (by layer parity) and a heterogeneous initial saturation."""
    base = layered_lognormal(dims=dims, seed=SEED0 + 5 if seed is None else seed)
    rng = np.random.default_rng(SEED0 + 6 if seed is None else seed + 1)
    nc = base.grid.num_cells
    nx, ny, _ = dims
    tables = [rock_table(0.1, 0.9), rock_table(0.15, 0.85, n=11, jmax=3.0, ew=3.0, eo=1.5)]
    cell_rock = ((np.arange(nc) // (nx * ny)) % 2).astype(np.int32)
    base.poro = rng.uniform(0.15, 0.3, nc)
    base.sat = rng.uniform(0.3, 0.6, nc)
    base.sat_value = np.full(base.grid.num_half_faces, 0.85)
    base.name = "layered_capillary"
    base.extra.update(tables=tables, cell_rock=cell_rock, sigma_cos_theta=1e-6)
    return base


def table_mobilities(tables, cell_rock, s, mu1, mu2):
    """kr / mu per cell from the rock tables (piecewise linear, end values outside)."""
    m1 = np.empty_like(s)
    m2 = np.empty_like(s)
    for r, t in enumerate(tables):
        c = cell_rock == r
        m1[c] = np.interp(s[c], t[:, 0], t[:, 1]) / mu1
        m2[c] = np.interp(s[c], t[:, 0], t[:, 2]) / mu2
    return m1, m2
