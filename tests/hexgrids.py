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


class FlatGrid:
    """Flattened grid built cell by cell: list of (volume, centroid, [faces]) with faces
    (neighbour, bid, area, centroid, unit normal).  Exposes the attributes the solvers read."""

    def __init__(self, cells):
        self.num_cells = len(cells)
        fp = [0]
        nb, bid, area, fc, fn, vol, cc = [], [], [], [], [], [], []
        for v, c, faces in cells:
            vol.append(v)
            cc.append(c)
            for (n, b, a, x, nrm) in faces:
                nb.append(n)
                bid.append(b)
                area.append(a)
                fc.append(x)
                fn.append(nrm)
            fp.append(fp[-1] + len(faces))
        self.facepos = np.array(fp, np.int32)
        self.neighbour = np.array(nb, np.int32)
        self.bid = np.array(bid, np.int32)
        self.area = np.array(area, float)
        self.fcentroid = np.array(fc, float)
        self.fnormal = np.array(fn, float)
        self.volume = np.array(vol, float)
        self.ccentroid = np.array(cc, float)
        self.side = np.where(self.neighbour < 0, self.bid, 0).astype(np.int32)

    @property
    def num_half_faces(self):
        return int(self.facepos[-1])

    @property
    def boundary(self):
        return self.neighbour < 0

    def arrays(self):
        return dict(num_cells=self.num_cells, facepos=self.facepos, neighbour=self.neighbour, bid=self.bid,
                    area=self.area, fcentroid=self.fcentroid, fnormal=self.fnormal, volume=self.volume,
                    ccentroid=self.ccentroid)


def refined_top(nx=4, ny=3, nzc=2, nzf=2):
    """Unit-size coarse cells (nx x ny x nzc) under a layer block refined 2 x 2 in x and y
    (2nx x 2ny x nzf cells of size 1/2 x 1/2 x 1).  Each top coarse cell meets four fine cells
    through four quarter faces, so it has 9 faces (the up-to-12-face kernels); face pairs match
    exactly.  Boundary ids 1..6 by side (x-, x+, y-, y+, z-, z+)."""
    ncoarse = nx * ny * nzc
    def cidx(i, j, k):
        return i + nx * (j + ny * k)
    def fidx(i, j, k):
        return ncoarse + i + 2 * nx * (j + 2 * ny * k)
    cells = []
    ex = [np.array(v, float) for v in ((1, 0, 0), (0, 1, 0), (0, 0, 1))]
    for k in range(nzc):
        for j in range(ny):
            for i in range(nx):
                c = np.array([i + 0.5, j + 0.5, k + 0.5])
                faces = []
                for ax, (lo, hi, dims) in enumerate(((i, i, nx), (j, j, ny), (k, k, nzc))):
                    for sgn in (-1, 1):
                        if ax == 2 and sgn == 1 and k == nzc - 1:
                            for dj in (0, 1):
                                for di in (0, 1):
                                    x = np.array([i + 0.25 + 0.5 * di, j + 0.25 + 0.5 * dj, k + 1.0])
                                    faces.append((fidx(2 * i + di, 2 * j + dj, 0), 0, 0.25, x, ex[2]))
                            continue
                        idx = [i, j, k]
                        idx[ax] += sgn
                        inside = 0 <= idx[ax] < dims
                        x = c + 0.5 * sgn * ex[ax]
                        n = cidx(*idx) if inside else -1
                        faces.append((n, 0 if inside else 2 * ax + (1 if sgn > 0 else 0) + 1, 1.0, x, sgn * ex[ax]))
                cells.append((1.0, c, faces))
    for k in range(nzf):
        for j in range(2 * ny):
            for i in range(2 * nx):
                c = np.array([0.25 + 0.5 * i, 0.25 + 0.5 * j, nzc + k + 0.5])
                faces = []
                h = (0.5, 0.5, 1.0)
                dims = (2 * nx, 2 * ny, nzf)
                for ax in range(3):
                    for sgn in (-1, 1):
                        idx = [i, j, k]
                        idx[ax] += sgn
                        x = c + 0.5 * h[ax] * sgn * ex[ax]
                        a = h[(ax + 1) % 3] * h[(ax + 2) % 3]
                        if ax == 2 and sgn == -1 and k == 0:
                            faces.append((cidx(i // 2, j // 2, nzc - 1), 0, a, x, -ex[2]))
                            continue
                        inside = 0 <= idx[ax] < dims[ax]
                        n = fidx(*idx) if inside else -1
                        faces.append((n, 0 if inside else 2 * ax + (1 if sgn > 0 else 0) + 1, a, x, sgn * ex[ax]))
                cells.append((0.25, c, faces))
    return FlatGrid(cells)
