"""Flattened Cartesian hexahedral grids in the layout the C-ABI consumes.

The reference walks a DUNE grid through ``GridInterfaceEuler`` (cells in
iteration order, each cell's intersections in local order; area, centroid,
unit outward normal, boundary flag, boundary id, neighbour index:
opm/porsol/common/GridInterfaceEuler.hpp:126-214, 346-360).  For a YaspGrid
the iteration order is lexicographic with x fastest and the local face order
is x-, x+, y-, y+, z-, z+ with boundary ids 1..6 on the six sides
(opm/porsol/common/setupBoundaryConditions.hpp:70-71, 89-90).  This module
produces exactly those arrays with numpy, so tests and benchmarks can feed the
same grid to the GPU library and to the CPU oracle.
"""
from __future__ import annotations

import numpy as np

# canonical side of each local face: 0=x-, 1=x+, 2=y-, 3=y+, 4=z-, 5=z+
_AXIS = np.array([0, 0, 1, 1, 2, 2])
_SIGN = np.array([-1, 1, -1, 1, -1, 1])


class CartesianGrid:
    """Flattened unit-stride Cartesian grid (nx, ny, nz cells of size dx, dy, dz).

    Attributes mirror ``porsol_grid`` in include/porsol_gpu.h:
    ``facepos`` (nc+1), ``neighbour``/``bid`` (nhf), ``area`` (nhf),
    ``fcentroid``/``fnormal`` (nhf, 3), ``volume`` (nc), ``ccentroid`` (nc, 3).
    With ``unique_bids`` every boundary face gets its own boundary id
    (1..num_boundary_faces, in half-face order), as CpGrid does after
    ``setUniqueBoundaryIds(true)``; ``side`` keeps the canonical side 1..6.
    """

    def __init__(self, nx: int, ny: int, nz: int, dx: float = None, dy: float = None,
                 dz: float = None, unique_bids: bool = False):
        self.dims = (int(nx), int(ny), int(nz))
        dx = 1.0 / nx if dx is None else float(dx)
        dy = 1.0 / ny if dy is None else float(dy)
        dz = 1.0 / nz if dz is None else float(dz)
        self.h = (dx, dy, dz)
        nc = nx * ny * nz
        self.num_cells = nc
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        i = i.ravel().astype(np.int64)
        j = j.ravel().astype(np.int64)
        k = k.ravel().astype(np.int64)
        ijk = np.stack([i, j, k], axis=1)
        n_per = np.array([nx, ny, nz])
        stride = np.array([1, nx, nx * ny])
        h = np.array([dx, dy, dz])
        self.ccentroid = (ijk + 0.5) * h
        self.volume = np.full(nc, dx * dy * dz)
        self.facepos = (np.arange(nc + 1, dtype=np.int32) * 6).astype(np.int32)
        nb = np.empty((nc, 6), dtype=np.int64)
        side = np.zeros((nc, 6), dtype=np.int32)
        fcent = np.repeat(self.ccentroid[:, None, :], 6, axis=1).copy()
        fnormal = np.zeros((nc, 6, 3))
        area = np.empty((nc, 6))
        areas = np.array([dy * dz, dx * dz, dx * dy])
        cidx = np.arange(nc, dtype=np.int64)
        for lf in range(6):
            ax, sg = _AXIS[lf], _SIGN[lf]
            coord = ijk[:, ax]
            inside = (coord > 0) if sg < 0 else (coord < n_per[ax] - 1)
            nb[:, lf] = np.where(inside, cidx + sg * stride[ax], -1)
            side[:, lf] = np.where(inside, 0, lf + 1)
            fcent[:, lf, ax] += sg * 0.5 * h[ax]
            fnormal[:, lf, ax] = sg
            area[:, lf] = areas[ax]
        self.neighbour = nb.ravel().astype(np.int32)
        self.side = side.ravel()
        if unique_bids:
            bid = np.zeros(nc * 6, dtype=np.int32)
            bmask = self.side > 0
            bid[bmask] = np.arange(1, int(bmask.sum()) + 1, dtype=np.int32)
            self.bid = bid
        else:
            self.bid = self.side.astype(np.int32).copy()
        self.area = area.ravel()
        self.fcentroid = fcent.reshape(-1, 3)
        self.fnormal = fnormal.reshape(-1, 3)
        self.unique_bids = unique_bids

    @property
    def num_half_faces(self) -> int:
        return int(self.facepos[-1])

    @property
    def boundary(self) -> np.ndarray:
        return self.neighbour < 0

    def cell_of_half_face(self) -> np.ndarray:
        return np.repeat(np.arange(self.num_cells, dtype=np.int32), np.diff(self.facepos))

    def periodic_partner_bids(self) -> np.ndarray:
        """Partner boundary id of every boundary half-face for full periodicity.

        Matches each face on side 2d-1 (low) with the face on side 2d (high) at
        the same transverse position, as findPeriodicPartners does geometrically
        (opm/porsol/common/BoundaryPeriodicity.hpp:86-180).  Requires unique
        boundary ids.  Interior half-faces get 0.
        """
        if not self.unique_bids:
            raise ValueError("periodic pairing needs unique boundary ids")
        nx, ny, nz = self.dims
        nc = self.num_cells
        partner = np.zeros(nc * 6, dtype=np.int32)
        stride = np.array([1, nx, nx * ny])
        n_per = np.array([nx, ny, nz])
        cidx = np.arange(nc, dtype=np.int64)
        ijk = np.stack([cidx % nx, (cidx // nx) % ny, cidx // (nx * ny)], axis=1)
        for ax in range(3):
            lo_cells = cidx[ijk[:, ax] == 0]
            hi_cells = lo_cells + (n_per[ax] - 1) * stride[ax]
            lo_hf = lo_cells * 6 + 2 * ax
            hi_hf = hi_cells * 6 + 2 * ax + 1
            partner[lo_hf] = self.bid[hi_hf]
            partner[hi_hf] = self.bid[lo_hf]
        return partner

    def arrays(self):
        """The eight arrays of the flattened grid interface, C-contiguous."""
        return dict(
            num_cells=self.num_cells,
            facepos=np.ascontiguousarray(self.facepos, dtype=np.int32),
            neighbour=np.ascontiguousarray(self.neighbour, dtype=np.int32),
            bid=np.ascontiguousarray(self.bid, dtype=np.int32),
            area=np.ascontiguousarray(self.area, dtype=np.float64),
            fcentroid=np.ascontiguousarray(self.fcentroid, dtype=np.float64),
            fnormal=np.ascontiguousarray(self.fnormal, dtype=np.float64),
            volume=np.ascontiguousarray(self.volume, dtype=np.float64),
            ccentroid=np.ascontiguousarray(self.ccentroid, dtype=np.float64),
        )


class UnionGrid:
    """Disjoint union of Cartesian sub-grids with unique boundary ids (batched upscaling).

    Sub-grid g owns cells [cellpos[g], cellpos[g+1]); neighbour indices and boundary ids are
    offset so that the union is one flattened grid; ``partner`` holds each boundary face's
    periodic partner id and ``side`` its canonical side (1..6).
    """

    def __init__(self, grids):
        self.grids = list(grids)
        cellpos = [0]
        nb, bid, side, partner, area, fc, fn, vol, cc, fp = [], [], [], [], [], [], [], [], [], [0]
        boff = 0
        for g in self.grids:
            if not g.unique_bids:
                raise ValueError("sub-grids need unique boundary ids")
            off = cellpos[-1]
            n = g.neighbour.astype(np.int64)
            nb.append(np.where(n >= 0, n + off, -1))
            b = g.bid.astype(np.int64)
            bid.append(np.where(b > 0, b + boff, 0))
            p = g.periodic_partner_bids().astype(np.int64)
            partner.append(np.where(p > 0, p + boff, 0))
            side.append(g.side)
            area.append(g.area)
            fc.append(g.fcentroid)
            fn.append(g.fnormal)
            vol.append(g.volume)
            cc.append(g.ccentroid)
            last = int(fp[-1][-1]) if isinstance(fp[-1], np.ndarray) else int(fp[-1])
            fp.append(g.facepos[1:].astype(np.int64) + last)
            boff += int(b.max())
            cellpos.append(off + g.num_cells)
        self.cellpos = np.array(cellpos, dtype=np.int32)
        self.num_cells = int(self.cellpos[-1])
        self.facepos = np.concatenate([np.zeros(1, np.int64)] + [np.asarray(x, np.int64) for x in fp[1:]]).astype(np.int32)
        self.neighbour = np.concatenate(nb).astype(np.int32)
        self.bid = np.concatenate(bid).astype(np.int32)
        self.partner = np.concatenate(partner).astype(np.int32)
        self.side = np.concatenate(side).astype(np.int32)
        self.area = np.concatenate(area)
        self.fcentroid = np.concatenate(fc)
        self.fnormal = np.concatenate(fn)
        self.volume = np.concatenate(vol)
        self.ccentroid = np.concatenate(cc)
        self.unique_bids = True

    @property
    def num_half_faces(self):
        return int(self.facepos[-1])

    @property
    def boundary(self):
        return self.neighbour < 0

    def arrays(self):
        return dict(
            num_cells=self.num_cells,
            facepos=np.ascontiguousarray(self.facepos, dtype=np.int32),
            neighbour=np.ascontiguousarray(self.neighbour, dtype=np.int32),
            bid=np.ascontiguousarray(self.bid, dtype=np.int32),
            area=np.ascontiguousarray(self.area, dtype=np.float64),
            fcentroid=np.ascontiguousarray(self.fcentroid, dtype=np.float64),
            fnormal=np.ascontiguousarray(self.fnormal, dtype=np.float64),
            volume=np.ascontiguousarray(self.volume, dtype=np.float64),
            ccentroid=np.ascontiguousarray(self.ccentroid, dtype=np.float64),
        )


class HexGrid(CartesianGrid):
    """Logically Cartesian hexahedral grid with vertices moved by `mapping` (a function of an
    (m, 3) array of reference points in the unit cube, returning (m, 3)).  Same cell/face order,
    neighbours and boundary ids as CartesianGrid; the geometry is computed from the 8 corners:
    each quadrilateral face is split into four triangles around its vertex average (area-weighted
    normal = sum of triangle normals, centroid = area-weighted triangle centroids), and the cell
    volume and centroid follow from the tetrahedra formed by those triangles and the cell's
    vertex average.  For an affine mapping the faces are planar parallelograms and the geometry
    is exact."""

    # local vertices (di, dj, dk) of each local face, ordered so the normal points outwards
    _FACE_VERTS = [
        [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)],   # x-
        [(1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)],   # x+
        [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)],   # y-
        [(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)],   # y+
        [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)],   # z-
        [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)],   # z+
    ]

    def __init__(self, nx, ny, nz, mapping, unique_bids=False):
        super().__init__(nx, ny, nz, unique_bids=unique_bids)
        k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        ref = np.stack([i.ravel() / nx, j.ravel() / ny, k.ravel() / nz], axis=1)
        V = np.asarray(mapping(ref), dtype=np.float64).reshape(nz + 1, ny + 1, nx + 1, 3)
        nc = self.num_cells
        kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
        corners = {}
        for dk in (0, 1):
            for dj in (0, 1):
                for di in (0, 1):
                    corners[(di, dj, dk)] = V[kk + dk, jj + dj, ii + di]
        xc0 = sum(corners.values()) / 8.0
        area = np.empty((nc, 6))
        fcent = np.empty((nc, 6, 3))
        fnorm = np.empty((nc, 6, 3))
        vol = np.zeros(nc)
        mom = np.zeros((nc, 3))
        for lf, fv in enumerate(self._FACE_VERTS):
            P = [corners[v] for v in fv]
            m = sum(P) / 4.0
            nsum = np.zeros((nc, 3))
            csum = np.zeros((nc, 3))
            asum = np.zeros(nc)
            for q in range(4):
                a, b = P[q], P[(q + 1) % 4]
                tn = 0.5 * np.cross(a - m, b - m)
                ta = np.linalg.norm(tn, axis=1)
                tc = (a + b + m) / 3.0
                nsum += tn
                csum += tc * ta[:, None]
                asum += ta
                # tetrahedron (xc0, m, a, b): signed volume and centroid
                tv = np.einsum("ij,ij->i", tn, m - xc0) / 3.0
                vol += tv
                mom += tv[:, None] * (xc0 + m + a + b) / 4.0
            A = np.linalg.norm(nsum, axis=1)
            area[:, lf] = A
            fnorm[:, lf] = nsum / A[:, None]
            fcent[:, lf] = csum / asum[:, None]
        self.area = area.ravel()
        self.fcentroid = fcent.reshape(-1, 3)
        self.fnormal = fnorm.reshape(-1, 3)
        self.volume = vol
        self.ccentroid = mom / vol[:, None]
