"""FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

ctypes binding of ``oracle/porsol_oracle.cpp``, the serial C++ restatement of
OPM/opm-porsol's mimetic pressure solver (IncompFlowSolverHybrid +
MimeticIPEvaluator) and explicit upstream transport (EulerUpstream).  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only to check results; the GPU product
library never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libporsol_oracle.so")

BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2


def build(verbose: bool = False) -> str:
    """Compile the oracle with g++ (plain -O3; portable to x86_64 and aarch64)."""
    os.makedirs(LIB_DIR, exist_ok=True)
    src = os.path.join(HERE, "porsol_oracle.cpp")
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", src, "-o", LIB_PATH]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB_PATH


class _Grid(C.Structure):
    _fields_ = [
        ("num_cells", C.c_int),
        ("cell_facepos", C.c_void_p),
        ("hf_neighbour", C.c_void_p),
        ("hf_bid", C.c_void_p),
        ("hf_area", C.c_void_p),
        ("hf_centroid", C.c_void_p),
        ("hf_normal", C.c_void_p),
        ("cell_volume", C.c_void_p),
        ("cell_centroid", C.c_void_p),
    ]


class TransportOpts(C.Structure):
    _fields_ = [
        ("courant_number", C.c_double),
        ("method_viscous", C.c_int), ("method_gravity", C.c_int), ("method_capillary", C.c_int),
        ("use_cfl_viscous", C.c_int), ("use_cfl_gravity", C.c_int), ("use_cfl_capillary", C.c_int),
        ("minimum_small_steps", C.c_int), ("maximum_small_steps", C.c_int),
        ("check_sat", C.c_int), ("clamp_sat", C.c_int),
    ]

    @classmethod
    def defaults(cls, **kw):
        """EulerUpstream defaults (EulerUpstream_impl.hpp:60-72)."""
        o = cls(0.5, 1, 1, 1, 1, 1, 1, 1, 10000, 1, 0)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class Fluid(C.Structure):
    _fields_ = [("viscosity1", C.c_double), ("viscosity2", C.c_double),
                ("density1", C.c_double), ("density2", C.c_double),
                ("rocks", C.c_void_p)]


class _RockTables(C.Structure):
    _fields_ = [("num_rocks", C.c_int), ("table_pos", C.c_void_p), ("s", C.c_void_p), ("krw", C.c_void_p),
                ("kro", C.c_void_p), ("jfunc", C.c_void_p), ("cell_rock", C.c_void_p),
                ("use_jfunction_scaling", C.c_int), ("sigma_cos_theta", C.c_double)]


class RockTables:
    """RockJfunc tables (common/RockJfunc.hpp:63-216): ``tables`` is a list of (n, 4) arrays with
    the columns s, krw, kro, J of each rock; ``cell_rock`` the rock of every cell."""

    def __init__(self, tables, cell_rock, use_jfunction_scaling=True, sigma_cos_theta=1.0):
        cat = np.concatenate([np.asarray(t, np.float64).reshape(-1, 4) for t in tables])
        self.pos = np.cumsum([0] + [len(np.asarray(t).reshape(-1, 4)) for t in tables]).astype(np.int32)
        self.cols = [np.ascontiguousarray(cat[:, k]) for k in range(4)]
        self.cell = _i32(cell_rock)
        self.s = _RockTables(len(tables), _p(self.pos), *(_p(c) for c in self.cols), _p(self.cell),
                             1 if use_jfunction_scaling else 0, float(sigma_cos_theta))

    def fluid(self, mu1, mu2, rho1=0.0, rho2=0.0) -> Fluid:
        f = Fluid(mu1, mu2, rho1, rho2, C.addressof(self.s))
        f._rocks_ref = self   # keep the tables alive with the fluid
        return f


class CapillaryOpts(C.Structure):
    _fields_ = [("method_viscous", C.c_int), ("method_gravity", C.c_int), ("check_sat", C.c_int),
                ("clamp_sat", C.c_int), ("residual_tolerance", C.c_double), ("linsolver_type", C.c_int),
                ("update_relaxation", C.c_double)]

    @classmethod
    def defaults(cls, **kw):
        """ImplicitCapillarity defaults (euler/ImplicitCapillarity_impl.hpp:59-68)."""
        o = cls(1, 1, 1, 0, 1e-8, 1, 1.0)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, ip, dp, i, d = C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(_Grid), ip, ip]
        L.orc_destroy.argtypes = [vp]
        for n in ("orc_num_dofs", "orc_nnz", "orc_max_ncf", "orc_num_internal_faces"):
            getattr(L, n).restype = i
            getattr(L, n).argtypes = [vp]
        L.orc_get_structure.argtypes = [vp, ip, ip, ip, ip]
        L.orc_compute_inner_products.argtypes = [vp, dp, dp]
        L.orc_get_inner_products.argtypes = [vp, dp, dp]
        L.orc_assemble.argtypes = [vp, dp, dp, ip, dp, dp]
        L.orc_get_system.argtypes = [vp, dp, dp, dp, dp, dp, ip]
        L.orc_solve.restype = i
        L.orc_solve.argtypes = [vp, dp, dp, ip, dp, dp, d, i, i, ip, dp]
        L.orc_solve_timed.restype = i
        L.orc_solve_timed.argtypes = [vp, dp, dp, ip, dp, dp, d, i, i, ip, dp, dp]
        L.orc_solve_milestone.restype = i
        L.orc_solve_milestone.argtypes = [vp, dp, dp, ip, dp, dp, d, i, i, ip, dp, dp, d, ip, dp]
        L.orc_get_solution.argtypes = [vp, dp, dp, dp]
        L.orc_post_process_fluxes.restype = d
        L.orc_post_process_fluxes.argtypes = [vp]
        L.orc_solve_tensor.restype = i
        L.orc_solve_tensor.argtypes = [vp, dp, dp, ip, dp, dp, d, i, ip, dp]
        L.orc_adjoint_gradient.restype = i
        L.orc_adjoint_gradient.argtypes = [vp, dp, dp, dp, i, d, dp, dp, ip]
        L.orc_ilu0_cg.restype = i
        L.orc_ilu0_cg.argtypes = [i, ip, ip, dp, dp, dp, d, i, ip, dp]
        L.orc_cfl_factors.argtypes = [C.POINTER(Fluid), i, dp, dp, dp]
        L.orc_transport_cfl.restype = d
        L.orc_transport_cfl.argtypes = [C.POINTER(_Grid), dp, dp, C.POINTER(Fluid), C.POINTER(TransportOpts), dp, dp]
        L.orc_transport_residual.argtypes = [C.POINTER(_Grid), dp, dp, C.POINTER(Fluid), C.POINTER(TransportOpts),
                                             ip, dp, ip, dp, dp, dp, dp, dp]
        L.orc_capillary_solve.restype = i
        L.orc_capillary_solve.argtypes = [vp, C.POINTER(_Grid), dp, dp, C.POINTER(Fluid), C.POINTER(CapillaryOpts),
                                          ip, dp, ip, ip, dp, dp, dp, dp, dp, dp, ip, ip]
        L.orc_transport_solve.restype = i
        L.orc_transport_solve.argtypes = [C.POINTER(_Grid), dp, dp, C.POINTER(Fluid), C.POINTER(TransportOpts),
                                          ip, dp, ip, dp, dp, dp, d, dp, ip, ip]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class GridRef:
    """Keeps numpy arrays of a flattened grid alive while C holds pointers."""

    def __init__(self, grid):
        a = grid.arrays()
        self._a = a
        self.num_cells = a["num_cells"]
        self.nhf = int(a["facepos"][-1])
        self.s = _Grid(a["num_cells"], _p(a["facepos"]), _p(a["neighbour"]), _p(a["bid"]), _p(a["area"]),
                       _p(a["fcentroid"]), _p(a["fnormal"]), _p(a["volume"]), _p(a["ccentroid"]))


class OraclePressure:
    """IncompFlowSolverHybrid restated on the CPU (FP64)."""

    def __init__(self, grid, hf_flow_type, hf_partner_bid=None):
        self.g = GridRef(grid)
        self._bct = _i32(hf_flow_type)
        self._pb = None if hf_partner_bid is None else _i32(hf_partner_bid)
        self.h = lib().orc_create(C.byref(self.g.s), _p(self._bct), _p(self._pb))
        if not self.h:
            raise RuntimeError("oracle init failed")
        L = lib()
        self.n = L.orc_num_dofs(self.h)
        self.nnz = L.orc_nnz(self.h)
        self.max_ncf = L.orc_max_ncf(self.h)
        self.num_internal_faces = L.orc_num_internal_faces(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def structure(self):
        cf = np.empty(self.g.nhf, np.int32)
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        pp = np.empty(self.n, np.int32)
        lib().orc_get_structure(self.h, _p(cf), _p(rp), _p(ci), _p(pp))
        return cf, rp, ci, pp

    def compute_inner_products(self, K9, grav=(0.0, 0.0, 0.0)):
        self._K = _f64(K9)
        g = _f64(grav)
        lib().orc_compute_inner_products(self.h, _p(self._K), _p(g))

    def inner_products(self):
        nf = np.diff(self.g._a["facepos"])
        B = np.empty(int((nf * nf).sum()))
        gf = np.empty(self.g.nhf)
        lib().orc_get_inner_products(self.h, _p(B), _p(gf))
        return B, gf

    def assemble(self, totmob, mobdens, bc_type, bc_value, src):
        args = [_f64(totmob), _f64(mobdens), _i32(bc_type), _f64(bc_value), _f64(src)]
        lib().orc_assemble(self.h, *[_p(a) for a in args])

    def system(self):
        S = np.empty(self.nnz)
        rhs = np.empty(self.n)
        F = np.empty(self.g.nhf)
        L = np.empty(self.g.num_cells)
        g = np.empty(self.g.num_cells)
        dr = np.zeros(1, np.int32)
        lib().orc_get_system(self.h, _p(S), _p(rhs), _p(F), _p(L), _p(g), _p(dr))
        return dict(S=S, rhs=rhs, F=F, L=L, g=g, do_reg=bool(dr[0]))

    def solve(self, totmob, mobdens, bc_type, bc_value, src, tol=1e-8, maxit=0, dirichlet_guess=False):
        args = [_f64(totmob), _f64(mobdens), _i32(bc_type), _f64(bc_value), _f64(src)]
        it = np.zeros(1, np.int32)
        red = np.zeros(1)
        rc = lib().orc_solve(self.h, *[_p(a) for a in args], float(tol), int(maxit), int(dirichlet_guess),
                             _p(it), _p(red))
        self.iterations = int(it[0])
        self.reduction = float(red[0])
        return rc

    def solve_tensor(self, lam9, rlam9, bc_type, bc_value, src, tol=1e-8, maxit=0):
        """Solve with per-cell total mobility tensors (MimeticIPAnisoRelpermEvaluator)."""
        keep = [_f64(lam9), None if rlam9 is None else _f64(rlam9), _i32(bc_type), _f64(bc_value), _f64(src)]
        it = np.zeros(1, np.int32)
        red = np.zeros(1)
        rc = lib().orc_solve_tensor(self.h, *[_p(a) for a in keep], float(tol), int(maxit), _p(it), _p(red))
        self.iterations = int(it[0])
        self.reduction = float(red[0])
        return rc

    def solve_timed(self, totmob, mobdens, bc_type, bc_value, src, tol=1e-8, maxit=0, dirichlet_guess=False):
        """As solve(); returns (rc, seconds of assembly+recovery, of the ILU0 factorisation, of CG)."""
        args = [_f64(totmob), _f64(mobdens), _i32(bc_type), _f64(bc_value), _f64(src)]
        it = np.zeros(1, np.int32)
        red = np.zeros(1)
        sec = np.zeros(3)
        rc = lib().orc_solve_timed(self.h, *[_p(a) for a in args], float(tol), int(maxit), int(dirichlet_guess),
                                   _p(it), _p(red), _p(sec))
        self.iterations = int(it[0])
        self.reduction = float(red[0])
        return rc, float(sec[0]), float(sec[1]), float(sec[2])

    def solve_milestone(self, totmob, mobdens, bc_type, bc_value, src, tol, milestone_tol, maxit=0,
                        dirichlet_guess=False):
        """As solve_timed(); also (iteration, CG seconds) at which the residual reduction first fell
        below milestone_tol.  Returns (rc, t_fixed, t_factor, t_cg, milestone_iteration, milestone_seconds)."""
        args = [_f64(totmob), _f64(mobdens), _i32(bc_type), _f64(bc_value), _f64(src)]
        it = np.zeros(1, np.int32)
        red = np.zeros(1)
        sec = np.zeros(3)
        mit = np.zeros(1, np.int32)
        msec = np.zeros(1)
        rc = lib().orc_solve_milestone(self.h, *[_p(a) for a in args], float(tol), int(maxit), int(dirichlet_guess),
                                       _p(it), _p(red), _p(sec), float(milestone_tol), _p(mit), _p(msec))
        self.iterations = int(it[0])
        self.reduction = float(red[0])
        return rc, float(sec[0]), float(sec[1]), float(sec[2]), int(mit[0]), float(msec[0])

    def solution(self):
        p = np.empty(self.g.num_cells)
        v = np.empty(self.g.nhf)
        pi = np.empty(self.n)
        lib().orc_get_solution(self.h, _p(p), _p(v), _p(pi))
        return p, v, pi

    def post_process_fluxes(self):
        return lib().orc_post_process_fluxes(self.h)

    def adjoint_gradient(self, cell_weight=None, cell_target=None, hf_weight=None, mode=0, tol=1e-12):
        """(rc, J, gradient) of J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf for the last solve;
        gradient per cell (mode 0) or (nc, 3) per axis (mode 1)."""
        keep = [None if a is None else _f64(a) for a in (cell_weight, cell_target, hf_weight)]
        nc = self.g.num_cells
        grad = np.zeros(nc * (3 if mode == 1 else 1))
        J = np.zeros(1)
        it = np.zeros(1, np.int32)
        rc = lib().orc_adjoint_gradient(self.h, *[_p(a) for a in keep], int(mode), float(tol), _p(grad), _p(J),
                                        _p(it))
        self.adjoint_iterations = int(it[0])
        return rc, float(J[0]), (grad.reshape(nc, 3) if mode == 1 else grad)


def upscale_periodic(grid, K9, tol=1e-13):
    """Effective permeability (3x3) of one fully periodic Cartesian grid with unique boundary ids.

    Three solves with unit total mobility: periodic pressure jump +1 on the low side and -1 on the
    high side of axis d (the pattern of setupUpscalingConditions,
    opm/porsol/common/setupBoundaryConditions.hpp:136-157), Neumann nowhere.  Darcy averaging over
    the periodic cell gives K_eff[i, d] = L_d Q_i / A_i, Q_i the flux through the high side of axis
    i, A_i its area, L_d the extent along d.  The reference leaves this step to opm-upscaling; the
    same formula is what the GPU batch computes.  Returns (keff, total CG iterations)."""
    pb = grid.periodic_partner_bids()
    bct = np.where(grid.boundary, BC_PERIODIC, BC_NEUMANN).astype(np.int32)
    o = OraclePressure(grid, bct, pb)
    o.compute_inner_products(np.ascontiguousarray(K9, dtype=np.float64).ravel())
    nc = grid.num_cells
    keff = np.zeros((3, 3))
    its = 0
    for d in range(3):
        bcv = np.zeros(grid.num_half_faces)
        bcv[grid.side == 2 * d + 1] = 1.0
        bcv[grid.side == 2 * d + 2] = -1.0
        rc = o.solve(np.ones(nc), np.zeros(nc), bct, bcv, np.zeros(nc), tol=tol)
        if rc != 0:
            raise RuntimeError(f"oracle periodic solve failed ({rc})")
        its += o.iterations
        _, v, _ = o.solution()
        lo, hi = grid.side == 2 * d + 1, grid.side == 2 * d + 2
        L = grid.fcentroid[hi, d].max() - grid.fcentroid[lo, d].min()
        for i in range(3):
            h = grid.side == 2 * i + 2
            keff[i, d] = L * v[h].sum() / grid.area[h].sum()
    return keff, its


def cell_fields(grid, outflux, sat=None, mu1=1.0, mu2=1.0):
    """Output fields of common/SimulatorUtilities.hpp restated with numpy: estimateCellVelocity
    (:54-82), computePhaseVelocities (:144-160) with the Corey-2 fractional flow, and
    computeCapPressure (:214-225) with the no-rock-table curve 1e5 (1 - s)
    (ReservoirPropertyCommon_impl.hpp:466-476)."""
    cell = np.repeat(np.arange(grid.num_cells), np.diff(grid.facepos))
    d = (grid.fcentroid - grid.ccentroid[cell]) * outflux[:, None]
    vel = np.zeros((grid.num_cells, 3))
    np.add.at(vel, cell, d)
    vel /= grid.volume[:, None]
    out = {"velocity": vel}
    if sat is not None:
        m1 = sat * sat / mu1
        m2 = (1.0 - sat) ** 2 / mu2
        fw = m1 / (m1 + m2)
        out.update(fractional_flow=fw, water_velocity=fw[:, None] * vel, oil_velocity=(1 - fw)[:, None] * vel,
                   cap_pressure=1e5 * (1.0 - sat))
    return out


def ilu0_cg(rowptr, colind, vals, b, x0=None, tol=1e-8, maxit=0):
    rowptr, colind, vals, b = _i32(rowptr), _i32(colind), _f64(vals), _f64(b)
    n = len(b)
    x = np.zeros(n) if x0 is None else _f64(x0).copy()
    it = np.zeros(1, np.int32)
    red = np.zeros(1)
    rc = lib().orc_ilu0_cg(n, _p(rowptr), _p(colind), _p(vals), _p(b), _p(x), float(tol), int(maxit), _p(it), _p(red))
    return rc, x, int(it[0]), float(red[0])


def cfl_factors(fluid: Fluid, K9=None, poro=None):
    out = np.zeros(3)
    K = None if K9 is None else _f64(K9)
    ph = None if poro is None else _f64(poro)
    lib().orc_cfl_factors(C.byref(fluid), 0 if ph is None else len(ph), _p(K), _p(ph), _p(out))
    return out


class OracleTransport:
    """EulerUpstream restated on the CPU (FP64), scalar mobilities: Corey-2, or the rock tables
    the fluid carries (RockTables.fluid)."""

    def __init__(self, grid, K9, poro, fluid: Fluid, sat_type, sat_value, partner_bid=None, opts=None):
        self.g = GridRef(grid)
        self.K = _f64(K9)
        self.poro = _f64(poro)
        self.fluid = fluid
        self.st = _i32(sat_type)
        self.sv = _f64(sat_value)
        self.pb = _i32(np.zeros(self.g.nhf, np.int32) if partner_bid is None else partner_bid)
        self.opts = opts if opts is not None else TransportOpts.defaults()

    def cfl(self, outflux, grav=(0.0, 0.0, 0.0)):
        return lib().orc_transport_cfl(C.byref(self.g.s), _p(self.K), _p(self.poro), C.byref(self.fluid),
                                       C.byref(self.opts), _p(_f64(outflux)), _p(_f64(grav)))

    def residual(self, sat, outflux, injection=None, grav=(0.0, 0.0, 0.0)):
        inj = np.zeros(self.g.num_cells) if injection is None else _f64(injection)
        res = np.empty(self.g.num_cells)
        lib().orc_transport_residual(C.byref(self.g.s), _p(self.K), _p(self.poro), C.byref(self.fluid),
                                     C.byref(self.opts),
                                     _p(self.st), _p(self.sv), _p(self.pb), _p(_f64(outflux)), _p(inj),
                                     _p(_f64(sat)), _p(_f64(grav)), _p(res))
        return res

    def solve(self, sat, time, outflux, injection=None, grav=(0.0, 0.0, 0.0)):
        s = _f64(sat).copy()
        inj = np.zeros(self.g.num_cells) if injection is None else _f64(injection)
        ns = np.zeros(1, np.int32)
        rp = np.zeros(1, np.int32)
        rc = lib().orc_transport_solve(C.byref(self.g.s), _p(self.K), _p(self.poro), C.byref(self.fluid),
                                       C.byref(self.opts), _p(self.st), _p(self.sv), _p(self.pb),
                                       _p(_f64(outflux)), _p(inj), _p(s), float(time), _p(_f64(grav)),
                                       _p(ns), _p(rp))
        return rc, s, int(ns[0]), int(rp[0])


def capillary_solve(pressure: OraclePressure, transport: OracleTransport, sat, outflux, bc_type, bc_value,
                    injection=None, grav=(0.0, 0.0, 0.0), opts=None):
    """ImplicitCapillarity::transportSolve restated (euler/ImplicitCapillarity_impl.hpp:138-226).
    ``pressure`` must hold the inner products for zero gravity.  Returns (rc, sat, shift,
    root_iterations, cg_iterations); rc as orc_capillary_solve."""
    T = transport
    s = _f64(sat).copy()
    inj = np.zeros(T.g.num_cells) if injection is None else _f64(injection)
    o = opts if opts is not None else CapillaryOpts.defaults()
    shift = np.zeros(1)
    rit = np.zeros(1, np.int32)
    cit = np.zeros(1, np.int32)
    rc = lib().orc_capillary_solve(pressure.h, C.byref(T.g.s), _p(T.K), _p(T.poro), C.byref(T.fluid), C.byref(o),
                                   _p(T.st), _p(T.sv), _p(T.pb), _p(_i32(bc_type)), _p(_f64(bc_value)),
                                   _p(_f64(outflux)), _p(inj), _p(s), _p(_f64(grav)), _p(shift), _p(rit), _p(cit))
    return rc, s, float(shift[0]), int(rit[0]), int(cit[0])
