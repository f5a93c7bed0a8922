"""porsol-gb300: GB300-native mimetic pressure / upstream transport library.

This Python module is the build driver and a thin ctypes binding of the C ABI
declared in include/porsol_gpu.h, used by the test-suite and the benchmark.
The product is the CUDA/C++ shared library ``lib/libporsol_gpu.so``; there is
no Python compute path and no CPU fallback: if the library is missing or
fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libporsol_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]
SOURCES = ["structure.cpp", "k_mimetic.cu", "k_krylov.cu", "k_amg.cu", "k_transport.cu", "k_capillary.cu", "k_adjoint.cu",
           "k_batch.cu", "k_upscale.cu", "capi.cu", "noalloc_cfl.cu"]

BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2
FLUID_CELLWISE, FLUID_COREY2, FLUID_TENSOR = 0, 1, 2
FP64, MIXED = 0, 1
GRAD_LOGK, GRAD_LOGK_AXES = 0, 1
UPSCALE_AMG, UPSCALE_PERSISTENT = 0, 1
ERR = {0: "OK", 1: "NOT_CONVERGED", 2: "BAD_ARG", 3: "NONFINITE", 4: "SAT_RANGE", 5: "CUDA", 6: "TIMEOUT",
       7: "STATE", 8: "UNKNOWN_SOLVER", 9: "CFL"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def build(verbose: bool = False, jobs: int = 8) -> str:
    """Compile every translation unit for sm_103a in parallel and link the shared library."""
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)

    def compile_one(src):
        out = os.path.join(obj_dir, src + ".o")
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", out]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return out

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ----------------------------------------------------------------------------- ctypes
class Grid(C.Structure):
    _fields_ = [("num_cells", C.c_int), ("cell_facepos", C.c_void_p), ("hf_neighbour", C.c_void_p),
                ("hf_bid", C.c_void_p), ("hf_area", C.c_void_p), ("hf_centroid", C.c_void_p),
                ("hf_normal", C.c_void_p), ("cell_volume", C.c_void_p), ("cell_centroid", C.c_void_p)]


class Fluid(C.Structure):
    _fields_ = [("model", C.c_int), ("viscosity1", C.c_double), ("viscosity2", C.c_double),
                ("density1", C.c_double), ("density2", C.c_double)]


class SolveOpts(C.Structure):
    _fields_ = [("residual_tolerance", C.c_double), ("linsolver_verbosity", C.c_int),
                ("linsolver_type", C.c_int), ("same_matrix", C.c_int), ("linsolver_maxit", C.c_int),
                ("prolongate_factor", C.c_double), ("smooth_steps", C.c_int), ("precision", C.c_int),
                ("inner_tolerance", C.c_double), ("max_outer", C.c_int)]


class Objective(C.Structure):
    _fields_ = [("cell_weight", C.c_void_p), ("cell_target", C.c_void_p), ("hf_weight", C.c_void_p)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int), ("reduction", C.c_double),
                ("amg_levels", C.c_int), ("mass_balance", C.c_double), ("ms_assemble", C.c_double),
                ("ms_precond_setup", C.c_double), ("ms_krylov", C.c_double), ("ms_recover", C.c_double)]


class TransportOpts(C.Structure):
    _fields_ = [("courant_number", C.c_double),
                ("method_viscous", C.c_int), ("method_gravity", C.c_int), ("method_capillary", C.c_int),
                ("use_cfl_viscous", C.c_int), ("use_cfl_gravity", C.c_int), ("use_cfl_capillary", C.c_int),
                ("minimum_small_steps", C.c_int), ("maximum_small_steps", C.c_int),
                ("check_sat", C.c_int), ("clamp_sat", C.c_int)]


class TransportStats(C.Structure):
    _fields_ = [("small_steps", C.c_int), ("repeats", C.c_int), ("cfl_dt", C.c_double)]


class RockTablesStruct(C.Structure):
    _fields_ = [("num_rocks", C.c_int), ("table_pos", C.c_void_p), ("s", C.c_void_p), ("krw", C.c_void_p),
                ("kro", C.c_void_p), ("jfunc", C.c_void_p), ("cell_rock", C.c_void_p),
                ("use_jfunction_scaling", C.c_int), ("sigma_cos_theta", C.c_double)]


class CapillaryOpts(C.Structure):
    _fields_ = [("method_viscous", C.c_int), ("method_gravity", C.c_int), ("check_sat", C.c_int),
                ("clamp_sat", C.c_int), ("residual_tolerance", C.c_double), ("linsolver_verbosity", C.c_int),
                ("linsolver_type", C.c_int), ("update_relaxation", C.c_double), ("precision", C.c_int)]


class CapillaryStats(C.Structure):
    _fields_ = [("shift", C.c_double), ("root_iterations", C.c_int), ("evaluations", C.c_int),
                ("pressure", SolveStats)]


# (name, restype, argtypes) of every exported entry point of include/porsol_gpu.h
_vp, _i, _d = C.c_void_p, C.c_int, C.c_double
EXPORTS = [
    ("porsol_solve_opts_default", None, [C.POINTER(SolveOpts)]),
    ("porsol_create", _i, [C.POINTER(_vp)]),
    ("porsol_destroy", None, [_vp]),
    ("porsol_last_error", C.c_char_p, [_vp]),
    ("porsol_clear", _i, [_vp]),
    ("porsol_init_system_structure", _i, [_vp, C.POINTER(Grid), _vp, _vp]),
    ("porsol_compute_inner_products", _i, [_vp, _vp, _vp]),
    ("porsol_assemble_static", _i, [_vp, _vp, _vp]),
    ("porsol_init", _i, [_vp, C.POINTER(Grid), _vp, _vp, _vp, _vp]),
    ("porsol_solve", _i, [_vp, C.POINTER(Fluid), _vp, _vp, _vp, _vp, _vp, C.POINTER(SolveOpts),
                          C.POINTER(SolveStats)]),
    ("porsol_solve_device", _i, [_vp, C.POINTER(Fluid), _vp, _vp, _vp, _vp, _vp, C.POINTER(SolveOpts),
                                 C.POINTER(SolveStats)]),
    ("porsol_post_process_fluxes", _i, [_vp, C.POINTER(_d)]),
    ("porsol_get_solution", _i, [_vp, _vp, _vp, _vp]),
    ("porsol_get_solution_device", _i, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    ("porsol_num_dofs", _i, [_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    ("porsol_get_structure", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("porsol_get_inner_products", _i, [_vp, _vp, _vp]),
    ("porsol_get_system", _i, [_vp, _vp, _vp]),
    ("porsol_amg_info", _i, [_vp, _i, C.POINTER(_i), _vp, _vp]),
    ("porsol_solve_bytes", _i, [_vp, _vp, _i, _vp]),
    ("porsol_upscale_periodic", _i, [_vp, C.POINTER(Grid), _i, _vp, _vp, _vp, _vp, C.POINTER(SolveOpts), _vp,
                                     C.POINTER(SolveStats)]),
    ("porsol_upscale_set_schedule", _i, [_vp, _i, _i, _i, _i, _i, _i]),
    ("porsol_upscale_last_schedule", _i, [_vp] + [C.POINTER(_i)] * 6),
    ("porsol_cell_fields", _i, [_vp, C.POINTER(Fluid), _vp, _vp, _vp, _vp, _vp, _vp]),
    ("porsol_write_field", _i, [_vp, _i, C.c_char_p]),
    ("porsol_objective_value", _i, [_vp, C.POINTER(Objective), C.POINTER(_d)]),
    ("porsol_adjoint_gradient", _i, [_vp, C.POINTER(Objective), _i, C.POINTER(SolveOpts), C.POINTER(_d), _vp,
                                     C.POINTER(SolveStats)]),
    ("porsol_transport_opts_default", None, [C.POINTER(TransportOpts)]),
    ("porsol_transport_create", _i, [C.POINTER(_vp)]),
    ("porsol_transport_destroy", None, [_vp]),
    ("porsol_transport_last_error", C.c_char_p, [_vp]),
    ("porsol_transport_init", _i, [_vp, C.POINTER(Grid), _vp, _vp, C.POINTER(Fluid), _vp, _vp, _vp,
                                   C.POINTER(TransportOpts)]),
    ("porsol_transport_solve", _i, [_vp, _vp, _d, _vp, _vp, _vp, C.POINTER(TransportStats)]),
    ("porsol_transport_solve_device", _i, [_vp, _vp, _d, _vp, _vp, _vp, C.POINTER(TransportStats)]),
    ("porsol_transport_set_options", _i, [_vp, C.POINTER(TransportOpts)]),
    ("porsol_transport_set_rock_tables", _i, [_vp, C.POINTER(RockTablesStruct)]),
    ("porsol_capillary_opts_default", None, [C.POINTER(CapillaryOpts)]),
    ("porsol_capillary_solve", _i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(CapillaryOpts),
                                    C.POINTER(CapillaryStats)]),
    ("porsol_capillary_solve_device", _i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(CapillaryOpts),
                                           C.POINTER(CapillaryStats)]),
    ("porsol_profile_enable", _i, [_vp, _i]),
    ("porsol_profile_get", _i, [_vp, _i, C.POINTER(_i), C.POINTER(_d), C.POINTER(_d)]),
    ("porsol_profile_reset", _i, [_vp]),
    ("porsol_stream", _vp, [_vp]),
    ("porsol_launch_count", C.c_longlong, []),
    ("porsol_selftest_bulk_wait", C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("porsol_transport_cfl_noalloc", _i, [_i, _vp, _vp, _vp, _vp, _d, C.POINTER(_d), _vp]),
]

_lib = None


def lib():
    """Load the CUDA library (fails loudly when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run build() first (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in EXPORTS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def selftest_bulk_wait(expire: bool = False):
    """One run of the finest-level smoother step that stages its slices by bulk copy, on the fixed
    64-row system of porsol_selftest_bulk_wait; expire makes every wait for the copies run out.
    Returns (status code, r, d, x)."""
    r = np.zeros(64, np.float32)
    d = np.zeros(64, np.float32)
    x = np.zeros(64, np.float32)
    rc = lib().porsol_selftest_bulk_wait(1 if expire else 0, _p(r), _p(d), _p(x))
    return rc, r, d, x


class PorsolError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{ERR.get(code, code)}] {msg}")
        self.code = code


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class _GridArrays:
    def __init__(self, grid):
        a = grid.arrays()
        self.a = a
        self.num_cells = a["num_cells"]
        self.nhf = int(a["facepos"][-1])
        self.s = Grid(a["num_cells"], _p(a["facepos"]).value, _p(a["neighbour"]).value, _p(a["bid"]).value,
                      _p(a["area"]).value, _p(a["fcentroid"]).value, _p(a["fnormal"]).value,
                      _p(a["volume"]).value, _p(a["ccentroid"]).value)


def write_field(field, filename):
    """writeField: count, then one value per line (%g), written by the library."""
    f = _f64(field)
    rc = lib().porsol_write_field(_p(f), len(f), str(filename).encode())
    if rc != 0:
        raise PorsolError(rc, f"cannot write {filename}")


def default_solve_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    lib().porsol_solve_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_capillary_opts(**kw) -> CapillaryOpts:
    o = CapillaryOpts()
    lib().porsol_capillary_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_transport_opts(**kw) -> TransportOpts:
    o = TransportOpts()
    lib().porsol_transport_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class PressureSolver:
    """Python face of the C ABI, named like IncompFlowSolverHybrid's methods."""

    def __init__(self):
        h = C.c_void_p()
        rc = lib().porsol_create(C.byref(h))
        if rc != 0:
            raise PorsolError(rc, "porsol_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().porsol_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise PorsolError(rc, lib().porsol_last_error(self.h).decode())

    def init(self, grid, perm, grav=(0.0, 0.0, 0.0), flow_type=None, partner_bid=None):
        self.grid = _GridArrays(grid)
        self._ft = None if flow_type is None else _i32(flow_type)
        self._pb = None if partner_bid is None else _i32(partner_bid)
        self._check(lib().porsol_init_system_structure(self.h, C.byref(self.grid.s), _p(self._ft), _p(self._pb)))
        self.compute_inner_products(perm, grav)
        n, nnz, mx, ni = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._check(lib().porsol_num_dofs(self.h, C.byref(n), C.byref(nnz), C.byref(mx), C.byref(ni)))
        self.n, self.nnz, self.max_ncf, self.num_internal_faces = n.value, nnz.value, mx.value, ni.value

    def compute_inner_products(self, perm, grav=(0.0, 0.0, 0.0)):
        self._perm = _f64(perm)
        g = _f64(grav)
        self._check(lib().porsol_compute_inner_products(self.h, _p(self._perm), _p(g)))

    assemble_static = compute_inner_products

    def solve(self, fluid: Fluid, sat, bc_type, bc_value, src, mobdens=None, opts: SolveOpts = None):
        st = SolveStats()
        o = opts if opts is not None else default_solve_opts()
        args = [_f64(sat), None if mobdens is None else _f64(mobdens), _i32(bc_type), _f64(bc_value), _f64(src)]
        self._check(lib().porsol_solve(self.h, C.byref(fluid), *[_p(a) for a in args], C.byref(o), C.byref(st)))
        return st

    def solve_device(self, fluid, d_sat, d_bct, d_bcv, d_src, d_mobdens=0, opts=None):
        """All arrays are raw device addresses (ints)."""
        st = SolveStats()
        o = opts if opts is not None else default_solve_opts()
        self._check(lib().porsol_solve_device(self.h, C.byref(fluid), C.c_void_p(d_sat), C.c_void_p(d_mobdens or None),
                                              C.c_void_p(d_bct), C.c_void_p(d_bcv), C.c_void_p(d_src), C.byref(o),
                                              C.byref(st)))
        return st

    def upscale_periodic(self, grid, cellpos, partner_bid, side, perm, opts=None):
        """Effective permeability (num_grids, 3, 3) of a batch of periodic sub-grids."""
        self.grid = _GridArrays(grid)
        keep = [_i32(cellpos), _i32(partner_bid), _i32(side), _f64(perm)]
        ng = len(keep[0]) - 1
        keff = np.zeros(9 * ng)
        st = SolveStats()
        o = opts if opts is not None else default_solve_opts()
        self._check(lib().porsol_upscale_periodic(self.h, C.byref(self.grid.s), ng, *[_p(a) for a in keep],
                                                  C.byref(o), _p(keff), C.byref(st)))
        n, nnz, mx, ni = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._check(lib().porsol_num_dofs(self.h, C.byref(n), C.byref(nnz), C.byref(mx), C.byref(ni)))
        self.n, self.nnz = n.value, nnz.value
        return keff.reshape(ng, 3, 3), st

    def set_upscale_schedule(self, schedule, cta_threads=0, warp_max_unknowns=0, vector_layout=1, cluster_ctas=1,
                             cluster_min_unknowns=0):
        """UPSCALE_AMG (default) or UPSCALE_PERSISTENT (one launch; cta_threads 0 = autotuned)."""
        self._check(lib().porsol_upscale_set_schedule(self.h, int(schedule), int(cta_threads),
                                                      int(warp_max_unknowns), int(vector_layout), int(cluster_ctas),
                                                      int(cluster_min_unknowns)))

    def upscale_last_schedule(self):
        """dict(cta_threads, warp_max_unknowns, vector_layout, cluster_ctas, cluster_min_unknowns, tuned) of the
        last persistent-schedule call (zeros after an AMG-schedule call)."""
        v = [C.c_int() for _ in range(6)]
        self._check(lib().porsol_upscale_last_schedule(self.h, *[C.byref(x) for x in v]))
        keys = ("cta_threads", "warp_max_unknowns", "vector_layout", "cluster_ctas", "cluster_min_unknowns")
        out = {k: x.value for k, x in zip(keys, v)}
        out["tuned"] = bool(v[5].value)
        return out

    def _objective(self, cell_weight, cell_target, hf_weight):
        keep = [None if a is None else _f64(a) for a in (cell_weight, cell_target, hf_weight)]
        obj = Objective(*[None if a is None else a.ctypes.data for a in keep])
        return obj, keep

    def objective(self, cell_weight=None, cell_target=None, hf_weight=None):
        """J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf of the last solve."""
        obj, keep = self._objective(cell_weight, cell_target, hf_weight)
        J = C.c_double()
        self._check(lib().porsol_objective_value(self.h, C.byref(obj), C.byref(J)))
        return J.value

    def adjoint_gradient(self, cell_weight=None, cell_target=None, hf_weight=None, mode=GRAD_LOGK, opts=None):
        """(J, dJ/d ln k per cell (mode 0) or (nc, 3) per axis (mode 1), stats) of the last solve."""
        obj, keep = self._objective(cell_weight, cell_target, hf_weight)
        nc = self.grid.num_cells
        grad = np.empty(nc * (3 if mode == GRAD_LOGK_AXES else 1))
        J = C.c_double()
        st = SolveStats()
        self._check(lib().porsol_adjoint_gradient(self.h, C.byref(obj), int(mode),
                                                  None if opts is None else C.byref(opts), C.byref(J), _p(grad),
                                                  C.byref(st)))
        return J.value, (grad.reshape(nc, 3) if mode == GRAD_LOGK_AXES else grad), st

    def cell_fields(self, fluid=None, sat=None):
        """Cell velocity (nc, 3) and, with a Corey-2 fluid and saturations, water/oil velocities,
        fractional flow and capillary pressure (the fields of writeVtkOutput)."""
        nc = self.grid.num_cells
        out = {"velocity": np.empty((nc, 3))}
        satf = sat is not None
        if satf:
            out.update(water_velocity=np.empty((nc, 3)), oil_velocity=np.empty((nc, 3)),
                       fractional_flow=np.empty(nc), cap_pressure=np.empty(nc))
        s = None if not satf else _f64(sat)
        ptrs = [_p(out.get(k)) for k in ("velocity", "water_velocity", "oil_velocity", "fractional_flow",
                                          "cap_pressure")]
        self._check(lib().porsol_cell_fields(self.h, None if fluid is None else C.byref(fluid), _p(s), *ptrs))
        return out

    def post_process_fluxes(self):
        m = C.c_double()
        self._check(lib().porsol_post_process_fluxes(self.h, C.byref(m)))
        return m.value

    def solution(self):
        p = np.empty(self.grid.num_cells)
        v = np.empty(self.grid.nhf)
        pi = np.empty(self.n)
        self._check(lib().porsol_get_solution(self.h, _p(p), _p(v), _p(pi)))
        return p, v, pi

    def solution_device(self):
        """Device addresses of (pressure, outflux, face pressure), valid until the next solve."""
        p, v, pi = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self._check(lib().porsol_get_solution_device(self.h, C.byref(p), C.byref(v), C.byref(pi)))
        return p.value, v.value, pi.value

    def structure(self):
        cf = np.empty(self.grid.nhf, np.int32)
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        pp = np.empty(self.n, np.int32)
        self._check(lib().porsol_get_structure(self.h, _p(cf), _p(rp), _p(ci), _p(pp)))
        return cf, rp, ci, pp

    def inner_products(self):
        nf = np.diff(self.grid.a["facepos"])
        B = np.empty(int((nf * nf).sum()))
        gf = np.empty(self.grid.nhf)
        self._check(lib().porsol_get_inner_products(self.h, _p(B), _p(gf)))
        return B, gf

    def amg_info(self):
        nl = C.c_int()
        rows = np.zeros(64, np.int32)
        ent = np.zeros(64, np.int64)
        self._check(lib().porsol_amg_info(self.h, 64, C.byref(nl), _p(rows), _p(ent)))
        return rows[:nl.value].tolist(), ent[:nl.value].tolist()

    def solve_bytes(self, max_levels=64):
        """Algorithmic bytes of the last solve: dict(assembly, krylov, recovery, post, vcycle_levels)."""
        out = np.zeros(4)
        lv = np.zeros(max_levels)
        self._check(lib().porsol_solve_bytes(self.h, _p(out), max_levels, _p(lv)))
        return dict(assembly=out[0], krylov=out[1], recovery=out[2], post=out[3],
                    vcycle_levels=lv[:int(np.count_nonzero(lv))].tolist())

    def system(self):
        S = np.empty(self.nnz)
        rhs = np.empty(self.n)
        self._check(lib().porsol_get_system(self.h, _p(S), _p(rhs)))
        return S, rhs

    # profiling
    def profile_enable(self, on=True):
        self._check(lib().porsol_profile_enable(self.h, int(on)))

    def profile_get(self, kernel):
        n, ms, b = C.c_int(), C.c_double(), C.c_double()
        self._check(lib().porsol_profile_get(self.h, kernel, C.byref(n), C.byref(ms), C.byref(b)))
        return n.value, ms.value, b.value

    def profile_reset(self):
        self._check(lib().porsol_profile_reset(self.h))

    def stream(self):
        return lib().porsol_stream(self.h)


class TransportSolver:
    """Python face of the EulerUpstream C ABI."""

    def __init__(self):
        h = C.c_void_p()
        rc = lib().porsol_transport_create(C.byref(h))
        if rc != 0:
            raise PorsolError(rc, "porsol_transport_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().porsol_transport_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise PorsolError(rc, lib().porsol_transport_last_error(self.h).decode())

    def init(self, grid, perm, poro, fluid: Fluid, sat_type, sat_value, partner_bid=None, opts=None):
        self.grid = _GridArrays(grid)
        self._keep = [_f64(perm), _f64(poro), _i32(sat_type), _f64(sat_value),
                      None if partner_bid is None else _i32(partner_bid)]
        o = opts if opts is not None else default_transport_opts()
        self._check(lib().porsol_transport_init(self.h, C.byref(self.grid.s), *[_p(a) for a in self._keep[:2]],
                                                C.byref(fluid), *[_p(a) for a in self._keep[2:]], C.byref(o)))

    def solve_device(self, d_sat, time, d_outflux, d_injection=0, grav=(0.0, 0.0, 0.0)):
        """In-place update of the device saturation array (raw device addresses)."""
        st = TransportStats()
        g = _f64(grav)
        self._check(lib().porsol_transport_solve_device(self.h, C.c_void_p(d_sat), float(time), _p(g),
                                                        C.c_void_p(d_outflux), C.c_void_p(d_injection or None),
                                                        C.byref(st)))
        return st

    def solve(self, sat, time, outflux, injection=None, grav=(0.0, 0.0, 0.0)):
        s = _f64(sat).copy()
        st = TransportStats()
        g = _f64(grav)
        inj = None if injection is None else _f64(injection)
        self._check(lib().porsol_transport_solve(self.h, _p(s), float(time), _p(g), _p(_f64(outflux)), _p(inj),
                                                 C.byref(st)))
        return s, st

    def set_rock_tables(self, tables, cell_rock, use_jfunction_scaling=True, sigma_cos_theta=1.0):
        """RockJfunc tables: ``tables`` a list of (n, 4) arrays (columns s, krw, kro, J), one per rock;
        ``cell_rock`` the rock of every cell.  ``tables=None`` returns to Corey-2."""
        if tables is None:
            self._check(lib().porsol_transport_set_rock_tables(self.h, None))
            return
        arrs = [np.asarray(x, np.float64).reshape(-1, 4) for x in tables]
        cat = np.concatenate(arrs)
        pos = np.cumsum([0] + [len(a) for a in arrs]).astype(np.int32)
        cols = [np.ascontiguousarray(cat[:, k]) for k in range(4)]
        cell = _i32(cell_rock)
        rt = RockTablesStruct(len(arrs), _p(pos), *(_p(c) for c in cols), _p(cell),
                              1 if use_jfunction_scaling else 0, float(sigma_cos_theta))
        self._check(lib().porsol_transport_set_rock_tables(self.h, C.byref(rt)))

    def capillary_solve(self, pressure: "PressureSolver", sat, outflux, bc_type, bc_value, injection=None,
                        grav=(0.0, 0.0, 0.0), opts=None):
        """ImplicitCapillarity::transportSolve: returns (new saturation, CapillaryStats)."""
        s = _f64(sat).copy()
        st = CapillaryStats()
        o = opts if opts is not None else default_capillary_opts()
        inj = None if injection is None else _f64(injection)
        self._check(lib().porsol_capillary_solve(self.h, pressure.h, _p(s), _p(_f64(grav)), _p(_f64(outflux)),
                                                 _p(inj), _p(_i32(bc_type)), _p(_f64(bc_value)), C.byref(o),
                                                 C.byref(st)))
        return s, st
