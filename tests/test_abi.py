"""The C-ABI library loads and exports every entry point declared in include/porsol_gpu.h
(CPU only: no compute calls are made)."""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "porsol_gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(porsol_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "porsol_solve" in names and "porsol_transport_solve" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(pkg):
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    L = ctypes.CDLL(pkg.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_header(pkg):
    bound = {e[0] for e in pkg.EXPORTS}
    assert set(declared_functions()) <= bound, set(declared_functions()) - bound


def test_defaults_without_gpu(pkg):
    """Option defaults are pure host code and match the reference's defaults."""
    o = pkg.default_solve_opts()
    assert o.residual_tolerance == 1e-8 and o.linsolver_type == 1 and o.linsolver_verbosity == 1
    assert o.prolongate_factor == 1.6 and o.smooth_steps == 1 and o.same_matrix == 0 and o.linsolver_maxit == 0
    t = pkg.default_transport_opts()
    assert t.courant_number == 0.5 and t.maximum_small_steps == 10000 and t.minimum_small_steps == 1
    assert t.check_sat == 1 and t.clamp_sat == 0 and t.method_capillary == 1
