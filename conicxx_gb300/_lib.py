"""ctypes binding of libconicxx_gb300.so (the C-ABI in include/conicxx_gb300.h).

The library is built in-tree by __graft_entry__.build() (conicxx_gb300/csrc/Makefile). There is
no Python or CPU fallback: if the library is missing, importing the solver classes fails.
"""
import ctypes as C
import os
import re

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libconicxx_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "conicxx_gb300.h")

_lib = None

vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)
SP, IP, PP = C.POINTER(_abi.Settings), C.POINTER(_abi.Info), C.POINTER(_abi.Problem)

# name -> (restype, argtypes)
SIGNATURES = {
    "cxg_default_settings": (None, [SP]),
    "cxg_status_string": (C.c_char_p, [C.c_int]),
    "cxg_version": (C.c_char_p, []),
    "cxg_last_error": (C.c_char_p, []),
    "cxg_device_count": (C.c_int, []),
    "cxg_solver_create": (C.c_int, [C.POINTER(vp)]),
    "cxg_solver_destroy": (None, [vp]),
    "cxg_solver_setup": (C.c_int, [vp, PP, SP]),
    "cxg_solver_update_data": (C.c_int, [vp, ip, ip, dp, dp, ip, ip, dp, dp]),
    "cxg_solver_set_warm_start": (C.c_int, [vp, dp, dp, dp]),
    "cxg_solver_set_settings": (C.c_int, [vp, SP]),
    "cxg_solver_get_settings": (C.c_int, [vp, SP]),
    "cxg_solver_solve": (C.c_int, [vp, dp, dp, dp, IP]),
    "cxg_solver_backward": (C.c_int, [vp, dp, dp, dp, dp, dp]),
    "cxg_batch_create": (C.c_int, [C.POINTER(vp), C.c_int, PP, SP]),
    "cxg_batch_destroy": (None, [vp]),
    "cxg_batch_count": (C.c_int, [vp]),
    "cxg_batch_sizes": (C.c_int, [vp, i64p, i64p, i64p, i64p]),
    "cxg_batch_offsets": (C.c_int, [vp, C.c_int, i64p, i64p, i64p, i64p]),
    "cxg_batch_update_values": (C.c_int, [vp, dp, dp, dp, dp]),
    "cxg_batch_replace": (C.c_int, [vp, C.c_int, ip, PP]),
    "cxg_batch_solve": (C.c_int, [vp, dp, dp, dp, IP]),
    "cxg_batch_update_values_device": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "cxg_batch_solve_device": (C.c_int, [vp, vp, vp, vp, IP, vp]),
    "cxg_batch_solve_device_noalloc": (C.c_int, [vp, vp, vp, vp, IP, vp]),
    "cxg_batch_autotune": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int]),
    "cxg_dense_ldlt": (C.c_int, [C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]),
    "cxg_grid_barrier_selftest": (C.c_int, [C.c_int, C.c_int, C.c_double, vp, vp, vp]),
    "cxg_batch_backward": (C.c_int, [vp, dp, dp, dp, dp, dp]),
    "cxg_batch_backward_device": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "cxg_batch_last_launches": (C.c_int, [vp]),
    "cxg_batch_trace": (C.c_int, [vp, C.c_int, dp, C.c_int]),
    "cxg_solver_trace": (C.c_int, [vp, dp, C.c_int]),
    "cxg_batch_describe": (C.c_int, [vp, C.c_char_p, C.c_int]),
    "cxg_batch_footprint": (C.c_int, [vp, i64p, i64p, i64p]),
    "cxg_cones_eval": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, ip, dp, dp, dp, dp, C.c_double, dp, dp, dp]),
    "cxg_equilibration": (C.c_int, [PP, SP, dp, dp, dp]),
    "cxg_plan_inspect": (C.c_int, [PP, SP, i64p, i64p, i64p, i64p, C.c_int]),
}


def header_symbols(path=HEADER):
    """Every function the public header declares (the C-ABI surface)."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cxg_[a-z0-9_]+)\s*\(", text)))


class LibraryMissing(ImportError):
    pass


def lib():
    """The loaded library (raises LibraryMissing if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class CxgError(RuntimeError):
    def __init__(self, code, where):
        msg = lib().cxg_last_error().decode(errors="replace")
        super().__init__(f"{where} failed ({code}): {msg}")
        self.code = code


def check(code, where):
    if code != _abi.OK:
        raise CxgError(code, where)
    return code
