"""ctypes binding of libgridoxide_gb300.so (the C ABI in include/gridoxide_gb300.h).

There is no fallback: if the library is missing or a CUDA call fails, the
call raises.  ``load()`` builds the library in-tree first when it is absent.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgridoxide_gb300.so")

GOX_OK = 0
GOX_SINGULAR = 1
GOX_PENDING = 2
GOX_ISLAND_SOLVABLE, GOX_ISLAND_NO_REFERENCE, GOX_ISLAND_AMBIGUOUS = 0, 1, 2
GOX_GUESS_GIVEN = 0
GOX_GUESS_LINEAR = 1
GOX_E_OUT_OF_MEMORY = -2
GOX_E_INVALID = -3
GOX_E_BUS_RANGE = -4
GOX_E_CUDA = -5
GOX_E_PATTERN = -6
GOX_E_NO_DEVICE = -7
GOX_E_TOO_LARGE = -8
GOX_E_DEVICE_WAIT = -9

GOX_CONVERGED = 0
GOX_MAX_ITERATIONS = 1
GOX_SINGULAR_SCENARIO = 2

GOX_PRECISION_FP64 = 0
GOX_PRECISION_MIXED = 1

ERRORS = {
    GOX_E_OUT_OF_MEMORY: "out of memory",
    GOX_E_INVALID: "invalid argument",
    GOX_E_BUS_RANGE: "outage slot outside the Y-bus",
    GOX_E_CUDA: "CUDA runtime error",
    GOX_E_PATTERN: "values given for a different pattern",
    GOX_E_NO_DEVICE: "no CUDA device visible",
    GOX_E_TOO_LARGE: "request exceeds a size limit",
    GOX_E_DEVICE_WAIT: "a bounded device wait gave up",
}


class GoxError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, code)} ({code})")


i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
vp = C.c_void_p
vpp = C.POINTER(C.c_void_p)

# name -> (restype, argtypes); every symbol include/gridoxide_gb300.h declares
SIGNATURES = {
    "gox_ls_create": (C.c_int, [C.c_int32, C.c_int32, i32p, i32p, f64p, C.POINTER(vp)]),
    "gox_ls_factor_solve_values": (C.c_int, [vp, f64p, f64p, f64p]),
    "gox_ls_factor_solve": (C.c_int, [vp, C.c_int32, i32p, i32p, f64p, f64p, f64p]),
    "gox_ls_destroy": (None, [vp]),
    "gox_ls_factor_solve_values_static": (C.c_int, [vp, f64p, f64p, f64p]),
    "gox_topo_register": (C.c_int, [C.c_int32, i32p, i32p, f64p, f64p, i32p, C.POINTER(vp)]),
    "gox_topo_reset": (C.c_int, [vp]),
    "gox_topo_destroy": (None, [vp]),
    "gox_batch_solve": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, C.c_int32, i32p, f64p,
                                  f64p, C.c_double, C.c_int32, C.c_int32, f64p, f64p, i32p, i32p,
                                  f64p, f64p]),
    "gox_outage_islands": (C.c_int, [vp, C.c_int32, i32p, f64p, f64p, i32p, i32p, i32p]),
    "gox_batch_solve_qlim": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, C.c_int32, f64p, f64p,
                                       C.c_double, C.c_int32, C.c_int32, C.c_int32, f64p, f64p, i32p,
                                       i32p, f64p, i32p, C.POINTER(C.c_uint8), i32p]),
    "gox_set_multi_persistent": (C.c_int, [C.c_int32]),
    "gox_multi_solve": (C.c_int, [C.c_int32, vpp, i32p, vpp, vpp, vpp, vpp, i32p, C.c_double,
                                  C.c_int32, C.c_int32, vpp, vpp, vpp, vpp, vpp]),
    "gox_batch_solve_scaled": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, f64p, C.c_double,
                                         C.c_int32, C.c_int32, f64p, f64p, i32p, i32p, f64p,
                                         f64p]),
    "gox_batch_solve_device": (C.c_int, [vp, C.c_int32, vp, vp, vp, vp, C.c_int32, vp, vp, vp,
                                         C.c_double, C.c_int32, C.c_int32, vp, vp, vp, vp, vp,
                                         vp, vp]),
    "gox_analyze": (C.c_int, [C.c_int32, i32p, i32p, i32p, i32p, i32p]),
    "gox_factor_host": (C.c_int, [C.c_int32, C.c_int32, i32p, i32p, f64p, i64p, i32p, i32p, f64p,
                                  i32p, i32p, f64p, i32p, i32p, f64p, i32p, i32p, i32p]),
    "gox_topo_prepare": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, C.c_int32, i32p, f64p,
                                   f64p, C.c_double]),
    "gox_topo_emulate_step": (C.c_int, [vp, f64p, f64p, f64p]),
    "gox_topo_factor_values": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, C.c_int32, f64p,
                                         f64p]),
    "gox_topo_pivot_solve": (C.c_int, [vp, f64p, f64p, f64p]),
    "gox_set_autotune": (C.c_int, [C.c_int32]),
    "gox_set_refactor_sync": (C.c_int, [C.c_int32]),
    "gox_set_refactor_wide": (C.c_int, [C.c_int32]),
    "gox_topo_tuning": (C.c_int, [vp, C.c_int32, i64p, f64p, C.c_int32]),
    "gox_topo_stream_word": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, i32p]),
    "gox_topo_info": (C.c_int, [vp, i64p]),
    "gox_topo_structure": (C.c_int, [vp, i32p, i32p, i32p, i32p, i32p, i32p, i32p, f64p]),
    "gox_topo_jacobian_pattern": (C.c_int, [vp, i32p, i32p]),
    "gox_set_timing": (C.c_int, [vp, C.c_int32]),
    "gox_last_timing": (C.c_int, [vp, f64p]),
    "gox_last_launches": (C.c_int64, [vp]),
    "gox_topo_repacks": (C.c_int64, [vp]),
    "gox_set_repack": (C.c_int, [C.c_int32]),
    "gox_set_pivot_tolerance": (C.c_int, [vp, C.c_double]),
    "gox_topo_set_initial_guess": (C.c_int, [vp, C.c_int32]),
    "gox_topo_set_graph": (C.c_int, [vp, C.c_int32]),
    "gox_topo_set_split": (C.c_int, [vp, C.c_int32]),
    "gox_topo_initial_guess": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, C.c_int32, f64p,
                                         f64p]),
    "gox_topo_set_zip": (C.c_int, [vp, f64p, f64p, f64p, f64p]),
    "gox_last_fallbacks": (C.c_int64, [vp]),
    "gox_version": (C.c_char_p, []),
    "gox_server_create": (C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(vp)]),
    "gox_server_add_topology": (C.c_int, [vp, vp, i32p]),
    "gox_server_submit": (C.c_int, [vp, C.c_int32, f64p, f64p, f64p, f64p, i32p, f64p, f64p, i64p]),
    "gox_server_poll": (C.c_int, [vp, C.c_int64, f64p, f64p, i32p, i32p, f64p, f64p]),
    "gox_server_submit_many": (C.c_int, [vp, C.c_int32, i32p, vpp, vpp, vpp, vpp, vpp, vpp, vpp,
                                         i64p]),
    "gox_server_set_budget": (C.c_int, [vp, C.c_int64]),
    "gox_server_set_lanes": (C.c_int, [vp, C.c_int32]),
    "gox_server_stats": (C.c_int, [vp, i64p]),
    "gox_server_destroy": (None, [vp]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Returns the loaded library (building it in-tree if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run gridoxide_gb300.build.build()")
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code: int, what: str) -> int:
    if code < 0:
        raise GoxError(code, what)
    return code
