"""ctypes binding of ``libaqua_gb300.so`` (the C ABI in include/aqua_gb300.h).

The library is the only compute path of this package: importing the binding
raises if the shared object is missing or does not export the declared
entry points; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaqua_gb300.so")

AQUA_OK = 0
AQUA_ERR_INVALID = -1
AQUA_ERR_CAPACITY = -2
AQUA_ERR_DT = -3
AQUA_ERR_CUDA = -4
AQUA_ERR_NO_MEMORY = -5
AQUA_ERR_NONFINITE = -6
AQUA_ERR_IO = -7
AQUA_ERR_FORMAT = -8
AQUA_ERR_TIMEOUT = -9

AQUA_PRECISION_EXACT = 0
AQUA_PRECISION_FAST = 1
AQUA_NOALLOC_SORT_MAX_KEYS = 1 << 20
AQUA_REPORT_MAX_VALUES = 1 << 20

# fields of aqua_get_unsorted: name -> (code, vector?)
FIELDS = {"r": (0, True), "normal": (1, True), "tangent": (2, True),
          "u": (3, True), "dudt": (4, True), "rho": (5, False),
          "drhodt": (6, False), "m": (7, False), "p": (8, False),
          "shepard": (9, False), "imove": (10, False)}
AQUA_COLUMN_FLOAT = 0
AQUA_COLUMN_INT = 1
AQUA_COLUMN_UINT = 2

STATUS_NAMES = {
    AQUA_OK: "AQUA_OK",
    AQUA_ERR_INVALID: "AQUA_ERR_INVALID",
    AQUA_ERR_CAPACITY: "AQUA_ERR_CAPACITY",
    AQUA_ERR_DT: "AQUA_ERR_DT",
    AQUA_ERR_CUDA: "AQUA_ERR_CUDA",
    AQUA_ERR_NO_MEMORY: "AQUA_ERR_NO_MEMORY",
    AQUA_ERR_NONFINITE: "AQUA_ERR_NONFINITE",
    AQUA_ERR_IO: "AQUA_ERR_IO",
    AQUA_ERR_FORMAT: "AQUA_ERR_FORMAT",
    AQUA_ERR_TIMEOUT: "AQUA_ERR_TIMEOUT",
}

_F = C.POINTER(C.c_float)
_U = C.POINTER(C.c_uint32)
_I = C.POINTER(C.c_int32)


class AquaError(RuntimeError):
    def __init__(self, fn, status):
        super().__init__(f"{fn} returned {STATUS_NAMES.get(status, status)}")
        self.status = status


class AquaParams(C.Structure):
    _fields_ = [
        ("dims", C.c_int32), ("n_sets", C.c_uint32),
        ("h", C.c_float), ("support", C.c_float),
        ("H", C.c_float), ("CONW", C.c_float), ("CONF", C.c_float),
        ("SUPPORT", C.c_float), ("DIMS", C.c_float),
        ("cs", C.c_float), ("p0", C.c_float), ("g", C.c_float * 4),
        ("courant", C.c_float), ("dt_Ma", C.c_float), ("dt_min", C.c_float),
        ("dt_fixed", C.c_float),
        ("domain_min", C.c_float * 4), ("domain_max", C.c_float * 4),
        ("dr_factor", C.c_float), ("min_bound_dist", C.c_float),
        ("relax_midpoint", C.c_float), ("iter_midpoint_max", C.c_uint32),
        ("refd", _F), ("visc_dyn", _F), ("delta", _F),
        ("boundary", C.c_int32), ("scheme", C.c_int32),
    ]


VARS_FIELDS = (("id", _U), ("iset", _U), ("imove", _I), ("r", _F),
               ("normal", _F), ("tangent", _F), ("binormal", _F), ("u", _F),
               ("dudt", _F), ("rho", _F), ("drhodt", _F), ("m", _F), ("p", _F),
               ("shepard", _F))
EXTRA_FIELDS = (("r_in", _F), ("u_in", _F), ("dudt_in", _F), ("rho_in", _F),
                ("drhodt_in", _F), ("icell", _U), ("id_sorted", _U),
                ("id_unsorted", _U), ("ihoc", _U), ("grad_p", _F),
                ("lap_u", _F), ("div_u", _F), ("lap_p", _F),
                ("grad_w_bi", _F), ("div_u_bi", _F))


class AquaVars(C.Structure):
    _fields_ = list(VARS_FIELDS)


class AquaExtra(C.Structure):
    _fields_ = list(EXTRA_FIELDS)


class AquaCase(C.Structure):
    _fields_ = [("t", C.c_float), ("dt", C.c_float), ("iter", C.c_uint32),
                ("roll_enabled", C.c_int32), ("roll_iset", C.c_uint32),
                ("roll_amplitude", C.c_float), ("roll_angular_freq", C.c_float),
                ("roll_center", C.c_float * 4)]


class AquaScalars(C.Structure):
    _fields_ = [("t", C.c_float), ("dt", C.c_float), ("iter", C.c_uint32),
                ("n_cells", C.c_uint32 * 4), ("r_min", C.c_float * 4),
                ("r_max", C.c_float * 4)]


# (name, restype, argtypes) of every function include/aqua_gb300.h declares
SIGNATURES = [
    ("aqua_version", C.c_char_p, []),
    ("aqua_malloc", C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    ("aqua_free", C.c_int, [C.c_void_p]),
    ("aqua_memcpy", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]),
    ("aqua_create", C.c_int, [C.POINTER(AquaParams), C.c_uint32, C.c_uint32,
                              C.POINTER(C.c_void_p)]),
    ("aqua_destroy", C.c_int, [C.c_void_p]),
    ("aqua_set_params", C.c_int, [C.c_void_p, C.POINTER(AquaParams)]),
    ("aqua_set_extras", C.c_int, [C.c_void_p, C.c_int]),
    ("aqua_set_precision", C.c_int, [C.c_void_p, C.c_int]),
    ("aqua_set_tuning", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    ("aqua_set_state", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(AquaVars),
                                 C.c_int, C.c_float, C.c_float, C.c_uint32,
                                 C.c_void_p]),
    ("aqua_get_state", C.c_int, [C.c_void_p, C.POINTER(AquaVars), C.c_int,
                                 C.c_void_p]),
    ("aqua_set_cases", C.c_int, [C.c_void_p, C.c_uint32, _U,
                                 C.POINTER(AquaCase), C.c_void_p]),
    ("aqua_get_case_scalars", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32,
                                        C.POINTER(AquaScalars), C.c_void_p]),
    ("aqua_get_extra", C.c_int, [C.c_void_p, C.POINTER(AquaExtra), C.c_int,
                                 C.c_void_p]),
    ("aqua_get_scalars", C.c_int, [C.c_void_p, C.POINTER(AquaScalars),
                                   C.c_void_p]),
    ("aqua_step", C.c_int, [C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]),
    ("aqua_check", C.c_int, [C.c_void_p, C.c_void_p]),
    ("aqua_linklist", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                _U, _F, _F, C.c_void_p]),
    ("aqua_radix_sort", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_uint32, C.c_uint32,
                                  C.c_void_p]),
    ("aqua_set_rate_sample", C.c_int, [C.c_void_p, C.c_float, C.c_uint32]),
    ("aqua_debug_fake_timeouts", C.c_int, [C.c_int]),
    ("aqua_radix_sort_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_uint32, C.c_uint32, C.c_void_p]),
    ("aqua_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("aqua_stage_times", C.c_int, [C.c_void_p, _F, C.c_uint32]),
    ("aqua_launches_per_step", C.c_uint32, [C.c_void_p]),
    ("aqua_get_unsorted", C.c_int, [C.c_void_p, C.c_int, C.c_uint32,
                                    C.c_uint32, C.c_void_p, C.c_int,
                                    C.c_void_p]),
    ("aqua_free_surface", C.c_int, [C.c_void_p, _F, C.c_uint32, C.c_float,
                                    C.c_int32, _F, C.c_void_p]),
    ("aqua_read_fastascii", C.c_int, [C.c_char_p, C.c_uint32, _I, C.c_void_p,
                                      C.c_uint64, C.POINTER(C.c_uint64),
                                      C.POINTER(C.c_uint64)]),
]

_lib = None


def load(path: str = LIB_PATH):
    """Loads the library (once) and binds the declared signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m aquagpusph_gb300.build`"
            " (there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, status: int):
    if status != AQUA_OK:
        raise AquaError(fn, status)


def params_struct(p) -> tuple:
    """AquaParams from a :class:`aquagpusph_gb300.case.Params` (returns the
    structure and the arrays it points into)."""
    keep = [np.ascontiguousarray(np.asarray(a, np.float32))
            for a in (p.refd, p.visc_dyn, p.delta)]
    s = AquaParams()
    s.dims = p.dims
    s.n_sets = p.n_sets
    s.h = p.h
    s.support = p.support
    s.H, s.CONW, s.CONF = p.H, p.CONW, p.CONF
    s.SUPPORT, s.DIMS = p.SUPPORT, p.DIMS
    s.cs, s.p0 = p.cs, p.p0
    s.g[:] = (list(p.g) + [0.0] * 4)[:4]
    s.courant, s.dt_Ma, s.dt_min = p.courant, p.dt_Ma, p.dt_min
    s.dt_fixed = p.dt_fixed
    s.domain_min[:] = (list(p.domain_min) + [0.0] * 4)[:4]
    s.domain_max[:] = (list(p.domain_max) + [0.0] * 4)[:4]
    s.dr_factor, s.min_bound_dist = p.dr_factor, p.min_bound_dist
    s.relax_midpoint = p.relax_midpoint
    s.iter_midpoint_max = p.iter_midpoint_max
    s.refd, s.visc_dyn, s.delta = (a.ctypes.data_as(_F) for a in keep)
    s.boundary = int(getattr(p, "boundary", 0))
    s.scheme = int(getattr(p, "scheme", 0))
    return s, keep
