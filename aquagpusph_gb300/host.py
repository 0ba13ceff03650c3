"""Python binding of the host runtime (``libaqua_host.so``,
``include/aqua_host.h``): a registry of named host Variables and the loader
of installable tools, which opens a tool library and builds the tool with its
``create_object(name, once)`` factory the way the reference's CalcServer does
for ``<Tool type="installable" path=...>`` (CalcServer.cpp:375-398).

``libaqua_cuda_tool.so`` is such a tool: one canonical WCSPH step on the GPU
through the C ABI on the registry's host Variables.

    rt = HostRuntime()
    arrays = rt.set_case(case)            # registers Variables and Definitions
    rt.add_installable("aqua cuda step")  # libaqua_cuda_tool.so by default
    rt.setup()
    rt.run(10)                            # arrays now hold the state after 10 steps
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HOST_LIB = _build.HOST_LIB
TOOL_LIB = _build.TOOL_LIB


class HostError(RuntimeError):
    pass


_SIGS = (
    ("aqua_host_set_variable", C.c_int, [C.c_char_p, C.c_char_p, C.c_void_p,
                                          C.c_size_t]),
    ("aqua_host_add_installable", C.c_int, [C.c_char_p, C.c_char_p, C.c_int]),
    ("aqua_host_setup", C.c_int, []),
    ("aqua_host_run", C.c_int, [C.c_uint32]),
    ("aqua_host_clear", None, []),
    ("aqua_host_tool_count", C.c_uint32, []),
    ("aqua_host_last_error", C.c_char_p, []),
)


def load(path: str = HOST_LIB):
    if not os.path.exists(path):
        raise HostError(f"{path} is missing: run aquagpusph_gb300.build first")
    lib = C.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class HostRuntime:
    """The process-wide host runtime (one simulation at a time)."""

    def __init__(self, path: str = HOST_LIB):
        self.lib = load(path)
        self._keep = {}
        self._types = {}

    def _check(self, what, status):
        if status != 0:
            raise HostError(f"{what}: {self.lib.aqua_host_last_error().decode()}")

    def set_variable(self, name: str, vtype: str, value) -> np.ndarray:
        """Registers `value` (copied to a contiguous array kept alive here)
        as the Variable `name` of reference type `vtype`; returns the array
        the runtime reads and writes."""
        a = np.ascontiguousarray(value)
        self._keep[name] = a
        self._types[name] = vtype
        self._check(f"set_variable {name}", self.lib.aqua_host_set_variable(
            name.encode(), vtype.encode(), a.ctypes.data_as(C.c_void_p),
            a.nbytes))
        return a

    def add_installable(self, name: str, path: str = TOOL_LIB,
                        once: bool = False):
        self._check(f"add_installable {name}",
                    self.lib.aqua_host_add_installable(name.encode(),
                                                       path.encode(), int(once)))

    def setup(self):
        self._check("setup", self.lib.aqua_host_setup())

    def run(self, steps: int = 1):
        self._check("run", self.lib.aqua_host_run(int(steps)))

    def tool_count(self) -> int:
        return int(self.lib.aqua_host_tool_count())

    def variables(self) -> dict:
        """name -> (type, array) of every registered Variable."""
        return {k: (self._types[k], a) for k, a in self._keep.items()}

    def clear(self):
        self.lib.aqua_host_clear()
        self._keep.clear()
        self._types.clear()

    def set_case(self, case, precision: int | None = None) -> dict:
        """Registers the case's Variables and Definitions under the names
        the step tool reads; returns the per-particle and scalar arrays."""
        p = case.params
        vs = 4 if p.dims == 3 else 2
        f32 = lambda x: np.asarray(x, np.float32)
        vec = lambda x: f32((list(x) + [0.0] * 4)[:vs])
        sv = self.set_variable
        sv("dims", "int", np.int32(p.dims).reshape(1))
        sv("n_sets", "unsigned int", np.uint32(len(p.refd)).reshape(1))
        for name in ("h", "support", "cs", "p0", "courant", "dt_Ma", "dt_min",
                     "relax_midpoint"):
            sv(name, "float", f32([getattr(p, name)]))
        sv("dt_fixed", "float", f32([p.dt_fixed]))
        # compiled Definitions (CalcServer.cpp:247-257 bakes them in)
        for name in ("H", "CONW", "CONF", "SUPPORT", "DIMS"):
            sv(name, "float", f32([getattr(p, name)]))
        sv("__DR_FACTOR__", "float", f32([p.dr_factor]))
        sv("__MIN_BOUND_DIST__", "float", f32([p.min_bound_dist]))
        sv("iter_midpoint_max", "unsigned int", np.uint32(p.iter_midpoint_max).reshape(1))
        for name in ("g", "domain_min", "domain_max"):
            sv(name, "vec", vec(getattr(p, name)))
        for name in ("refd", "visc_dyn", "delta"):
            sv(name, "float*", f32(getattr(p, name)))
        sv("boundary", "int", np.int32(getattr(p, "boundary", 0)).reshape(1))
        sv("scheme", "int", np.int32(getattr(p, "scheme", 0)).reshape(1))
        if precision is not None:
            sv("aqua_precision", "int", np.int32(precision).reshape(1))
        out = {}
        out["N"] = sv("N", "unsigned int", np.uint32(case.N).reshape(1))
        out["t"] = sv("t", "float", f32([case.t]))
        out["dt"] = sv("dt", "float", f32([case.dt]))
        out["iter"] = sv("iter", "unsigned int", np.uint32(case.iter).reshape(1))
        types = {"id": "unsigned int*", "iset": "unsigned int*", "imove": "int*",
                 "r": "vec*", "normal": "vec*", "tangent": "vec*",
                 "binormal": "vec*", "u": "vec*", "dudt": "vec*",
                 "rho": "float*", "drhodt": "float*", "m": "float*",
                 "p": "float*"}
        for name, vt in types.items():
            out[name] = sv(name, vt, getattr(case, name).copy())
        out["shepard"] = sv("shepard", "float*", np.zeros(case.N, np.float32))
        return out
