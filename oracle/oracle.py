"""ctypes front end of the CPU oracles (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, and only to check or to time against; the
product (``aquagpusph_gb300``) never imports it.

Two libraries share one C interface (``oracle/aqua_oracle.h``):

* ``liboracle.so`` -- the restatement of the reference pipeline
  (``oracle/aqua_oracle.cpp``), built on every host by ``make -C oracle``;
* ``_ref/libaqua_ref{2,3}d.so`` -- the reference's own OpenCL kernel sources
  compiled as C++ (``make -C oracle ref``, only where the reference tree is
  mounted).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

AQ_OK = 0
AQ_ERR_INVALID = -1
AQ_ERR_CAPACITY = -2
AQ_ERR_DT = -3

_F = C.POINTER(C.c_float)
_U = C.POINTER(C.c_uint32)
_I = C.POINTER(C.c_int32)


class AqParams(C.Structure):
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
        ("roll_enabled", C.c_int32), ("roll_iset", C.c_uint32),
        ("roll_amplitude", C.c_float), ("roll_angular_freq", C.c_float),
        ("roll_center", C.c_float * 4),
    ]


STATE_U32 = ("id", "iset")
STATE_I32 = ("imove",)
STATE_VEC = ("r", "normal", "tangent", "binormal", "u", "dudt")
STATE_F32 = ("rho", "drhodt", "m", "p")
BACKUP_U32 = ("id_in", "iset_in")
BACKUP_I32 = ("imove_in",)
BACKUP_VEC = ("r_in", "normal_in", "tangent_in", "u_in", "dudt_in")
BACKUP_F32 = ("rho_in", "drhodt_in", "m_in")
INTER_VEC = ("grad_p", "lap_u")
INTER_F32 = ("div_u", "shepard", "lap_p")
INTER_VEC2 = ("grad_w_bi",)
INTER_F32B = ("div_u_bi", "dt_var")
LL_U32 = ("icell", "id_sorted", "id_unsorted", "ihoc")


class AqState(C.Structure):
    _fields_ = ([("N", C.c_uint32), ("ihoc_capacity", C.c_uint32)] +
                [(n, _U) for n in STATE_U32] + [(n, _I) for n in STATE_I32] +
                [(n, _F) for n in STATE_VEC + STATE_F32] +
                [(n, _U) for n in BACKUP_U32] + [(n, _I) for n in BACKUP_I32] +
                [(n, _F) for n in BACKUP_VEC + BACKUP_F32] +
                [(n, _F) for n in INTER_VEC + INTER_F32 + INTER_VEC2 +
                 INTER_F32B] +
                [(n, _U) for n in LL_U32] +
                [("r_min", C.c_float * 4), ("r_max", C.c_float * 4),
                 ("n_cells", C.c_uint32 * 4), ("t", C.c_float),
                 ("dt", C.c_float), ("iter", C.c_uint32)])


def make_params(p, motion=None) -> tuple:
    """AqParams from a :class:`aquagpusph_gb300.case.Params` (and an optional
    :class:`aquagpusph_gb300.case.Motion`); returns the structure and the
    arrays it points into (keep them alive)."""
    keep = [np.ascontiguousarray(np.asarray(a, np.float32))
            for a in (p.refd, p.visc_dyn, p.delta)]
    s = AqParams()
    s.dims = p.dims
    s.n_sets = p.n_sets
    s.h = p.h
    s.support = p.support
    s.H, s.CONW, s.CONF = p.H, p.CONW, p.CONF
    s.SUPPORT, s.DIMS = p.SUPPORT, p.DIMS
    s.cs, s.p0 = p.cs, p.p0
    s.g[:] = list(p.g)[:4] + [0.0] * (4 - len(p.g))
    s.courant, s.dt_Ma, s.dt_min = p.courant, p.dt_Ma, p.dt_min
    s.dt_fixed = p.dt_fixed
    s.domain_min[:] = list(p.domain_min)[:4] + [0.0] * (4 - len(p.domain_min))
    s.domain_max[:] = list(p.domain_max)[:4] + [0.0] * (4 - len(p.domain_max))
    s.dr_factor, s.min_bound_dist = p.dr_factor, p.min_bound_dist
    s.relax_midpoint = p.relax_midpoint
    s.iter_midpoint_max = p.iter_midpoint_max
    s.refd, s.visc_dyn, s.delta = (a.ctypes.data_as(_F) for a in keep)
    s.boundary = int(getattr(p, "boundary", 0))
    s.scheme = int(getattr(p, "scheme", 0))
    if motion is not None:
        s.roll_enabled = 1
        s.roll_iset = motion.iset
        s.roll_amplitude = motion.amplitude
        s.roll_angular_freq = motion.angular_freq
        s.roll_center[:] = (list(motion.center) + [0.0] * 4)[:4]
    return s, keep


class OracleState:
    """All Variables one step reads and writes, as numpy arrays."""

    def __init__(self, case, ihoc_capacity=None):
        n, vs = case.N, case.vs
        self.case = case
        self.arrays = {}
        for name in STATE_U32:
            self.arrays[name] = np.array(getattr(case, name), np.uint32)
        self.arrays["imove"] = np.array(case.imove, np.int32)
        for name in STATE_VEC:
            self.arrays[name] = np.array(getattr(case, name), np.float32)
        for name in STATE_F32:
            self.arrays[name] = np.array(getattr(case, name), np.float32)
        for name in BACKUP_U32 + LL_U32[:3]:
            self.arrays[name] = np.zeros(n, np.uint32)
        self.arrays["imove_in"] = np.zeros(n, np.int32)
        for name in BACKUP_VEC + INTER_VEC + INTER_VEC2:
            self.arrays[name] = np.zeros((n, vs), np.float32)
        for name in BACKUP_F32 + INTER_F32 + INTER_F32B:
            self.arrays[name] = np.zeros(n, np.float32)
        cap = ihoc_capacity or case.params.max_cells()
        self.arrays["ihoc"] = np.zeros(cap, np.uint32)
        self.s = AqState()
        self.s.N = n
        self.s.ihoc_capacity = cap
        for name, a in self.arrays.items():
            ptr = _I if a.dtype == np.int32 else (_U if a.dtype == np.uint32 else _F)
            setattr(self.s, name, a.ctypes.data_as(ptr))
        self.s.t = case.t
        self.s.dt = case.dt
        self.s.iter = case.iter

    def __getitem__(self, name):
        if name == "ihoc":
            return self.arrays["ihoc"][: self.s.n_cells[3]]
        if name in ("t", "dt", "iter"):
            return getattr(self.s, name)
        if name in ("r_min", "r_max", "n_cells"):
            return np.array(getattr(self.s, name)[:])
        return self.arrays[name]

    def to_case(self):
        c = self.case.copy()
        for name in c.state_arrays():
            getattr(c, name)[...] = self.arrays[name]
        c.t, c.dt, c.iter = self.s.t, self.s.dt, self.s.iter
        return c


class Oracle:
    """One of the oracle libraries."""

    def __init__(self, path):
        self.path = path
        self.lib = C.CDLL(path)
        for fn in ("aq_step", "aq_linklist"):
            getattr(self.lib, fn).argtypes = [C.POINTER(AqState),
                                              C.POINTER(AqParams), C.c_int]
            getattr(self.lib, fn).restype = C.c_int
        self.lib.aq_sort.argtypes = [_U, _U, _U, C.c_uint32]
        self.lib.aq_sort.restype = C.c_int

    def step(self, st: OracleState, nthreads=0, steps=1, motion=None):
        p, keep = make_params(st.case.params, motion)
        for _ in range(steps):
            err = self.lib.aq_step(C.byref(st.s), C.byref(p), nthreads)
            if err:
                raise RuntimeError(f"{os.path.basename(self.path)}: aq_step failed ({err})")
        return st

    def linklist(self, st: OracleState, nthreads=0):
        p, keep = make_params(st.case.params)
        err = self.lib.aq_linklist(C.byref(st.s), C.byref(p), nthreads)
        if err:
            raise RuntimeError(f"aq_linklist failed ({err})")
        return st

    def sort(self, keys):
        k = np.array(keys, np.uint32)
        perm = np.zeros(len(k), np.uint32)
        inv = np.zeros(len(k), np.uint32)
        self.lib.aq_sort(k.ctypes.data_as(_U), perm.ctypes.data_as(_U),
                         inv.ctypes.data_as(_U), len(k))
        return k, perm, inv


def oracle_path():
    return os.path.join(HERE, "liboracle.so")


def ref_path(dims):
    return os.path.join(HERE, "_ref", f"libaqua_ref{dims}d.so")


def load_oracle(build=True) -> Oracle:
    path = oracle_path()
    if not os.path.exists(path) and build:
        build_oracle()
    return Oracle(path)


def load_ref(dims):
    """The reference-kernel harness, or None where it was not built."""
    path = ref_path(dims)
    return Oracle(path) if os.path.exists(path) else None


def reference_dir():
    """The reference source tree (sanguinariojoe/aquagpusph), from the
    AQUA_REFERENCE_DIR environment variable; None when it is unset or does
    not name a directory (the tests that read the tree then skip)."""
    d = os.environ.get("AQUA_REFERENCE_DIR")
    return d if d and os.path.isdir(d) else None


def build_oracle(ref=False):
    import subprocess
    targets = ["all"]
    extra = []
    if ref:
        d = reference_dir()
        if d is None:
            raise RuntimeError("the reference-kernel harness needs the "
                               "reference tree: set AQUA_REFERENCE_DIR")
        targets.append("ref")
        extra = [f"REF={d}"]
    subprocess.run(["make", "-s", "-C", HERE] + targets + extra, check=True)


def free_surface(st: OracleState, sensors, dr: float, dims: int):
    """Wave-height sensors restated on the oracle's state
    (examples/3D/spheric_testcase2_dambreak/src/templates/h_sensor.cl:37-61
    and the max reductions of Sensors.xml:43-62): h_i = r_i[up] + dr/2 for
    fluid particles within 2 dr of the sensor horizontally, 0 otherwise;
    H = max_i h_i.  ``sensors``: x (2-D) or (x, y) (3-D) per sensor."""
    r = st["r"]
    fluid = st["imove"] > 0
    dr = np.float32(dr)
    two = np.float32(2.0) * dr
    out = []
    for s in sensors:
        s = np.atleast_1d(np.asarray(s, np.float32))
        far = np.abs(r[:, 0] - s[0]) > two
        if dims == 3:
            far |= np.abs(r[:, 1] - s[1]) > two
        h = np.where(fluid & ~far, r[:, dims - 1] + np.float32(0.5) * dr,
                     np.float32(0.0)).astype(np.float32)
        out.append(np.float32(h.max()) if len(h) else np.float32(-np.inf))
    return np.array(out, np.float32)


def probe_values(st: OracleState, field: str, first: int, n: int):
    """Values of ``field`` for the particles of original index
    [first, first + n), in original order (the oracle keeps its state sorted
    by cell, like the reference)."""
    pos = np.empty(n, np.int64)
    ids = st["id"]
    sel = np.nonzero((ids >= first) & (ids < first + n))[0]
    pos[ids[sel] - first] = sel
    return st[field][pos]
