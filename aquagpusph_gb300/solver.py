"""Host-side mirror of the reference's CalcServer for the canonical WCSPH
step: one resident case on one GPU, advanced by the CUDA library.

The reference builds a CalcServer from the XML presets, registers the
particle Variables, and calls ``CalcServer::update`` (CalcServer.cpp:592-623)
to run the tool list once per step.  :class:`Solver` plays that role for the
tool list this library replaces (include/aqua_gb300.h lists it): it owns the
library context (device Variables + scratch), loads a :class:`Case`, steps
it, and reads the Variables back.  All compute goes through
``libaqua_gb300.so``; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .case import Case, Params

__all__ = ["Solver"]


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


class Solver:
    """A resident case on the current CUDA device."""

    def __init__(self, params: Params, capacity: int, ihoc_capacity: int = 0):
        self.lib = _lib.load()
        self.params = params
        self._pstruct, self._pkeep = _lib.params_struct(params)
        self.ctx = C.c_void_p()
        self.ncap = int(ihoc_capacity or params.max_cells())
        _lib.check("aqua_create", self.lib.aqua_create(
            C.byref(self._pstruct), int(capacity), self.ncap,
            C.byref(self.ctx)))
        self.capacity = int(capacity)
        self.N = 0
        self.vs = 4 if params.dims == 3 else 2

    # ------------------------------------------------------------------
    def close(self):
        if self.ctx:
            self.lib.aqua_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_extras(self, on: bool = True):
        _lib.check("aqua_set_extras", self.lib.aqua_set_extras(self.ctx, int(on)))

    def set_precision(self, fast: bool):
        """Exact (reference arithmetic, default) or fast step kernels."""
        mode = _lib.AQUA_PRECISION_FAST if fast else _lib.AQUA_PRECISION_EXACT
        _lib.check("aqua_set_precision",
                   self.lib.aqua_set_precision(self.ctx, mode))

    def set_rate_sample(self, fraction: float, seed: int = 0):
        """Steps evaluate the sums and rates only on a hashed sample of the
        cells (about `fraction` of them) and the cells around the probes
        (fast 3-D build); fraction >= 1 turns it off."""
        _lib.check("aqua_set_rate_sample", self.lib.aqua_set_rate_sample(
            self.ctx, float(fraction), int(seed) & 0xFFFFFFFF))

    def get_icell_raw(self, ptr: int, stream=None):
        """The sorted cell keys of the last step (device address, N uint32)."""
        e = _lib.AquaExtra()
        e.icell = C.cast(C.c_void_p(ptr), _lib._U)
        _lib.check("aqua_get_extra", self.lib.aqua_get_extra(
            self.ctx, C.byref(e), 0, C.c_void_p(stream or 0)))

    def set_tuning(self, sweep_variant: int, blocks_per_sm: int):
        """Launch shape of the sweep (results do not depend on it)."""
        _lib.check("aqua_set_tuning", self.lib.aqua_set_tuning(
            self.ctx, int(sweep_variant), int(blocks_per_sm)))
        self.tuning = (int(sweep_variant), int(blocks_per_sm))

    def set_params(self, params: Params):
        self.params = params
        self._pstruct, self._pkeep = _lib.params_struct(params)
        _lib.check("aqua_set_params",
                   self.lib.aqua_set_params(self.ctx, C.byref(self._pstruct)))

    # ------------------------------------------------------------------
    def vars_struct(self, arrays: dict) -> _lib.AquaVars:
        """AquaVars from a dict of host numpy arrays or raw addresses."""
        v = _lib.AquaVars()
        for name, typ in _lib.VARS_FIELDS:
            a = arrays.get(name)
            if a is None:
                continue
            addr = a if isinstance(a, int) else a.ctypes.data
            setattr(v, name, C.cast(C.c_void_p(addr), typ))
        return v

    def set_state_raw(self, n, arrays: dict, on_host: bool, t=0.0, dt=0.0,
                      it=0, stream=None):
        v = self.vars_struct(arrays)
        _lib.check("aqua_set_state", self.lib.aqua_set_state(
            self.ctx, int(n), C.byref(v), int(on_host), float(t), float(dt),
            int(it), C.c_void_p(stream or 0)))
        self.N = int(n)

    def get_state_raw(self, arrays: dict, on_host: bool, stream=None):
        v = self.vars_struct(arrays)
        _lib.check("aqua_get_state", self.lib.aqua_get_state(
            self.ctx, C.byref(v), int(on_host), C.c_void_p(stream or 0)))

    def set_case(self, case: Case, stream=None):
        arrays = {k: np.ascontiguousarray(v) for k, v in case.state_arrays().items()}
        self._host_in = arrays
        self.set_state_raw(case.N, arrays, True, case.t, case.dt, case.iter,
                           stream)
        self._case = case
        self.n_cases = 1

    def set_batch(self, batch, stream=None):
        """Loads a :class:`aquagpusph_gb300.case.Batch`: its concatenated
        particles, then the split into independent cases (aqua_set_cases)."""
        self.set_case(batch.case, stream)
        self.set_cases(batch, stream)

    def set_cases(self, batch, stream=None):
        """The case split of a Batch whose particles are already resident.
        The case records are built once per Batch and (t, dt, iter) and
        reused on later calls."""
        key = (id(batch), batch.case.t, batch.case.dt, batch.case.iter)
        cached = getattr(self, "_cases_cache", None)
        if cached is None or cached[0] != key or cached[1] is not batch:
            n = len(batch.offsets) - 1
            offs = np.ascontiguousarray(batch.offsets, np.uint32)
            arr = (_lib.AquaCase * n)()
            for k, m in enumerate(batch.motions):
                a = arr[k]
                a.t, a.dt, a.iter = batch.case.t, batch.case.dt, batch.case.iter
                if m is not None:
                    a.roll_enabled = 1
                    a.roll_iset = m.iset
                    a.roll_amplitude = m.amplitude
                    a.roll_angular_freq = m.angular_freq
                    a.roll_center[:] = (list(m.center) + [0.0] * 4)[:4]
            cached = (key, batch, n, offs, arr)
            self._cases_cache = cached
        _, _, n, offs, arr = cached
        _lib.check("aqua_set_cases", self.lib.aqua_set_cases(
            self.ctx, n, offs.ctypes.data_as(_lib._U), arr,
            C.c_void_p(stream or 0)))
        self.n_cases = n

    def case_scalars(self, stream=None) -> list:
        n = getattr(self, "n_cases", 1)
        out = (_lib.AquaScalars * n)()
        _lib.check("aqua_get_case_scalars", self.lib.aqua_get_case_scalars(
            self.ctx, 0, n, out, C.c_void_p(stream or 0)))
        return [{"t": s.t, "dt": s.dt, "iter": s.iter,
                 "n_cells": np.array(s.n_cells[:], np.uint32)} for s in out]

    def step(self, n: int = 1, graph: bool = True, stream=None):
        _lib.check("aqua_step", self.lib.aqua_step(
            self.ctx, int(n), int(graph), C.c_void_p(stream or 0)))

    def check(self, stream=None):
        _lib.check("aqua_check", self.lib.aqua_check(self.ctx,
                                                     C.c_void_p(stream or 0)))

    def scalars(self, stream=None) -> dict:
        s = _lib.AquaScalars()
        _lib.check("aqua_get_scalars", self.lib.aqua_get_scalars(
            self.ctx, C.byref(s), C.c_void_p(stream or 0)))
        return {"t": s.t, "dt": s.dt, "iter": s.iter,
                "n_cells": np.array(s.n_cells[:], np.uint32),
                "r_min": np.array(s.r_min[:], np.float32),
                "r_max": np.array(s.r_max[:], np.float32)}

    def get_case(self, stream=None) -> Case:
        """The resident Variables as a host :class:`Case` (synchronises)."""
        c = Case(self.params, self.N)
        arrays = c.state_arrays()
        arrays["shepard"] = np.zeros(self.N, np.float32)
        self.get_state_raw(arrays, True, stream)
        sc = self.scalars(stream)
        c.t, c.dt, c.iter = sc["t"], sc["dt"], sc["iter"]
        c.shepard = arrays["shepard"]
        return c

    def get_extra(self, stream=None) -> dict:
        """Backups, link-list tables and (with extras on) the intermediate
        operators of the last step, as host arrays (synchronises)."""
        n, vs = self.N, self.vs
        sc = self.scalars(stream)
        vec_names = ("r_in", "u_in", "dudt_in", "grad_p", "lap_u", "grad_w_bi")
        out = {}
        for name, typ in _lib.EXTRA_FIELDS:
            if name == "ihoc":
                out[name] = np.zeros(self.ncap, np.uint32)
            elif typ is _lib._U:
                out[name] = np.zeros(n, np.uint32)
            elif name in vec_names:
                out[name] = np.zeros((n, vs), np.float32)
            else:
                out[name] = np.zeros(n, np.float32)
        e = _lib.AquaExtra()
        for name, typ in _lib.EXTRA_FIELDS:
            setattr(e, name, C.cast(C.c_void_p(out[name].ctypes.data), typ))
        _lib.check("aqua_get_extra", self.lib.aqua_get_extra(
            self.ctx, C.byref(e), 1, C.c_void_p(stream or 0)))
        self.scalars(stream)
        out["ihoc"] = out["ihoc"][: int(sc["n_cells"][3])].copy()
        out.update({k: sc[k] for k in ("n_cells", "r_min", "r_max")})
        return out

    def linklist(self, r_in: int, n: int, icell: int, id_sorted: int,
                 id_unsorted: int, ihoc: int, ihoc_capacity: int,
                 stream=None) -> dict:
        """The link-list tool on caller device buffers (addresses)."""
        nc = (C.c_uint32 * 4)()
        mn = (C.c_float * 4)()
        mx = (C.c_float * 4)()
        _lib.check("aqua_linklist", self.lib.aqua_linklist(
            self.ctx, C.c_void_p(r_in), int(n), C.c_void_p(icell),
            C.c_void_p(id_sorted), C.c_void_p(id_unsorted), C.c_void_p(ihoc),
            int(ihoc_capacity), nc, mn, mx, C.c_void_p(stream or 0)))
        return {"n_cells": np.array(nc[:], np.uint32),
                "r_min": np.array(mn[:], np.float32),
                "r_max": np.array(mx[:], np.float32)}

    def radix_sort(self, keys: int, perm: int, inv_perm: int, n: int,
                   key_bits: int, stream=None):
        """The radix-sort tool on caller device buffers (addresses)."""
        _lib.check("aqua_radix_sort", self.lib.aqua_radix_sort(
            self.ctx, C.c_void_p(keys), C.c_void_p(perm), C.c_void_p(inv_perm),
            int(n), int(key_bits), C.c_void_p(stream or 0)))

    def set_profiling(self, on: bool = True):
        _lib.check("aqua_set_profiling",
                   self.lib.aqua_set_profiling(self.ctx, int(on)))

    def stage_times(self) -> dict:
        """Milliseconds of the stages of the last step (profiling on)."""
        ms = (C.c_float * 4)()
        _lib.check("aqua_stage_times", self.lib.aqua_stage_times(self.ctx, ms, 4))
        return dict(zip(("linklist", "gather", "sweep", "finalize"), ms[:]))

    def launches_per_step(self) -> int:
        return int(self.lib.aqua_launches_per_step(self.ctx))

    def get_unsorted(self, field: str, first: int, n: int, stream=None):
        """Values of ``field`` for the particles of original index
        [first, first + n), in original order (host array, synchronises):
        shape (n,) for scalars, (n, 2|4) for vec fields."""
        code, is_vec = _lib.FIELDS[field]
        nc = (4 if self.params.dims == 3 else 2) if is_vec else 1
        out = np.empty((n, nc), np.int32 if field == "imove" else np.float32)
        _lib.check("aqua_get_unsorted", self.lib.aqua_get_unsorted(
            self.ctx, code, int(first), int(n), out.ctypes.data_as(C.c_void_p),
            1, C.c_void_p(stream or 0)))
        return out if is_vec else out[:, 0]

    def free_surface(self, sensors, dr: float, case_index: int = -1,
                     stream=None) -> np.ndarray:
        """Free-surface elevation at each sensor: ``sensors`` is a list of
        horizontal positions (x in 2-D, (x, y) in 3-D)."""
        xy = np.zeros((len(sensors), 2), np.float32)
        for k, s in enumerate(sensors):
            s = np.atleast_1d(np.asarray(s, np.float32))
            xy[k, :len(s)] = s[:2]
        out = np.empty(len(sensors), np.float32)
        _lib.check("aqua_free_surface", self.lib.aqua_free_surface(
            self.ctx, xy.ctypes.data_as(_lib._F), len(sensors), float(dr),
            int(case_index), out.ctypes.data_as(_lib._F),
            C.c_void_p(stream or 0)))
        return out
