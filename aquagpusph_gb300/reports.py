"""Reports of a run: probe histories and scalar time series, in the
reference's file formats.

* :class:`SetTabFile` -- the "particles" report (``<Report type="particles"
  fields="p,shepard" path="sensors.out" set=... ipf=... fps=.../>``,
  CalcServer/Reports/SetTabFile.cpp): one line per output, the time then
  every field of every particle of the range, in original particle order.
* :class:`TabFile` -- the "file" report of scalars (``<Report type="file"
  fields="t, H1, H2" path=.../>``, CalcServer/Reports/TabFile.cpp).
* :class:`FreeSurfaceSensors` -- wave-height sensors (the h_sensor.cl
  kernel and max reductions of the 3-D dam-break example), evaluated on the
  GPU by ``aqua_free_surface``.
* :class:`Run` -- steps a :class:`~aquagpusph_gb300.solver.Solver` and
  writes the reports when their output rule fires.

Numbers are written as the reference's streams write them: the time with
the default six significant digits, particle fields with 16 (the precision
the reference sets on devices with 64-bit addresses), vec fields as
``(x,y[,z,w])``.
"""
from __future__ import annotations

import numpy as np


def _g(v) -> str:
    # std::ostream << float with the default precision (%g, 6 digits)
    return format(float(np.float32(v)), "g")


def _g16(v) -> str:
    return format(float(v), ".16g")


class Report:
    """Output rule of the reference's reports (CalcServer/Reports/
    Report.cpp:134-161): with ipf > 0 a report fires when no output was made
    yet or when ipf iterations passed since the last one; with fps > 0 when
    the last output time is 0 or 1/fps seconds passed since it."""

    def __init__(self, ipf: int = 0, fps: float = 0.0):
        self.ipf = int(ipf)
        self.fps = float(fps)
        self._iter = 0
        self._t = np.float32(0.0)

    def must_update(self, t: float, iteration: int) -> bool:
        t = np.float32(t)
        if self.ipf > 0:
            if not self._iter or (iteration - self._iter >= self.ipf):
                self._iter, self._t = iteration, t
                return True
        if self.fps > 0.0:
            period = np.float32(1.0) / np.float32(self.fps)   # float division
            if self._t == 0.0 or np.float32(t - self._t) >= period:
                self._iter, self._t = iteration, t
                return True
        return False


class SetTabFile(Report):
    """Particles report: ``# Time p_7200 shepard_7200 ...`` header, then per
    output ``t v v ...`` (SetTabFile.cpp:70-94 header, :110-160 rows)."""

    def __init__(self, path: str, fields, first: int, n: int, ipf: int = 0,
                 fps: float = 0.0):
        super().__init__(ipf, fps)
        if isinstance(fields, str):
            fields = [f.strip() for f in fields.split(",") if f.strip()]
        self.path, self.fields = path, list(fields)
        self.first, self.n = int(first), int(n)
        self.rows = []        # (t, {field: values}) kept for the caller
        self._f = open(path, "w")
        head = "# Time "
        for i in range(self.first, self.first + self.n):
            for f in self.fields:
                head += f"{f}_{i} "
        self._f.write(head + "\n")
        self._f.flush()

    def write(self, t: float, values: dict):
        line = _g(t) + " "
        for i in range(self.n):
            for f in self.fields:
                v = values[f][i]
                if np.ndim(v):
                    line += "(" + ",".join(_g16(x) for x in v) + ")"
                else:
                    line += str(int(v)) if f == "imove" else _g16(v)
                line += " "
        self._f.write(line + "\n")
        self._f.flush()
        self.rows.append((float(t), {f: np.array(values[f]) for f in self.fields}))

    def collect(self, solver, stream=None) -> dict:
        return {f: solver.get_unsorted(f, self.first, self.n, stream)
                for f in self.fields}

    def close(self):
        self._f.close()


class TabFile:
    """Scalar report: ``# t H1 H2 `` header, then ``v v v `` per step
    (TabFile.cpp:63-84: every scalar with the default precision, the line
    ending in a space)."""

    def __init__(self, path: str, fields):
        if isinstance(fields, str):
            fields = [f.strip() for f in fields.split(",") if f.strip()]
        self.path, self.fields = path, list(fields)
        self.rows = []
        self._f = open(path, "w")
        self._f.write("# " + "".join(f"{f} " for f in self.fields) + "\n")
        self._f.flush()

    def write(self, values: dict):
        self._f.write("".join(f"{_g(values[f])} " for f in self.fields) + "\n")
        self._f.flush()
        self.rows.append({f: float(values[f]) for f in self.fields})

    def close(self):
        self._f.close()


class FreeSurfaceSensors:
    """Named wave-height sensors: ``{"H1": x}`` in 2-D or ``{"H1": (x, y)}``
    in 3-D, ``dr`` the particle spacing of the h_sensor kernel."""

    def __init__(self, sensors: dict, dr: float, case_index: int = -1):
        self.names = list(sensors)
        self.positions = [sensors[k] for k in self.names]
        self.dr = float(dr)
        self.case_index = int(case_index)

    def evaluate(self, solver, stream=None) -> dict:
        h = solver.free_surface(self.positions, self.dr, self.case_index, stream)
        return dict(zip(self.names, h))


def read_set_tab_file(path: str):
    """Parses a particles report back: (times, {column: values})."""
    with open(path) as f:
        names = f.readline().split()[2:]
        t, cols = [], {n: [] for n in names}
        for line in f:
            parts = line.split()
            if not parts:
                continue
            t.append(float(parts[0]))
            for n, v in zip(names, parts[1:]):
                cols[n].append(float(v) if "(" not in v else
                               [float(x) for x in v.strip("()").split(",")])
    return np.array(t), {k: np.array(v) for k, v in cols.items()}


class Run:
    """Steps a solver one step at a time and writes reports.

    The reference appends its reports after the step's tools, so they see
    the advanced time and iteration; the free-surface sensors are evaluated
    on the positions the step ends with (they run before the time-step
    tool in the example's pipeline, after the corrector)."""

    def __init__(self, solver, particle_reports=(), sensors=None,
                 sensors_file=None, stream=None):
        self.sv = solver
        self.particle_reports = list(particle_reports)
        self.sensors = sensors
        self.sensors_file = sensors_file
        self.stream = stream

    def step(self):
        sv, s = self.sv, self.stream
        sv.step(1, graph=True, stream=s)
        sc = sv.scalars(s)
        t, it = sc["t"], sc["iter"]
        for r in self.particle_reports:
            if r.must_update(t, it):
                r.write(t, r.collect(sv, s))
        if self.sensors is not None and self.sensors_file is not None:
            vals = {"t": t}
            vals.update(self.sensors.evaluate(sv, s))
            self.sensors_file.write(vals)
        return t, it

    def advance(self, end_time: float = None, steps: int = None):
        n = 0
        t = self.sv.scalars(self.stream)["t"]
        while (steps is None or n < steps) and (end_time is None or t < end_time):
            t, _ = self.step()
            n += 1
        self.sv.check(self.stream)
        return n

    def close(self):
        for r in self.particle_reports:
            r.close()
        if self.sensors_file is not None:
            self.sensors_file.close()
