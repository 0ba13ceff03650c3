"""Particle sets and case parameters of the canonical WCSPH step.

A :class:`Case` holds the particle Variables of one simulation in the
reference's layout (``vec`` = 4 floats per particle in 3-D, 2 in 2-D; index
arrays as unsigned 32-bit values, the reference's 32-bit ``usize``) together
with the scalar Variables and the compiled Definitions of the canonical preset
stack:

    basic.xml + basic/time_scheme/midpoint.xml (iter_midpoint_max=1,
    relax_midpoint=0) + basic/domain.xml + cfd.xml (__LAP_MORRIS__) +
    cfd/deltaSPH.xml + cfd/BIe.xml + cfd/variableTimeStep.xml,
    Wendland kernel, SUPPORT = 2.

The generators build the synthetic dam-break and sloshing cases the
benchmarks and tests run; their geometry follows the reference examples'
``Create.py`` scripts (fluid lattice at ((i+1/2)dx, ...), hydrostatic density
through the linear EOS, outward wall normals, wall "mass" = element area).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

__all__ = [
    "define_float",
    "Params",
    "Case",
    "dam_break_2d",
    "dam_break_3d",
]

FLUID = 1
SENSOR = 0
WALL = -3          # boundary-integral element
BUFFER = -256      # removed particle (Domain.cl)


def define_float(value: float) -> float:
    """Value of an evaluated ``<Define>`` as the kernels see it.

    CalcServer.cpp:247-257 evaluates the expression into a float and bakes it
    into the program as ``"%#G" + "f"``: six significant digits, then parsed
    as a float literal.
    """
    f = float(np.float32(value))
    return float(np.float32(float("%#G" % f)))


def _f32(x) -> float:
    return float(np.float32(x))


@dataclasses.dataclass
class Params:
    """Scalar Variables and Definitions of one case (``aqua_params``)."""
    dims: int
    h: float
    cs: float
    g: tuple
    refd: tuple
    visc_dyn: tuple
    delta: tuple
    domain_min: tuple
    domain_max: tuple
    support: float = 2.0
    p0: float = 0.0
    courant: float = 0.1
    dt_Ma: float = 0.1
    dt_min: float = 0.0
    dr_factor: float = 0.5
    min_bound_dist: float = 0.0
    relax_midpoint: float = 0.0
    iter_midpoint_max: int = 1
    # wall formulation: 0 = BIe (canonical), 1 = BI (analytic Shepard,
    # free-slip boundary integrals)
    boundary: int = 0
    # time scheme: 0 = midpoint (canonical), 1 = improved Euler
    # (basic/time_scheme/improved_euler.xml; BI walls only)
    scheme: int = 0

    # compiled Definitions (CalcServer.cpp:235-264, basic.xml:118-129)
    @property
    def H(self) -> float:
        return define_float(_f32(self.h))

    @property
    def CONW(self) -> float:
        return define_float(1.0 / float(np.float32(self.h)) ** self.dims)

    @property
    def CONF(self) -> float:
        return define_float(1.0 / float(np.float32(self.h)) ** (self.dims + 2))

    @property
    def DIMS(self) -> float:
        return define_float(self.dims)

    @property
    def SUPPORT(self) -> float:
        return 2.0

    @property
    def dt_fixed(self) -> float:
        """``fixed time step`` set_scalar: courant*h/cs, in double from the
        float Variables, stored as float (basic.xml:161)."""
        return _f32(_f32(self.courant) * _f32(self.h) / _f32(self.cs))

    @property
    def n_sets(self) -> int:
        return len(self.refd)

    @property
    def cell_length(self) -> float:
        return _f32(np.float32(self.support) * np.float32(self.h))

    def max_cells(self) -> int:
        """Upper bound of n_cells.w for any particle cloud inside the
        computational domain (the Domain tool parks escaping particles at
        domain_max, so r_min/r_max never leave the domain box)."""
        n = 1
        for k in range(self.dims):
            span = float(self.domain_max[k]) - float(self.domain_min[k])
            n *= int(span / self.cell_length) + 8
        return n


class Case:
    """Particle Variables of one case (host numpy arrays)."""

    ARRAYS_VEC = ("r", "normal", "tangent", "binormal", "u", "dudt")
    ARRAYS_F32 = ("rho", "drhodt", "m", "p")

    def __init__(self, params: Params, n: int):
        self.params = params
        self.dims = params.dims
        self.vs = 4 if params.dims == 3 else 2
        self.N = int(n)
        self.id = np.arange(n, dtype=np.uint32)
        self.iset = np.zeros(n, np.uint32)
        self.imove = np.ones(n, np.int32)
        for name in self.ARRAYS_VEC:
            setattr(self, name, np.zeros((n, self.vs), np.float32))
        for name in self.ARRAYS_F32:
            setattr(self, name, np.zeros(n, np.float32))
        self.t = 0.0
        self.dt = 0.0      # CalcServer.cpp:197 registers dt = 0
        self.iter = 0

    def copy(self) -> "Case":
        c = Case.__new__(Case)
        c.__dict__.update(self.__dict__)
        for name in ("id", "iset", "imove") + self.ARRAYS_VEC + self.ARRAYS_F32:
            setattr(c, name, getattr(self, name).copy())
        return c

    @property
    def n_fluid(self) -> int:
        return int((self.imove == FLUID).sum())

    def state_arrays(self):
        return {name: getattr(self, name) for name in
                ("id", "iset", "imove") + self.ARRAYS_VEC + self.ARRAYS_F32}


def _concat(parts, dims, vs):
    n = sum(len(p["r"]) for p in parts)
    out = {
        "r": np.zeros((n, vs), np.float32),
        "normal": np.zeros((n, vs), np.float32),
        "tangent": np.zeros((n, vs), np.float32),
        "u": np.zeros((n, vs), np.float32),
        "rho": np.zeros(n, np.float32),
        "m": np.zeros(n, np.float32),
        "p": np.zeros(n, np.float32),
        "imove": np.zeros(n, np.int32),
        "iset": np.zeros(n, np.uint32),
    }
    o = 0
    for p in parts:
        k = len(p["r"])
        for name in ("r", "normal", "tangent"):
            if name in p:
                out[name][o:o + k, :dims] = p[name]
        for name in ("rho", "m", "p", "imove", "iset"):
            out[name][o:o + k] = p[name]
        o += k
    return out


def _fill_case(params, parts):
    vs = 4 if params.dims == 3 else 2
    a = _concat(parts, params.dims, vs)
    c = Case(params, len(a["r"]))
    for name, v in a.items():
        getattr(c, name)[...] = v
    return c


def dam_break_2d(dx: float = 0.01, tank=(3.22, 1.8), column=(1.2, 0.6),
                 c0: float = 45.0, probe_y: float = 0.16, top: bool = True,
                 refd: float = 998.0, nu: float = 1.0e-6, delta: float = 0.1,
                 g: float = 9.81, hfac: float = 2.0,
                 extra_probes=()) -> Case:
    """2-D dam break: a water column at the left wall of a closed tank,
    boundary-integral walls at spacing dx, one pressure probe on the right
    wall (pattern of examples/2D/lobovsky_etal_2014/src/Create.py), plus
    optional probes at the (x, y) points of ``extra_probes`` (after it)."""
    L, Ht = tank
    nx = int(round(column[0] / dx))
    ny = int(round(column[1] / dx))
    hf = ny * dx
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    x = ((i.ravel() + 0.5) * dx)
    y = ((j.ravel() + 0.5) * dx)
    press = refd * g * (hf - y)
    dens = refd + press / c0 ** 2
    fluid = dict(r=np.stack([x, y], 1), rho=dens, m=dens * dx ** 2,
                 p=press, imove=np.full(len(x), FLUID), iset=np.zeros(len(x)))
    walls = []
    nL = int(round(L / dx))
    nH = int(round(Ht / dx))
    s = (np.arange(nL) + 0.5) * dx
    walls.append((np.stack([s, np.zeros_like(s)], 1), (0.0, -1.0)))
    if top:
        walls.append((np.stack([s, np.full_like(s, nH * dx)], 1), (0.0, 1.0)))
    s = (np.arange(nH) + 0.5) * dx
    walls.append((np.stack([np.zeros_like(s), s], 1), (-1.0, 0.0)))
    walls.append((np.stack([np.full_like(s, nL * dx), s], 1), (1.0, 0.0)))
    parts = [fluid]
    for pos, nrm in walls:
        k = len(pos)
        parts.append(dict(r=pos, normal=np.tile(nrm, (k, 1)),
                          tangent=np.tile((nrm[1], -nrm[0]), (k, 1)),
                          rho=np.full(k, refd), m=np.full(k, dx),
                          p=np.zeros(k), imove=np.full(k, WALL),
                          iset=np.ones(k)))
    probes = np.array([[nL * dx, probe_y]] + [list(q) for q in extra_probes])
    k = len(probes)
    parts.append(dict(r=probes, rho=np.full(k, refd), m=np.zeros(k),
                      p=np.zeros(k), imove=np.full(k, SENSOR), iset=np.ones(k)))
    margin = 4 * hfac * dx
    params = Params(dims=2, h=hfac * dx, cs=c0, g=(0.0, -g, 0.0, 0.0),
                    refd=(refd, refd), visc_dyn=(nu * refd, nu * refd),
                    delta=(delta, delta),
                    domain_min=(-margin, -margin, 0.0, 0.0),
                    domain_max=(nL * dx + margin, nH * dx + margin, 0.0, 0.0))
    return _fill_case(params, parts)


def dam_break_3d(dx: float = 0.005, tank=(3.22, 1.0, 1.0),
                 block=(1.228, 1.0, 0.55), c0: float = 40.0,
                 probes_z=(0.02, 0.06, 0.10, 0.14), top: bool = False,
                 refd: float = 998.0, nu: float = 1.0e-6, delta: float = 0.1,
                 g: float = 9.81, hfac: float = 2.0) -> Case:
    """3-D dam break (SPHERIC test 2 geometry without the obstacle): a water
    block at the x=0 wall of a tank, boundary-integral elements at dx on the
    five walls (six if ``top``), probes on the impact wall x = L
    (pattern of examples/3D/spheric_testcase2_dambreak/src/Create.py)."""
    L, W, Ht = tank
    nx = int(round(block[0] / dx))
    ny = int(round(block[1] / dx))
    nz = int(round(block[2] / dx))
    hf = nz * dx
    ii = np.arange(nx, dtype=np.float64)
    jj = np.arange(ny, dtype=np.float64)
    kk = np.arange(nz, dtype=np.float64)
    x = np.repeat((ii + 0.5) * dx, ny * nz)
    y = np.tile(np.repeat((jj + 0.5) * dx, nz), nx)
    z = np.tile((kk + 0.5) * dx, nx * ny)
    press = refd * g * (hf - z)
    dens = refd + press / c0 ** 2
    fluid = dict(r=np.stack([x, y, z], 1), rho=dens, m=dens * dx ** 3,
                 p=press, imove=np.full(len(x), FLUID), iset=np.zeros(len(x)))
    NX = int(round(L / dx))
    NY = int(round(W / dx))
    NZ = int(round(Ht / dx))
    Lx, Wy, Hz = NX * dx, NY * dx, NZ * dx

    def face(a_n, b_n, fix, axes, fixval, nrm, tng):
        a = (np.arange(a_n) + 0.5) * dx
        b = (np.arange(b_n) + 0.5) * dx
        A, B = np.meshgrid(a, b, indexing="ij")
        pos = np.zeros((A.size, 3))
        pos[:, axes[0]] = A.ravel()
        pos[:, axes[1]] = B.ravel()
        pos[:, fix] = fixval
        k = len(pos)
        return dict(r=pos, normal=np.tile(nrm, (k, 1)),
                    tangent=np.tile(tng, (k, 1)), rho=np.full(k, refd),
                    m=np.full(k, dx * dx), p=np.zeros(k),
                    imove=np.full(k, WALL), iset=np.ones(k))

    parts = [fluid,
             face(NX, NY, 2, (0, 1), 0.0, (0, 0, -1.0), (-1.0, 0, 0)),
             face(NY, NZ, 0, (1, 2), 0.0, (-1.0, 0, 0), (0, -1.0, 0)),
             face(NY, NZ, 0, (1, 2), Lx, (1.0, 0, 0), (0, 1.0, 0)),
             face(NX, NZ, 1, (0, 2), 0.0, (0, -1.0, 0), (1.0, 0, 0)),
             face(NX, NZ, 1, (0, 2), Wy, (0, 1.0, 0), (-1.0, 0, 0))]
    if top:
        parts.append(face(NX, NY, 2, (0, 1), Hz, (0, 0, 1.0), (1.0, 0, 0)))
    pz = np.asarray(probes_z, np.float64)
    if len(pz):
        parts.append(dict(r=np.stack([np.full_like(pz, Lx),
                                      np.full_like(pz, 0.5 * Wy), pz], 1),
                          rho=np.full(len(pz), refd), m=np.zeros(len(pz)),
                          p=np.zeros(len(pz)),
                          imove=np.full(len(pz), SENSOR),
                          iset=np.ones(len(pz))))
    margin = 4 * hfac * dx
    params = Params(dims=3, h=hfac * dx, cs=c0, g=(0.0, 0.0, -g, 0.0),
                    refd=(refd, refd), visc_dyn=(nu * refd, nu * refd),
                    delta=(delta, delta),
                    domain_min=(-margin, -margin, -margin, 0.0),
                    domain_max=(Lx + margin, Wy + margin, Hz + margin, 0.0))
    return _fill_case(params, parts)


@dataclasses.dataclass
class Motion:
    """Prescribed roll of a case's boundary elements and probes (particles
    of set ``iset`` that are not fluid) about the z axis through ``center``:
    psi(t) = amplitude * sin(angular_freq * t)."""
    amplitude: float          # rad
    angular_freq: float       # rad/s
    center: tuple = (0.0, 0.0, 0.0, 0.0)
    iset: int = 1


@dataclasses.dataclass
class Batch:
    """Independent cases packed into one concatenated particle set: case k
    holds particles [offsets[k], offsets[k+1]) of ``case``."""
    case: Case
    offsets: np.ndarray
    motions: list
    cases: list

    @property
    def n_cases(self) -> int:
        return len(self.offsets) - 1


def pack(cases: list, motions: list = None) -> Batch:
    """Concatenates cases that share their Params into one Batch."""
    params = cases[0].params
    n = sum(c.N for c in cases)
    big = Case(params, n)
    offsets = np.zeros(len(cases) + 1, np.uint32)
    o = 0
    for k, c in enumerate(cases):
        for name in big.state_arrays():
            getattr(big, name)[o:o + c.N] = getattr(c, name)
        o += c.N
        offsets[k + 1] = o
    big.id[:] = np.arange(n, dtype=np.uint32)
    big.t, big.dt, big.iter = cases[0].t, cases[0].dt, cases[0].iter
    return Batch(big, offsets, list(motions or [None] * len(cases)), cases)


def sloshing_tank_2d(fill: float, dx: float = 0.004, tank=(0.9, 0.5),
                     c0: float = 25.0, probe_above: float = 0.05,
                     refd: float = 998.0, nu: float = 1.0e-6,
                     delta: float = 0.1, g: float = 9.81,
                     hfac: float = 2.0) -> Case:
    """One closed 2-D sloshing tank (BIe walls on its four sides) filled to
    ``fill`` with water at hydrostatic density, and a pressure probe on the
    left wall ``probe_above`` above the still-water level."""
    W, Ht = tank
    nx = int(round(W / dx))
    ny = int(round(fill / dx))
    hf = ny * dx
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    x = (i.ravel() + 0.5) * dx
    y = (j.ravel() + 0.5) * dx
    press = refd * g * (hf - y)
    dens = refd + press / c0 ** 2
    parts = [dict(r=np.stack([x, y], 1), rho=dens, m=dens * dx ** 2, p=press,
                  imove=np.full(len(x), FLUID), iset=np.zeros(len(x)))]
    NX, NY = int(round(W / dx)), int(round(Ht / dx))
    s = (np.arange(NX) + 0.5) * dx
    t = (np.arange(NY) + 0.5) * dx
    walls = [(np.stack([s, np.zeros_like(s)], 1), (0.0, -1.0)),
             (np.stack([s, np.full_like(s, NY * dx)], 1), (0.0, 1.0)),
             (np.stack([np.zeros_like(t), t], 1), (-1.0, 0.0)),
             (np.stack([np.full_like(t, NX * dx), t], 1), (1.0, 0.0))]
    for pos, nrm in walls:
        k = len(pos)
        parts.append(dict(r=pos, normal=np.tile(nrm, (k, 1)),
                          tangent=np.tile((nrm[1], -nrm[0]), (k, 1)),
                          rho=np.full(k, refd), m=np.full(k, dx), p=np.zeros(k),
                          imove=np.full(k, WALL), iset=np.ones(k)))
    parts.append(dict(r=np.array([[0.0, hf + probe_above]]),
                      rho=np.array([refd]), m=np.array([0.0]), p=np.array([0.0]),
                      imove=np.array([SENSOR]), iset=np.ones(1)))
    # the domain holds the tank rolled by up to ~20 degrees about its bottom
    # centre
    cx = 0.5 * NX * dx
    reach = float(np.hypot(cx, NY * dx)) + 8 * hfac * dx
    params = Params(dims=2, h=hfac * dx, cs=c0, g=(0.0, -g, 0.0, 0.0),
                    refd=(refd, refd), visc_dyn=(nu * refd, nu * refd),
                    delta=(delta, delta),
                    domain_min=(cx - reach, -reach, 0.0, 0.0),
                    domain_max=(cx + reach, reach, 0.0, 0.0))
    return _fill_case(params, parts)


def sloshing_batch_2d(n_cases: int = 64, seed: int = 2026, dx: float = 0.004,
                      fill_range=(0.1, 0.4), amp_deg=(2.0, 8.0),
                      period=(1.2, 2.0), **kw) -> Batch:
    """Independent 2-D sloshing tanks of uneven fill, each rolled
    sinusoidally about its bottom centre with its own amplitude and period
    (seeded: numpy.random.default_rng(seed))."""
    rng = np.random.default_rng(seed)
    cases, motions = [], []
    for _ in range(n_cases):
        fill = float(rng.uniform(*fill_range))
        amp = float(np.deg2rad(rng.uniform(*amp_deg)))
        T = float(rng.uniform(*period))
        c = sloshing_tank_2d(fill, dx=dx, **kw)
        c.dt = c.params.dt_fixed
        cx = 0.5 * round(0.9 / dx) * dx if "tank" not in kw else 0.5 * kw["tank"][0]
        cases.append(c)
        motions.append(Motion(amplitude=amp, angular_freq=2.0 * math.pi / T,
                              center=(cx, 0.0, 0.0, 0.0), iset=1))
    return pack(cases, motions)
