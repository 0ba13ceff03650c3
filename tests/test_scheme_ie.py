"""The improved Euler time scheme (basic/time_scheme/improved_euler.xml with
BI walls, as in the reference's BI examples) on the CPU.

1. The committed fixtures (tests/golden/step_ie_{2d,3d}.npz, made by the
   reference's own kernel sources through the oracle/_ref harness) obey the
   scheme's published formulas (improved_euler.cl:29-48): for fluid
   particles u1 = u0 + dt/2 (a0 + a1) and r1 = r0 + dt u0 + dt^2/4 (a0 + a1)
   with a0 the old and a1 the new rates.
2. The rates Variables of the particles whose rates are not computed keep
   the unpermuted old array: nothing in that stack re-sorts dudt/drhodt.
3. Where the reference tree is mounted, the harness regenerates the
   fixtures bit for bit, and with dt = 0 and zero rates the improved Euler
   and the midpoint sequences give the same state.
4. The C ABI refuses BIe walls with the improved Euler scheme (host-side
   validation, before any CUDA call), and so does the oracle's own
   restatement of the canonical stack, which covers neither BI walls nor
   this scheme.
"""
import ctypes
import dataclasses
import os

import numpy as np
import pytest

import oracle as O
from aquagpusph_gb300 import case as cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
REF_TREE = O.reference_dir()
STATE = ("id", "iset", "imove", "r", "normal", "tangent", "binormal", "u",
         "dudt", "rho", "drhodt", "m", "p")


def fixture(dims, name="ie"):
    return np.load(os.path.join(GOLD, f"step_{name}_{dims}d.npz"))


def fixture_case(d, dims, scheme=1):
    from golden_cases import small_case
    base = small_case(dims)
    c = cases.Case(dataclasses.replace(base.params, boundary=1, scheme=scheme),
                   len(d["in_r"]))
    for k in STATE:
        getattr(c, k)[...] = d["in_" + k]
    c.t, c.dt, c.iter = float(d["in_t"]), float(d["in_dt"]), int(d["in_iter"])
    return c


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))
    return bool(np.array_equal(a, b))


@pytest.mark.parametrize("dims", [2, 3])
def test_fixture_obeys_the_heun_formulas(dims):
    d = fixture(dims)
    dt = float(d["in_dt"])
    ids_in = d["in_id"]
    pos = np.empty(len(ids_in), np.int64)
    pos[ids_in] = np.arange(len(ids_in))          # id -> input index
    ids = d["out1_id"]
    k = pos[ids]                                  # sorted -> input index
    fl = (d["out1_imove"] == 1) & (d["in_imove"][k] == 1)
    D = dims
    f64 = lambda a: np.asarray(a, np.float64)
    r0, u0, a0 = f64(d["in_r"])[k][fl, :D], f64(d["in_u"])[k][fl, :D], f64(d["in_dudt"])[k][fl, :D]
    a1 = f64(d["out1_dudt"])[fl, :D]
    u1 = u0 + 0.5 * dt * (a0 + a1)
    r1 = r0 + dt * u0 + 0.25 * dt * dt * (a0 + a1)
    uscale = max(np.abs(u1).max(), 1e-3)
    assert np.abs(f64(d["out1_u"])[fl, :D] - u1).max() <= 1e-5 * uscale
    assert np.abs(f64(d["out1_r"])[fl, :D] - r1).max() <= 1e-6 * np.abs(r1).max()
    rho0, b0 = f64(d["in_rho"])[k][fl], f64(d["in_drhodt"])[k][fl]
    rho1 = rho0 + 0.5 * dt * (b0 + f64(d["out1_drhodt"])[fl])
    assert np.abs(f64(d["out1_rho"])[fl] - rho1).max() <= 1e-5 * np.abs(rho1).max()


@pytest.mark.parametrize("dims", [2, 3])
def test_fixture_rates_of_other_particles_keep_the_old_order(dims):
    """The walls' dudt after a step is the input array at the wall's new
    sorted index: BI/GradP.cl reads that stale value."""
    d = fixture(dims)
    nf = d["out1_imove"] != 1
    assert same(d["out1_dudt"][nf], d["in_dudt"][nf])
    assert same(d["out1_drhodt"][nf], d["in_drhodt"][nf])
    # the fixture exercises it: some walls read a fluid particle's rates
    wl = d["out1_imove"] == -3
    assert (np.abs(d["out1_dudt"][wl]).sum(1) > 0).any()


@pytest.fixture(scope="module")
def ref():
    if REF_TREE is None:
        pytest.skip("reference tree not given (AQUA_REFERENCE_DIR)")
    if not (os.path.exists(O.ref_path(2)) and os.path.exists(O.ref_path(3))):
        O.build_oracle(ref=True)
    return {2: O.load_ref(2), 3: O.load_ref(3)}


@pytest.mark.parametrize("name", ["bi", "ie"])
@pytest.mark.parametrize("dims", [2, 3])
def test_reference_kernels_regenerate_fixture(ref, dims, name):
    d = fixture(dims, name)
    st = O.OracleState(fixture_case(d, dims, scheme=1 if name == "ie" else 0))
    for step in (1, 2, 3, 4, 5):
        ref[dims].step(st)
        if step in (1, 2, 5):
            for k in STATE:
                assert same(st[k], d[f"out{step}_" + k]), (step, k)


@pytest.mark.parametrize("dims", [2, 3])
def test_dt0_improved_euler_equals_midpoint(ref, dims):
    d = fixture(dims)
    c = fixture_case(d, dims)
    c.dt = 0.0
    c.dudt[...] = 0.0
    c.drhodt[...] = 0.0
    a = O.OracleState(c)
    c0 = c.copy()
    c0.params = dataclasses.replace(c.params, scheme=0)
    b = O.OracleState(c0)
    ref[dims].step(a)
    ref[dims].step(b)
    for k in STATE + ("shepard",):
        assert same(a[k], b[k]), k
    assert a["dt"] == b["dt"]


def test_oracle_restatement_refuses_bi_and_improved_euler():
    orc = O.load_oracle()
    d = fixture(2)
    for scheme, boundary in ((1, 1), (0, 1), (1, 0)):
        c = fixture_case(d, 2, scheme)
        c.params = dataclasses.replace(c.params, boundary=boundary)
        with pytest.raises(RuntimeError):
            orc.step(O.OracleState(c))


def test_abi_refuses_bie_walls_with_improved_euler():
    from aquagpusph_gb300 import _lib, build
    lib = _lib.load(build.build())
    d = fixture(2)
    for boundary, scheme in ((0, 1), (1, 2), (0, -1)):
        c = fixture_case(d, 2, scheme)
        p, keep = _lib.params_struct(dataclasses.replace(c.params,
                                                         boundary=boundary))
        ctx = ctypes.c_void_p()
        st = lib.aqua_create(ctypes.byref(p), c.N, 0, ctypes.byref(ctx))
        assert st == _lib.AQUA_ERR_INVALID
        assert not ctx.value
