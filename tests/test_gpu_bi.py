"""BI walls (cfd/BI.xml in place of cfd/BIe.xml) on the GPU against the
golden fixtures that the reference's own BI kernels produced through the
reference-kernel harness: with the midpoint scheme
(tests/golden/step_bi_{2d,3d}.npz) and with the improved Euler scheme
(basic/time_scheme/improved_euler.xml, tests/golden/step_ie_{2d,3d}.npz).

The analytic Shepard factor goes through atan (2-D) and acos (3-D), whose
last bits differ between CUDA and the host libm, so after the link-list
(compared bit for bit) the Variables are compared with the per-step rate
tolerance, 1e-5 relative to each field's largest magnitude, after
one step, and 1e-4 after five (reordered by particle id)."""
import dataclasses
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from aquagpusph_gb300 import case as cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
STATE = ("id", "iset", "imove", "r", "normal", "tangent", "binormal", "u",
         "dudt", "rho", "drhodt", "m", "p")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


SCHEMES = {"bi": 0, "ie": 1}


def fixture_case(dims, name="bi"):
    from golden_cases import small_case
    d = np.load(os.path.join(GOLD, f"step_{name}_{dims}d.npz"))
    base = small_case(dims)
    c = cases.Case(dataclasses.replace(base.params, boundary=1,
                                       scheme=SCHEMES[name]),
                   len(d["in_r"]))
    for k in STATE:
        getattr(c, k)[...] = d["in_" + k]
    c.t, c.dt, c.iter = float(d["in_t"]), float(d["in_dt"]), int(d["in_iter"])
    return c, d


def close(a, b, mask=None):
    """max |a - b| over the finite entries, relative to max |b|"""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    if not fin.any():
        return 0.0
    return float(np.abs(a[fin] - b[fin]).max() / max(np.abs(b[fin]).max(), 1e-30))


@pytest.mark.parametrize("name", ["bi", "ie"])
@pytest.mark.parametrize("dims", [2, 3])
def test_bi_one_step_matches_reference_kernels(gpu, dims, name):
    from aquagpusph_gb300.solver import Solver
    c, d = fixture_case(dims, name)
    sv = Solver(c.params, capacity=c.N)
    sv.set_extras(True)
    sv.set_case(c)
    assert sv.launches_per_step() == 1 + Solver(  # one launch more than BIe
        dataclasses.replace(c.params, boundary=0, scheme=0),
        capacity=c.N).launches_per_step()
    sv.step(1, graph=False)
    sv.check()
    g = sv.get_case()
    # link-list and sort: exact
    for k in ("id", "iset", "imove"):
        assert np.array_equal(getattr(g, k), d["out1_" + k]), k
    fl = d["out1_imove"] == 1
    wl = d["out1_imove"] == -3
    errs = {
        "dudt": close(g.dudt, d["out1_dudt"], fl),
        "drhodt": close(g.drhodt, d["out1_drhodt"], fl),
        "u": close(g.u, d["out1_u"]),
        "rho": close(g.rho, d["out1_rho"]),
        "r": close(g.r, d["out1_r"]),
        "p_walls": close(g.p[wl], d["out1_p"][wl]),
        "rho_walls": close(g.rho[wl], d["out1_rho"][wl]),
    }
    sh = g.shepard
    active = (d["out1_imove"] >= -3) & (d["out1_imove"] <= 1)
    errs["shepard"] = close(sh[active], d["out1_shepard"][active])
    assert max(errs.values()) <= 1e-5, errs
    if name == "ie":
        # the rates Variables of every particle whose rates are not computed
        # are the unpermuted old arrays, copied bit for bit
        nf = ~fl
        assert np.array_equal(g.dudt[nf], d["out1_dudt"][nf])
        assert np.array_equal(g.drhodt[nf], d["out1_drhodt"][nf])
    sv.close()


@pytest.mark.parametrize("name", ["bi", "ie"])
@pytest.mark.parametrize("dims", [2, 3])
def test_bi_five_steps_match_reference_kernels(gpu, dims, name):
    from aquagpusph_gb300.solver import Solver
    c, d = fixture_case(dims, name)
    sv = Solver(c.params, capacity=c.N)
    sv.set_case(c)
    sv.step(5, graph=True)
    sv.check()
    g = sv.get_case()
    ga, sa = np.argsort(g.id), np.argsort(d["out5_id"])
    for k in ("imove", "iset"):
        assert np.array_equal(getattr(g, k)[ga], d["out5_" + k][sa]), k
    errs = {k: close(getattr(g, k)[ga], d["out5_" + k][sa])
            for k in ("r", "u", "rho", "dudt", "drhodt")}
    assert max(errs.values()) <= 1e-4, errs
    sv.close()


@pytest.mark.parametrize("name", ["bi", "ie"])
def test_bi_fast_build_close_to_exact(gpu, name):
    """The fast build stays within 1e-4 of the exact one over three steps."""
    from aquagpusph_gb300.solver import Solver
    c, d = fixture_case(2, name)
    runs = []
    for fast in (False, True):
        sv = Solver(c.params, capacity=c.N)
        sv.set_precision(fast)
        sv.set_case(c)
        sv.step(3, graph=True)
        sv.check()
        g = sv.get_case()
        runs.append(g)
        sv.close()
    a, b = runs
    ia, ib = np.argsort(a.id), np.argsort(b.id)
    for k in ("r", "u", "rho"):
        assert close(getattr(b, k)[ib], getattr(a, k)[ia]) <= 1e-4, k


def test_improved_euler_needs_bi_walls(gpu):
    """BIe walls with the improved Euler scheme are refused at creation."""
    from aquagpusph_gb300 import _lib
    from aquagpusph_gb300.solver import Solver
    c, _ = fixture_case(2, "ie")
    with pytest.raises(_lib.AquaError):
        Solver(dataclasses.replace(c.params, boundary=0), capacity=c.N)
