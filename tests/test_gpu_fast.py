"""The fast step kernels (-use_fast_math) against the exact oracle: from
the same snapshot, one step's rates dv/dt and drho/dt within the north
star's 1e-5 relative tolerance (norm-relative: max |a-b| / max |b| per
field), the link-list still bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O
from aquagpusph_gb300 import case as cases

RTOL = 1e-5


def rel(a, b, mask=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def cases_under_test():
    from golden_cases import perturbed
    return [
        ("c0", cases.dam_break_2d(), False),
        ("c0-perturbed", perturbed(cases.dam_break_2d(), 41), True),
        ("3d", cases.dam_break_3d(dx=0.01, tank=(0.6, 0.3, 0.4),
                                  block=(0.2, 0.3, 0.2), probes_z=(0.02,)), False),
        ("3d-perturbed", perturbed(cases.dam_break_3d(
            dx=0.01, tank=(0.6, 0.3, 0.4), block=(0.2, 0.3, 0.2),
            probes_z=(0.02,)), 42), True),
    ]


@pytest.mark.parametrize("idx", range(4))
def test_fast_step_rates_within_tolerance(gpu, idx):
    from aquagpusph_gb300.solver import Solver
    name, c, _ = cases_under_test()[idx]
    if c.dt == 0.0:
        c.dt = c.params.dt_fixed
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(True)
    sv.set_case(c)
    sv.step(1, graph=True)
    sv.check()
    g = sv.get_case()
    st = O.OracleState(c)
    O.load_oracle().step(st)
    assert np.array_equal(g.id, st["id"]), name       # link-list exact
    fl = st["imove"] == 1
    errs = {k: rel(getattr(g, k), st[k], fl) for k in ("dudt", "drhodt")}
    errs["r"] = rel(g.r, st["r"], fl)
    errs["u"] = rel(g.u, st["u"], fl)
    errs["rho"] = rel(g.rho, st["rho"], fl)
    print(name, errs)
    assert errs["dudt"] <= RTOL and errs["drhodt"] <= RTOL, (name, errs)
    assert errs["r"] <= 1e-6 and errs["u"] <= RTOL and errs["rho"] <= 1e-6
    sv.close()
