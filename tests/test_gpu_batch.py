"""Batched cases (independent tanks packed into one particle set, one launch
per kernel for the whole batch) against the oracle run case by case, and
against the same cases run alone on the GPU.  The boundary of every tank
rolls (prescribed motion applied after the time step)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O
from aquagpusph_gb300 import case as cases


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def small_batch(n=4, seed=7):
    # 2-D sloshing tanks at dx = 0.01: ~1-4 thousand particles each
    return cases.sloshing_batch_2d(n_cases=n, seed=seed, dx=0.01)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def solver_for_batch(b):
    from aquagpusph_gb300.solver import Solver
    sv = Solver(b.case.params, capacity=b.case.N,
                ihoc_capacity=b.n_cases * b.case.params.max_cells())
    sv.set_batch(b)
    return sv


def test_batch_one_step_matches_oracle_per_case(gpu):
    b = small_batch()
    sv = solver_for_batch(b)
    sv.step(1, graph=True)
    sv.check()
    g = sv.get_case()
    scal = sv.case_scalars()
    orc = O.load_oracle()
    for k, c in enumerate(b.cases):
        lo, hi = int(b.offsets[k]), int(b.offsets[k + 1])
        st = O.OracleState(c)
        orc.step(st, motion=b.motions[k])
        # ids are global in the batch, local in the single case
        assert np.array_equal(g.id[lo:hi] - lo, st["id"])
        fl = st["imove"] == 1
        for name in ("dudt", "drhodt", "rho", "p"):
            assert np.array_equal(getattr(g, name)[lo:hi][fl], st[name][fl]), (k, name)
        assert np.array_equal(g.u[lo:hi][fl], st["u"][fl]), k
        # positions and the rolled boundary (cos/sin in double on both sides)
        assert rel(g.r[lo:hi], st["r"]) <= 1e-6, k
        assert rel(g.u[lo:hi], st["u"]) <= 1e-6, k
        assert scal[k]["dt"] == st["dt"] and scal[k]["iter"] == 1
        assert abs(scal[k]["t"] - st["t"]) <= 1e-12
    sv.close()


def test_batch_many_steps_matches_oracle(gpu):
    b = small_batch(n=3, seed=11)
    sv = solver_for_batch(b)
    sv.step(25, graph=True)
    sv.check()
    g = sv.get_case()
    orc = O.load_oracle()
    for k, c in enumerate(b.cases):
        lo, hi = int(b.offsets[k]), int(b.offsets[k + 1])
        st = O.OracleState(c)
        orc.step(st, steps=25, motion=b.motions[k])
        ga = np.argsort(g.id[lo:hi])
        sa = np.argsort(st["id"])
        for name in ("r", "u", "rho", "dudt"):
            assert rel(getattr(g, name)[lo:hi][ga], st[name][sa]) <= 1e-5, (k, name)
    sv.close()


def test_batch_equals_cases_run_alone(gpu):
    """Each case of a batch advances exactly as it does alone."""
    from aquagpusph_gb300.solver import Solver
    b = small_batch(n=3, seed=5)
    sv = solver_for_batch(b)
    sv.step(5, graph=True)
    sv.check()
    g = sv.get_case()
    for k, c in enumerate(b.cases):
        lo, hi = int(b.offsets[k]), int(b.offsets[k + 1])
        one = cases.pack([c], [b.motions[k]])
        s1 = solver_for_batch(one)
        s1.step(5, graph=True)
        s1.check()
        a = s1.get_case()
        for name in ("id", "imove", "r", "u", "dudt", "rho", "drhodt", "p"):
            x = getattr(g, name)[lo:hi]
            if name == "id":
                x = x - lo
            assert np.array_equal(x, getattr(a, name)), (k, name)
        s1.close()
    sv.close()


def test_config2_batch_runs(gpu):
    """The 64-tank batch of the sloshing workload steps without errors and
    every tank keeps its particles and mass."""
    b = cases.sloshing_batch_2d()
    sv = solver_for_batch(b)
    sv.step(10, graph=True)
    sv.check()
    g = sv.get_case()
    scal = sv.case_scalars()
    assert len(scal) == 64 and all(s["iter"] == 10 for s in scal)
    for k in range(64):
        lo, hi = int(b.offsets[k]), int(b.offsets[k + 1])
        assert np.all((g.id[lo:hi] >= lo) & (g.id[lo:hi] < hi))
        fl = g.imove[lo:hi] == 1
        m0 = b.cases[k].m[b.cases[k].imove == 1].astype(np.float64).sum()
        assert abs(g.m[lo:hi][fl].astype(np.float64).sum() - m0) <= 1e-9 * m0
    sv.close()
