"""Parity at the workloads' full sizes, through the C ABI.

The other parity tests run reduced cases (a few thousand to twenty thousand
particles).  These run the cases the throughput is quoted on:

- the 3-D dam break of 5,878,404 particles (dx = 0.005 m, h = 0.01 m): its
  link-list (about 5e5 cells, three radix passes over 19-bit keys) bit-exact
  against the oracle's (LinkList.cl.in:32-113, LinkList.cpp:185-232, a
  stable sort), and one step of the exact build bit-exact on every Variable
  but the positions (1e-6: powf in the BIe PST), of the fast build within
  the per-step rate tolerance 1e-5 (norm-relative per field, fluid only);
- the 64-tank batch of the sloshing workload (935,414 particles): one step,
  every tank against the oracle run on that tank alone.

The oracle steps the 3-D case in about 8 s on 16 host threads.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O
from aquagpusph_gb300 import case as cases

RTOL_R = 1e-6
RTOL_RATES = 1e-5


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.set_device(0)
    from aquagpusph_gb300 import _lib
    _lib.load()
    return torch


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


def rel(a, b, mask=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    return float(np.abs(a[fin] - b[fin]).max() / max(np.abs(b[fin]).max(), 1e-30))


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))
    return bool(np.array_equal(a, b))


@pytest.fixture(scope="module")
def c1():
    c = cases.dam_break_3d()
    assert c.N == 5_878_404
    return c


def test_config1_linklist_bit_exact(gpu, orc, c1):
    """aqua_linklist on the 5.88M-particle dam break, its particles given in
    a shuffled order (so that the stable sort's ties all matter), equals
    the oracle's link-list: bounding box, n_cells, icell, both
    permutations and ihoc."""
    torch = gpu
    from aquagpusph_gb300.solver import Solver
    rng = np.random.default_rng(2026)
    order = rng.permutation(c1.N)
    c = c1.copy()
    for k in c.state_arrays():
        getattr(c, k)[...] = getattr(c1, k)[order]
    st = O.OracleState(c)
    st.arrays["r_in"][...] = c.r
    orc.linklist(st)
    nw = int(st["n_cells"][3])
    assert 4e5 < nw <= st.s.ihoc_capacity
    sv = Solver(c.params, capacity=c.N, ihoc_capacity=st.s.ihoc_capacity)
    r = torch.from_numpy(np.ascontiguousarray(c.r)).cuda()
    n = c.N
    icell = torch.zeros(n, dtype=torch.int32, device="cuda")
    ids = torch.zeros(n, dtype=torch.int32, device="cuda")
    idu = torch.zeros(n, dtype=torch.int32, device="cuda")
    ihoc = torch.zeros(st.s.ihoc_capacity, dtype=torch.int32, device="cuda")
    res = sv.linklist(r.data_ptr(), n, icell.data_ptr(), ids.data_ptr(),
                      idu.data_ptr(), ihoc.data_ptr(), st.s.ihoc_capacity)
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    assert same(res["n_cells"], st["n_cells"])
    assert same(res["r_min"][:3], st["r_min"][:3])
    assert same(res["r_max"][:3], st["r_max"][:3])
    assert same(u32(icell), st["icell"])
    assert same(u32(ids), st["id_sorted"])
    assert same(u32(idu), st["id_unsorted"])
    assert same(u32(ihoc)[:nw], st["ihoc"])
    sv.close()


@pytest.fixture(scope="module")
def c1_step(orc, c1):
    """The perturbed 5.88M-particle dam break (random velocities and rates,
    position jitter, one NaN and one out-of-domain particle) and the
    oracle's state after one step from it."""
    from golden_cases import perturbed
    c = perturbed(c1, 77)
    st = O.OracleState(c)
    orc.step(st)
    return c, st


def run_one_step(c, fast):
    from aquagpusph_gb300.solver import Solver
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(fast)
    sv.set_extras(True)
    sv.set_case(c)
    sv.step(1, graph=True)
    sv.check()
    out, ex = sv.get_case(), sv.get_extra()
    sv.close()
    return out, ex


def test_config1_one_step_exact(gpu, c1_step):
    c, st = c1_step
    out, ex = run_one_step(c, fast=False)
    for k in ("icell", "id_sorted", "id_unsorted", "ihoc", "n_cells"):
        assert same(ex[k], st[k]), k
    for k in ("id", "iset", "imove", "u", "dudt", "rho", "drhodt", "m", "p",
              "normal", "tangent", "binormal"):
        assert same(getattr(out, k), st[k]), k
    assert same(out.shepard, st["shepard"])
    for k in ("grad_p", "lap_u", "div_u", "lap_p", "grad_w_bi", "div_u_bi"):
        assert same(ex[k], st[k]), k
    assert rel(out.r, st["r"]) <= RTOL_R
    assert out.dt == st["dt"]


def test_config1_one_step_fast(gpu, c1_step):
    c, st = c1_step
    out, ex = run_one_step(c, fast=True)
    for k in ("icell", "id_sorted", "id_unsorted", "ihoc", "n_cells"):
        assert same(ex[k], st[k]), k
    assert same(out.id, st["id"]) and same(out.imove, st["imove"])
    fl = st["imove"] == 1
    errs = {k: rel(getattr(out, k), st[k], fl)
            for k in ("dudt", "drhodt", "u", "rho", "r")}
    print("config-1 fast step, norm-relative errors:", errs)
    assert errs["dudt"] <= RTOL_RATES and errs["drhodt"] <= RTOL_RATES, errs
    assert errs["u"] <= RTOL_RATES and errs["rho"] <= RTOL_R and errs["r"] <= RTOL_R
    assert abs(out.dt - st["dt"]) <= RTOL_RATES * st["dt"]


def test_config2_batch_one_step_per_tank(gpu, orc):
    """One step of the 64-tank sloshing batch; every tank equals the oracle
    run on that tank alone (rates, velocities, densities and pressures
    bit-exact, positions and the rolled walls 1e-6)."""
    from aquagpusph_gb300.solver import Solver
    b = cases.sloshing_batch_2d()
    assert b.n_cases == 64 and b.case.N == 935_414
    sv = Solver(b.case.params, capacity=b.case.N,
                ihoc_capacity=b.n_cases * b.case.params.max_cells())
    sv.set_batch(b)
    sv.step(1, graph=True)
    sv.check()
    g = sv.get_case()
    scal = sv.case_scalars()
    for k, c in enumerate(b.cases):
        lo, hi = int(b.offsets[k]), int(b.offsets[k + 1])
        st = O.OracleState(c)
        orc.step(st, motion=b.motions[k])
        assert np.array_equal(g.id[lo:hi] - lo, st["id"]), k
        fl = st["imove"] == 1
        for name in ("dudt", "drhodt", "rho", "p", "u"):
            assert np.array_equal(getattr(g, name)[lo:hi][fl], st[name][fl]), (k, name)
        assert rel(g.r[lo:hi], st["r"]) <= RTOL_R, k
        assert rel(g.u[lo:hi], st["u"]) <= RTOL_R, k
        assert scal[k]["dt"] == st["dt"] and scal[k]["iter"] == 1
    sv.close()
