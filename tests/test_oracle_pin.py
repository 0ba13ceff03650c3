"""Pins the CPU oracle (oracle/aqua_oracle.cpp).

1. Against the golden fixtures of tests/golden/ -- computed by the
   reference's own kernel sources (oracle/_ref harness) on the reference's
   own test inputs (LinkList, RadixSort) and on perturbed dam breaks -- and
   against the assertions of the reference's tests
   (tests/3D/RadixSort/cMake/check.py, tests/{2D,3D}/LinkList/cMake/check.py,
   tests/2D/Regressions/midpoint_predictor/cMake/check.py).
2. Directly against the reference-kernel harness, step by step, where the
   reference tree is mounted (bit-exact on every Variable).
"""
import os

import numpy as np
import pytest

import oracle as O
from aquagpusph_gb300 import case as cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
REF_TREE = O.reference_dir()


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


@pytest.fixture(scope="module")
def ref():
    if REF_TREE is None:
        pytest.skip("reference tree not given (AQUA_REFERENCE_DIR)")
    if not (os.path.exists(O.ref_path(2)) and os.path.exists(O.ref_path(3))):
        O.build_oracle(ref=True)
    return {2: O.load_ref(2), 3: O.load_ref(3)}


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))
    return bool(np.array_equal(a, b))


def linklist_state(g):
    dims = 3 if g["r"].shape[1] == 4 else 2
    p = cases.Params(dims=dims, h=float(g["h"]), cs=1.0, g=(0, 0, 0, 0),
                     refd=(1.0, 1.0), visc_dyn=(0.0, 0.0), delta=(0.0, 0.0),
                     domain_min=(-10, -10, -10, 0), domain_max=(10, 10, 10, 0))
    c = cases.Case(p, len(g["r"]))
    c.r[...] = g["r"]
    st = O.OracleState(c, ihoc_capacity=1 << 16)
    st.arrays["r_in"][...] = g["r"]
    return st


@pytest.mark.parametrize("dims", [2, 3])
def test_linklist_golden(orc, dims):
    g = np.load(os.path.join(GOLD, f"linklist_{dims}d.npz"))
    st = linklist_state(g)
    orc.linklist(st)
    for k in ("icell", "id_sorted", "id_unsorted", "ihoc", "n_cells"):
        assert same(st[k], g[k]), k
    assert same(st["r_min"][:dims], g["r_min"][:dims])
    assert same(st["r_max"][:dims], g["r_max"][:dims])


@pytest.mark.parametrize("dims", [2, 3])
def test_linklist_reference_checks(orc, dims):
    """tests/{2D,3D}/LinkList/cMake/check.py: after sorting and unsorting,
    the ids come back in order 0..N-1; plus the ihoc contract."""
    g = np.load(os.path.join(GOLD, f"linklist_{dims}d.npz"))
    st = linklist_state(g)
    orc.linklist(st)
    n = len(g["r"])
    ids = np.arange(n, dtype=np.uint32)
    sorted_ids = np.empty_like(ids)
    sorted_ids[st["id_sorted"]] = ids          # sort stage1 scatter
    unsorted = sorted_ids[st["id_sorted"]]     # UnSort gather
    assert np.array_equal(unsorted, ids)
    icell = st["icell"]
    assert np.all(np.diff(icell.astype(np.int64)) >= 0)
    ihoc = st["ihoc"]
    nw = int(st["n_cells"][3])
    assert len(ihoc) == nw
    for c in np.unique(icell):
        assert ihoc[c] == np.flatnonzero(icell == c)[0]
    empty = np.setdiff1d(np.arange(nw), icell)
    assert np.all(ihoc[empty] == n)
    # isolated, coincident and out-of-box particles of the fixture
    assert icell[st["id_sorted"][0]] != icell[st["id_sorted"][3]]
    assert icell[st["id_sorted"][1]] == icell[st["id_sorted"][2]]


def test_radix_sort_golden(orc):
    g = np.load(os.path.join(GOLD, "radixsort_3d.npz"))
    k, perm, inv = orc.sort(g["keys"])
    assert same(k, g["sorted"]) and same(perm, g["perm"]) and same(inv, g["inv_perm"])
    # tests/3D/RadixSort/cMake/check.py
    f, f_orig = list(k), list(g["keys"])
    assert f == sorted(f) and f == sorted(f_orig) and f_orig != sorted(f_orig)
    for i in range(len(f)):
        assert f[i] == f_orig[perm[i]]
        assert f[inv[i]] == f_orig[i]
    # stability (ties keep the input order)
    assert np.array_equal(perm, np.argsort(g["keys"], kind="stable"))


@pytest.mark.parametrize("dims", [2, 3])
def test_step_golden(orc, dims):
    g = np.load(os.path.join(GOLD, f"step_{dims}d.npz"))
    c = golden_case(g, dims)
    st = O.OracleState(c)
    for step in (1, 2):
        orc.step(st)
        for k in st.arrays:
            assert same(st[k], g[f"out{step}_" + k]), (step, k)
        for k in ("n_cells", "t", "dt", "iter"):
            assert same(st[k], g[f"out{step}_" + k]), (step, k)


def golden_case(g, dims):
    from golden_cases import small_case
    c = small_case(dims)
    for k in ("id", "iset", "imove", "r", "normal", "tangent", "binormal", "u",
              "dudt", "rho", "drhodt", "m", "p"):
        getattr(c, k)[...] = g["in_" + k]
    c.t, c.dt, c.iter = float(g["in_t"]), float(g["in_dt"]), int(g["in_iter"])
    return c


def test_dt0_leaves_state(orc):
    """Regression analogue of tests/2D/Regressions/midpoint_predictor: with
    dt = 0 a step moves no particle and changes no velocity or density."""
    c = cases.dam_break_2d()
    c.dt = 0.0
    st = O.OracleState(c)
    orc.step(st)
    ids = st["id"]
    assert np.array_equal(st["r"], c.r[ids])
    assert np.array_equal(st["u"], c.u[ids])
    fl = st["imove"] == 1
    assert np.array_equal(st["rho"][fl], c.rho[ids][fl])


def test_boundary_paths_exercised(orc):
    """The perturbed fixture reaches the elastic bounce and the PST: turning
    them off (__DR_FACTOR__ = 0) changes the result."""
    g = np.load(os.path.join(GOLD, "step_3d.npz"))
    c = golden_case(g, 3)
    st1 = O.OracleState(c)
    orc.step(st1, steps=2)
    c2 = c.copy()
    c2.params = cases.Params(**{**c.params.__dict__, "dr_factor": 0.0})
    st2 = O.OracleState(c2)
    orc.step(st2, steps=2)
    assert not same(st1["r"], st2["r"])
    assert not same(st1["dudt"], st2["dudt"])


@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_matches_reference_kernels(orc, ref, dims):
    """Step by step, bit-exact on every Variable, against the reference's
    own kernel sources (built from the reference tree in place)."""
    from golden_cases import perturbed, small_case
    c = perturbed(small_case(dims), 100 + dims)
    a, b = O.OracleState(c), O.OracleState(c)
    for step in range(6):
        orc.step(a)
        ref[dims].step(b)
        for k in a.arrays:
            assert same(a[k], b[k]), (step, k)
        assert a["dt"] == b["dt"] and a["t"] == b["t"]


def test_oracle_matches_reference_kernels_c0(orc, ref):
    """The 2-D dam break of the benchmark configs (8,205 particles)."""
    from golden_cases import perturbed
    c = perturbed(cases.dam_break_2d(), 5)
    a, b = O.OracleState(c), O.OracleState(c)
    orc.step(a, steps=5)
    ref[2].step(b, steps=5)
    for k in a.arrays:
        assert same(a[k], b[k]), k
