"""The installable step tool (libaqua_cuda_tool.so), loaded by the host
runtime the way the reference's CalcServer loads <Tool type="installable">
(dlopen + create_object), stepping the perturbed dam-break fixtures on the
GPU: one step equals the reference kernels' step (tests/golden/step_*d.npz)
bit for bit but the positions (within 1e-6: powf in the BIe PST), the second
within 1e-5, exactly as the direct C ABI does (tests/test_gpu_parity.py)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from aquagpusph_gb300 import case as cases
from test_gpu_parity import GOLD, RTOL_RATES, compare_state, golden_case, same


@pytest.fixture(scope="module")
def rt():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    from aquagpusph_gb300 import host
    r = host.HostRuntime()
    r.clear()
    yield r
    r.clear()


def as_case(params, arrays):
    n = int(arrays["N"][0])
    c = cases.Case(params, n)
    for k in c.state_arrays():
        getattr(c, k)[...] = arrays[k]
    c.t = float(arrays["t"][0])
    c.dt = float(arrays["dt"][0])
    c.iter = int(arrays["iter"][0])
    c.shepard = arrays["shepard"].copy()
    return c


@pytest.mark.parametrize("dims", [2, 3])
def test_installable_tool_steps_like_the_reference(rt, dims):
    g = np.load(os.path.join(GOLD, f"step_{dims}d.npz"))
    c = golden_case(g, dims)
    rt.clear()
    arrays = rt.set_case(c)
    rt.add_installable("aqua cuda step")
    rt.setup()
    rt.run(1)
    out = as_case(c.params, arrays)
    gold = {k[5:]: g[k] for k in g.files if k.startswith("out1_")}
    compare_state(out, gold)
    assert same(out.shepard, gold["shepard"])
    assert out.dt == float(gold["dt"]) and out.iter == int(gold["iter"])
    assert out.t == float(gold["t"])
    rt.run(1)
    out = as_case(c.params, arrays)
    gold = {k[5:]: g[k] for k in g.files if k.startswith("out2_")}
    compare_state(out, gold, exact_floats=False)
    assert abs(out.dt - float(gold["dt"])) <= RTOL_RATES * float(gold["dt"])
    rt.clear()


def test_once_tool_runs_once(rt):
    """A tool added with once=true steps only the first time the list runs
    (the reference's Tool(name, once) semantics)."""
    g = np.load(os.path.join(GOLD, "step_2d.npz"))
    c = golden_case(g, 2)
    rt.clear()
    arrays = rt.set_case(c)
    rt.add_installable("aqua cuda step", once=True)
    rt.setup()
    rt.run(3)
    assert int(arrays["iter"][0]) == c.iter + 1
    rt.clear()


@pytest.mark.parametrize("dims", [2, 3])
def test_link_list_tool_matches_reference_kernels(rt, dims):
    """The link-list tool alone, on the reference's LinkList test input
    (tests/{2D,3D}/LinkList), gives the link-list the reference's own kernels
    give, bit for bit."""
    g = np.load(os.path.join(GOLD, f"linklist_{dims}d.npz"))
    n = len(g["r"])
    vs = 4 if dims == 3 else 2
    cap = 1 << 16
    rt.clear()
    sv = rt.set_variable
    sv("N", "unsigned int", np.uint32(n).reshape(1))
    sv("dims", "int", np.int32(dims).reshape(1))
    sv("h", "float", np.float32([g["h"]]))
    sv("support", "float", np.float32([g["support"]]))
    sv("r_in", "vec*", np.ascontiguousarray(g["r"], np.float32))
    out = {k: sv(k, "unsigned int*", np.zeros(n, np.uint32))
           for k in ("icell", "id_sorted", "id_unsorted")}
    out["ihoc"] = sv("ihoc", "unsigned int*", np.zeros(cap, np.uint32))
    out["n_cells"] = sv("n_cells", "uivec4", np.zeros(4, np.uint32))
    out["r_min"] = sv("r_min", "vec", np.zeros(vs, np.float32))
    out["r_max"] = sv("r_max", "vec", np.zeros(vs, np.float32))
    rt.add_installable("link-list")
    rt.setup()
    rt.run(1)
    nw = int(out["n_cells"][3])
    assert same(out["n_cells"], g["n_cells"])
    assert same(out["r_min"][:dims], g["r_min"][:dims])
    assert same(out["r_max"][:dims], g["r_max"][:dims])
    for k in ("icell", "id_sorted", "id_unsorted"):
        assert same(out[k], g[k]), k
    assert same(out["ihoc"][:nw], g["ihoc"])
    rt.clear()
