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
