"""3-D run history: a small 3-D dam break (0.6 x 0.2 x 0.4 m tank, 0.2 m water
cube at the x = 0 wall, dx = 0.01 m, BIe walls, 15,602 particles) from rest
through the impact of the front on the far wall (first wetted at t = 0.225 s)
to t = 0.3 s, 6,001 steps.  The pressure histories of two probes on the
impact wall (z = 0.02 and 0.06 m) from the GPU run, with the exact and with
the fast build, agree with the CPU oracle's within 2% in relative L2 norm.
The oracle's history is the golden fixture tests/golden/history_3d.npz
(tests/golden/make_golden.py); two oracle runs whose inputs differ by one
ulp in one particle position give the same history over this window."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from aquagpusph_gb300 import reports as R
from make_golden import HISTORY_T_END, history_case_3d

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


@pytest.mark.parametrize("fast", [False, True])
def test_3d_probe_histories_within_2_percent(gpu, tmp_path, fast):
    from aquagpusph_gb300.solver import Solver
    gold = np.load(os.path.join(HERE, "golden", "history_3d.npz"))
    c = history_case_3d()
    assert c.N == int(gold["n"])
    first = int(gold["first"])
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(fast)
    sv.set_case(c)
    probes = R.SetTabFile(str(tmp_path / "sensors.out"), "p, shepard",
                          first=first, n=2, ipf=1)
    run = R.Run(sv, [probes])
    steps = run.advance(end_time=HISTORY_T_END)
    run.close()
    sv.close()
    t_gpu, cols = R.read_set_tab_file(str(tmp_path / "sensors.out"))
    assert len(t_gpu) == steps
    errs = {}
    for k in range(2):
        ref = np.interp(t_gpu, gold["t"], gold["p"][:, k].astype(np.float64))
        assert np.abs(gold["p"][:, k]).max() > 1000.0   # the probe is wetted
        got = np.asarray(cols[f"p_{first + k}"], np.float64)
        errs[k] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    assert all(np.isfinite(v) and v <= 0.02 for v in errs.values()), errs
