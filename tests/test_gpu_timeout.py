"""The time-out path of the kernels' bounded waits, without a real
time-out.

Every wait of the library on an asynchronous copy or tensor-core operation
(an mbarrier poll) gives up after a fixed number of polls, records a
time-out in the error word and lets the kernel return.  A real time-out
cannot be caused on a shared GPU without leaving a copy or an MMA in
flight, so aqua_debug_fake_timeouts(1) makes each wait that COMPLETED
report a time-out: the error path (the kernel's early exit, the error word,
AQUA_ERR_TIMEOUT from aqua_check, a nonzero *err from the tensor-core entry
points) runs with nothing in flight.  The next call with the switch off
succeeds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from aquagpusph_gb300 import case as cases


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    from aquagpusph_gb300 import _lib
    lib = _lib.load()
    yield torch, _lib, lib
    lib.aqua_debug_fake_timeouts(0)


def small_3d():
    c = cases.dam_break_3d(dx=0.01, tank=(0.6, 0.3, 0.4), block=(0.2, 0.3, 0.2),
                           probes_z=(0.02,))
    c.dt = c.params.dt_fixed
    return c


@pytest.mark.parametrize("fast,variant", [(True, None), (False, 3)])
def test_step_wait_timeout_reaches_check(gpu, fast, variant):
    """The clustered sweep (bulk copies of the neighbourhood, fast build)
    and the queued sweep with bulk-copied groups (exact build, variant 3)."""
    torch, _lib, lib = gpu
    from aquagpusph_gb300.solver import Solver
    c = small_3d()
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(fast)
    if variant is not None:
        sv.set_tuning(variant, 8)
    sv.set_case(c)
    lib.aqua_debug_fake_timeouts(1)
    try:
        sv.step(1, graph=False)
        with pytest.raises(_lib.AquaError) as e:
            sv.check()
        assert e.value.status == _lib.AQUA_ERR_TIMEOUT
    finally:
        lib.aqua_debug_fake_timeouts(0)
    # the context stays usable: a fresh state steps cleanly
    sv.set_case(c)
    sv.step(2, graph=False)
    sv.check()
    g = sv.get_case()
    assert np.all(np.isfinite(g.r)) and g.iter == 2
    sv.close()


def test_tcgen05_wait_timeout_sets_err(gpu):
    torch, _lib, lib = gpu
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    M, K, N = 1000, 64, 64
    X = torch.randn((M, K), device="cuda").to(torch.bfloat16)
    W = torch.randn((N, K), device="cuda").to(torch.bfloat16)
    b = torch.zeros(N, dtype=torch.float32, device="cuda")
    Y = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.aqua_debug_fake_timeouts(1)
    try:
        assert L.aqua_gnn_linear_fwd_tc(M, K, N, Lm._p(X), K, Lm._p(W), Lm._p(b),
                                        None, 0, Lm._p(Y), N, 1, Lm._p(err),
                                        None) == 0
        torch.cuda.synchronize()
        assert int(err.item()) != 0
    finally:
        lib.aqua_debug_fake_timeouts(0)
    err.zero_()
    assert L.aqua_gnn_linear_fwd_tc(M, K, N, Lm._p(X), K, Lm._p(W), Lm._p(b),
                                    None, 0, Lm._p(Y), N, 1, Lm._p(err),
                                    None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
