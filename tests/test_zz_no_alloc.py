"""aqua_radix_sort_noalloc(): the radix sort for callers that cannot
allocate device memory.

Hosts such as a tool running inside another runtime's pre-allocated step
loop, code that runs while a stream is captured into a graph, or a process
held to a fixed device-memory budget cannot call cudaMalloc.  The entry
point gives them the library's stable sort with no context: its scratch is
a fixed array inside the library.  This test calls it through the C ABI and
checks it against the context-based aqua_radix_sort on two calls in a row
(the shared scratch keeps the first call's contents, so the second call
shows that nothing stale leaks into a result), and that sizes above the
stated maximum are refused.

The file name puts it last in collection order; it passes alone in a fresh
process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "needs a CUDA device"
    torch.cuda.set_device(0)
    from aquagpusph_gb300 import _lib
    return torch, _lib, _lib.load()


def sort_with_context(torch, k, bits):
    from aquagpusph_gb300 import case as cases
    from aquagpusph_gb300.solver import Solver
    sv = Solver(cases.dam_break_2d(dx=0.05).params, capacity=len(k))
    keys = torch.from_numpy(k.view(np.int32).copy()).cuda()
    perm = torch.zeros_like(keys)
    inv = torch.zeros_like(keys)
    sv.radix_sort(keys.data_ptr(), perm.data_ptr(), inv.data_ptr(), len(k), bits)
    torch.cuda.synchronize()
    out = [t.cpu().numpy().view(np.uint32).copy() for t in (keys, perm, inv)]
    sv.close()
    return out


def sort_without_allocation(torch, lib, k, bits):
    keys = torch.from_numpy(k.view(np.int32).copy()).cuda()
    perm = torch.zeros_like(keys)
    inv = torch.zeros_like(keys)
    st = lib.aqua_radix_sort_noalloc(C.c_void_p(keys.data_ptr()),
                                     C.c_void_p(perm.data_ptr()),
                                     C.c_void_p(inv.data_ptr()),
                                     len(k), bits, None)
    torch.cuda.synchronize()
    assert st == 0
    return [t.cpu().numpy().view(np.uint32).copy() for t in (keys, perm, inv)]


def test_noalloc_sort_matches_context_sort_twice(env):
    torch, _lib, lib = env
    rng = np.random.default_rng(2026)
    for n, bits in ((1_000_000, 24), (123_457, 17)):
        k = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        k[: n // 7] = k[n // 3]   # ties: stability matters
        got = sort_without_allocation(torch, lib, k, bits)
        ref = sort_with_context(torch, k, bits)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
        assert np.array_equal(got[1], np.argsort(k, kind="stable"))


def test_noalloc_sort_rejects_oversize(env):
    torch, _lib, lib = env
    n = _lib.AQUA_NOALLOC_SORT_MAX_KEYS + 1
    keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = lib.aqua_radix_sort_noalloc(C.c_void_p(keys.data_ptr()), None, None,
                                     n, 8, None)
    torch.cuda.synchronize()
    assert st == _lib.AQUA_ERR_CAPACITY
