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


# A child process without torch: a driver-API host that owns its contexts.
# It sorts in the device's primary context, in a context of its own, back in
# the primary one, and in a second context of its own created after the
# first was destroyed (which may reuse the old handle value).  The scratch
# array has a different address in every context, so each must look it up
# again; a result equal to numpy's stable argsort shows that it did.
_CONTEXT_SCRIPT = r"""
import ctypes as C
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from aquagpusph_gb300 import _lib
lib = _lib.load()
cu = C.CDLL("libcuda.so.1")
def ok(r, what):
    assert r == 0, f"{what}: CUresult {r}"
ok(cu.cuInit(0), "cuInit")
dev = C.c_int()
ok(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
primary = C.c_void_p()
ok(cu.cuDevicePrimaryCtxRetain(C.byref(primary), dev), "retain")
def new_context():
    ctx = C.c_void_p()
    if hasattr(cu, "cuCtxCreate_v2"):
        ok(cu.cuCtxCreate_v2(C.byref(ctx), 0, dev), "cuCtxCreate_v2")
    else:
        ok(cu.cuCtxCreate_v4(C.byref(ctx), None, 0, dev), "cuCtxCreate_v4")
    ok(cu.cuCtxSetCurrent(ctx), "set current")
    return ctx
def sort_here(seed, n, bits):
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
    k[: n // 5] = k[n // 2]
    bufs = []
    for _ in range(3):
        p = C.c_uint64()
        ok(cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(4 * n)), "cuMemAlloc")
        bufs.append(p)
    ok(cu.cuMemcpyHtoD_v2(bufs[0], k.ctypes.data_as(C.c_void_p),
                          C.c_size_t(4 * n)), "HtoD")
    st = lib.aqua_radix_sort_noalloc(C.c_void_p(bufs[0].value),
                                     C.c_void_p(bufs[1].value),
                                     C.c_void_p(bufs[2].value), n, bits, None)
    assert st == 0, st
    ok(cu.cuCtxSynchronize(), "sync")
    out = [np.empty(n, np.uint32) for _ in range(3)]
    for o, b in zip(out, bufs):
        ok(cu.cuMemcpyDtoH_v2(o.ctypes.data_as(C.c_void_p), b,
                              C.c_size_t(4 * n)), "DtoH")
        ok(cu.cuMemFree_v2(b), "cuMemFree")
    ref = np.argsort(k, kind="stable").astype(np.uint32)
    assert np.array_equal(out[1], ref), "perm"
    assert np.array_equal(out[0], k[ref]), "keys"
    inv = np.empty(n, np.uint32)
    inv[ref] = np.arange(n, dtype=np.uint32)
    assert np.array_equal(out[2], inv), "inverse perm"
ok(cu.cuCtxSetCurrent(primary), "set primary")
sort_here(1, 300_001, 20)
own = new_context()
sort_here(2, 654_321, 24)
ok(cu.cuCtxSetCurrent(primary), "set primary")
sort_here(3, 99_999, 12)
ok(cu.cuCtxDestroy_v2(own), "destroy")
own = new_context()
sort_here(4, 1 << 20, 24)
ok(cu.cuCtxDestroy_v2(own), "destroy")
ok(cu.cuDevicePrimaryCtxRelease_v2(dev), "release")
print("contexts ok")
"""


def test_noalloc_sort_in_each_cuda_context(env):
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _CONTEXT_SCRIPT, root],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "contexts ok" in r.stdout, r.stdout + r.stderr
