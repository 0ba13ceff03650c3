"""The tcgen05 (tensor-memory) dense-layer forward against the mma.sync one
and numpy, on the same BF16 inputs: pre-activations within FP32 rounding,
activations within one BF16 rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import gnn_oracle as G


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("M,K", [(128, 16), (300, 64), (1000, 144), (5000, 80),
                                 (1, 64), (200000, 64)])
def test_tcgen05_forward_matches(torch, M, K):
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    N = 64
    rng = np.random.default_rng(M * 7 + K)
    X = G.bf16(rng.normal(0, 1, (M, K)).astype(np.float32))
    W = G.bf16(rng.normal(0, 0.2, (N, K)).astype(np.float32))
    b = rng.normal(0, 0.1, N).astype(np.float32)
    Xd = torch.from_numpy(X).cuda().to(torch.bfloat16)
    Wd = torch.from_numpy(W).cuda().to(torch.bfloat16)
    bd = torch.from_numpy(b).cuda()
    Z1 = torch.empty((M, N), dtype=torch.float32, device="cuda")
    Y1 = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.aqua_gnn_linear_fwd_tc(M, K, N, Lm._p(Xd), K, Lm._p(Wd), Lm._p(bd),
                                    Lm._p(Z1), N, Lm._p(Y1), N, 1, Lm._p(err),
                                    None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    Z2 = torch.empty_like(Z1)
    Y2 = torch.empty_like(Y1)
    assert L.aqua_gnn_linear_fwd(M, K, N, Lm._p(Xd), K, Lm._p(Wd), Lm._p(bd),
                                 Lm._p(Z2), N, Lm._p(Y2), N, 1, None) == 0
    zref = X.astype(np.float64) @ W.T.astype(np.float64) + b
    z1 = Z1.cpu().numpy()
    assert rel(z1, zref) < 1e-5
    assert np.abs(z1 - Z2.cpu().numpy()).max() <= 1e-4 * max(np.abs(zref).max(), 1)
    y1 = Y1.float().cpu().numpy()
    assert rel(y1, G.silu(zref)) < 1e-2
    # the two tensor-core paths agree to within one bf16 rounding
    y2 = Y2.float().cpu().numpy()
    assert np.abs(y1 - y2).max() <= 2.0 ** -7 * max(np.abs(y2).max(), 1)
