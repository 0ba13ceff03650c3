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


def three_layers(torch, Lm, L, X, K, Ws, bs, acts, err):
    """Three aqua_gnn_linear_fwd_tc calls, bf16 activations in between."""
    cur, ldc = X, K
    for W, b, act in zip(Ws, bs, acts):
        y = torch.empty((X.shape[0], 64), dtype=torch.bfloat16, device="cuda")
        assert L.aqua_gnn_linear_fwd_tc(X.shape[0], ldc, 64, Lm._p(cur), ldc,
                                        Lm._p(W), Lm._p(b), None, 0, Lm._p(y),
                                        64, act, Lm._p(err), None) == 0
        cur, ldc = y, 64
    return cur


def weights(torch, rng, K1):
    Ws, bs = [], []
    for k in (K1, 64, 64):
        W = G.bf16(rng.normal(0, 0.2, (64, k)).astype(np.float32))
        Ws.append(torch.from_numpy(W).cuda().to(torch.bfloat16))
        bs.append(torch.from_numpy(rng.normal(0, 0.1, 64).astype(np.float32)).cuda())
    return Ws, bs


@pytest.mark.parametrize("K1", [16, 80])
@pytest.mark.parametrize("E", [1, 127, 128, 1000, 100000])
def test_fused_edge_mlp_rows_equals_three_layers(torch, E, K1):
    """Layer-1 input from rows: the first message-passing step's edge
    features (16 wide), or the first node MLP's input (80 wide, output
    written to columns 64..127 of rows 144 apart)."""
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(E + K1)
    X = torch.from_numpy(G.bf16(rng.normal(0, 1, (E, K1)).astype(np.float32))
                         ).cuda().to(torch.bfloat16)
    Ws, bs = weights(torch, rng, K1)
    acts = (1, 1, 0)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = three_layers(torch, Lm, L, X, K1, Ws, bs, acts, err)
    ld = 64 if K1 == 16 else 144
    Yb = torch.full((E, ld), -1, dtype=torch.int16, device="cuda")
    col = 0 if K1 == 16 else 64
    assert L.aqua_gnn_edge_mlp_tc(E, K1, Lm._p(X), K1, None, None, None, 0, None,
                                  Lm._p(Ws[0]), Lm._p(bs[0]), Lm._p(Ws[1]),
                                  Lm._p(bs[1]), Lm._p(Ws[2]), Lm._p(bs[2]),
                                  *acts, Lm._vp(Yb.data_ptr() + 2 * col), ld,
                                  Lm._p(err), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(Yb[:, col:col + 64], ref.view(torch.int16))
    # the other columns of the rows are not written
    assert bool((Yb[:, :col] == -1).all()) and bool((Yb[:, col + 64:] == -1).all())


@pytest.mark.parametrize("E,n", [(1, 3), (300, 40), (100000, 2500),
                                 (1000000, 25000)])
def test_fused_edge_mlp_pairs_equals_gather_and_three_layers(torch, E, n):
    """Layer-1 input gathered on chip from the node latents of both ends and
    the edge features ([H[recv], H[send], Ef], as aqua_gnn_gather_pair)."""
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(E + n)
    node = G.bf16(rng.normal(0, 1, (n, 144)).astype(np.float32))
    nd = torch.from_numpy(node).cuda().to(torch.bfloat16)
    H = Lm._vp(nd.data_ptr() + 2 * 64)   # columns 64..127 of rows 144 apart
    Ef = torch.from_numpy(G.bf16(rng.normal(0, 1, (E, 16)).astype(np.float32))
                          ).cuda().to(torch.bfloat16)
    recv = torch.from_numpy(np.sort(rng.integers(0, n, E)).astype(np.uint32)
                            .view(np.int32)).cuda()
    send = torch.from_numpy(rng.integers(0, n, E).astype(np.uint32)
                            .view(np.int32)).cuda()
    X2 = torch.empty((E, 144), dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_gather_pair(E, Lm._p(recv), Lm._p(send), H, 144,
                                  Lm._p(Ef), Lm._p(X2), None) == 0
    Ws, bs = weights(torch, rng, 144)
    acts = (1, 1, 0)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = three_layers(torch, Lm, L, X2, 144, Ws, bs, acts, err)
    Y = torch.empty((E, 64), dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_edge_mlp_tc(E, 144, None, 0, Lm._p(recv), Lm._p(send), H,
                                  144, Lm._p(Ef), Lm._p(Ws[0]), Lm._p(bs[0]),
                                  Lm._p(Ws[1]), Lm._p(bs[1]), Lm._p(Ws[2]),
                                  Lm._p(bs[2]), *acts, Lm._p(Y), 64, Lm._p(err),
                                  None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(Y.view(torch.int16), ref.view(torch.int16))


def test_fused_edge_mlp_rejects_bad_arguments(torch):
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    W = torch.zeros((64, 64), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros(64, dtype=torch.float32, device="cuda")
    Y = torch.empty((8, 64), dtype=torch.bfloat16, device="cuda")
    X = torch.zeros((8, 32), dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    args = [Lm._p(W), Lm._p(b)] * 3 + [1, 1, 0, Lm._p(Y), 64, Lm._p(err), None]
    # rows input must have K1 = 16; pair input needs its index arrays
    assert L.aqua_gnn_edge_mlp_tc(8, 32, Lm._p(X), 32, None, None, None, 0, None,
                                  *args) == -1
    assert L.aqua_gnn_edge_mlp_tc(8, 144, None, 0, None, None, None, 144, None,
                                  *args) == -1


def csr_graph(rng, n, mean_deg, n_big=0, big=300):
    """Receiver-major edges: random degrees (about 10% zero), n_big nodes
    of degree `big` (runs across several 128-edge tiles), random senders."""
    deg = rng.integers(0, 2 * mean_deg + 1, n)
    deg[rng.random(n) < 0.1] = 0
    if n_big:
        deg[rng.choice(n, n_big, replace=False)] = big
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint32)
    E = int(off[-1])
    recv = np.repeat(np.arange(n, dtype=np.uint32), deg)
    send = rng.integers(0, max(n, 1), E).astype(np.uint32)
    return off, recv, send, E


def dev_u32(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)
                            if len(a) else np.zeros(1, np.int32)).cuda()


GRAPHS = [(3, 2, 0, 0), (40, 8, 1, 300), (2500, 40, 5, 700), (25000, 40, 0, 0),
          (1, 0, 1, 1000), (50, 0, 0, 0)]


@pytest.mark.parametrize("pair", [False, True])
@pytest.mark.parametrize("n,deg,n_big,big", GRAPHS)
def test_fused_edge_mlp_sum_equals_mlp_then_segment_sum(torch, pair, n, deg,
                                                        n_big, big):
    """The edge MLP with the receiver sums fused in gives aqua_gnn_edge_mlp_tc
    followed by aqua_gnn_segment_sum bit for bit: receivers without edges,
    receivers whose edges span several tiles (and CTAs' ranges), a graph
    without edges; the columns of the output rows outside the 64 written
    stay untouched."""
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(n * 31 + deg + big + int(pair))
    off, recv, send, E = csr_graph(rng, n, deg, n_big, big)
    offd, recvd, sendd = (dev_u32(torch, a) for a in (off, recv, send))
    Ef = torch.from_numpy(G.bf16(rng.normal(0, 1, (max(E, 1), 16))
                                 .astype(np.float32))).cuda().to(torch.bfloat16)
    node = torch.from_numpy(G.bf16(rng.normal(0, 1, (n, 144)).astype(np.float32))
                            ).cuda().to(torch.bfloat16)
    H = Lm._vp(node.data_ptr() + 2 * 64)
    K1 = 144 if pair else 16
    Ws, bs = weights(torch, rng, K1)
    acts = (1, 1, 0)
    wargs = [Lm._p(Ws[0]), Lm._p(bs[0]), Lm._p(Ws[1]), Lm._p(bs[1]),
             Lm._p(Ws[2]), Lm._p(bs[2]), *acts]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    Y = torch.empty((max(E, 1), 64), dtype=torch.bfloat16, device="cuda")
    if pair:
        inputs = [None, 0, Lm._p(recvd), Lm._p(sendd), H, 144, Lm._p(Ef)]
    else:
        inputs = [Lm._p(Ef), 16, None, None, None, 0, None]
    assert L.aqua_gnn_edge_mlp_tc(E, K1, *inputs, *wargs, Lm._p(Y), 64,
                                  Lm._p(err), None) == 0
    ld = 80
    ref = torch.full((n, ld), 7.0, dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_segment_sum(n, Lm._p(offd), Lm._p(Y), 64, Lm.AGG_SCALE,
                                  Lm._p(ref), ld, 8, None) == 0
    out = torch.full((n, ld), 7.0, dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_edge_mlp_sum_tc(n, E, K1, inputs[0], inputs[1],
                                      Lm._p(offd), Lm._p(recvd),
                                      *inputs[3:], *wargs, Lm.AGG_SCALE,
                                      Lm._p(out), ld, 8, Lm._p(err), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(out.view(torch.int16), ref.view(torch.int16))
    assert bool((out[:, :8].float() == 7.0).all())
    assert bool((out[:, 72:].float() == 7.0).all())


def test_fused_edge_mlp_sum_rejects_bad_arguments(torch):
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    W = torch.zeros((64, 144), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros(64, dtype=torch.float32, device="cuda")
    X = torch.zeros((8, 16), dtype=torch.bfloat16, device="cuda")
    out = torch.empty((4, 80), dtype=torch.bfloat16, device="cuda")
    off = torch.zeros(5, dtype=torch.int32, device="cuda")
    recv = torch.zeros(8, dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    w = [Lm._p(W), Lm._p(b)] * 3 + [1, 1, 0, 0.5]
    ok = [4, 8, 16, Lm._p(X), 16, Lm._p(off), Lm._p(recv), None, None, 0, None,
          *w, Lm._p(out), 80, 0, Lm._p(err), None]
    bad = []
    for i, v in ((5, None), (6, None), (len(ok) - 5, None)):   # offsets, recv, out
        a = list(ok)
        a[i] = v
        bad.append(a)
    for i, v in ((len(ok) - 3, 3), (len(ok) - 3, 24), (len(ok) - 4, 68)):
        a = list(ok)                                         # col, ld
        a[i] = v
        bad.append(a)
    for a in bad:
        assert L.aqua_gnn_edge_mlp_sum_tc(*a) == -1


@pytest.mark.parametrize("M,N,K", [(1000, 64, 144), (300, 16, 64), (200000, 64, 64),
                                   (1, 64, 80), (5000, 64, 16), (777, 16, 144)])
def test_tcgen05_backward_matches(torch, M, N, K):
    """The tensor-core backward of a dense layer (data gradient with the
    SiLU' of the previous layer, weight and bias gradients) against numpy
    (float64) and against the mma.sync kernels on the same BF16 inputs."""
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(M + 3 * N + 7 * K)
    dY = G.bf16(rng.normal(0, 1, (M, N)).astype(np.float32))
    W = G.bf16(rng.normal(0, 0.2, (N, K)).astype(np.float32))
    X = G.bf16(rng.normal(0, 1, (M, K)).astype(np.float32))
    Zp = rng.normal(0, 1.5, (M, K)).astype(np.float32)
    dYd = torch.from_numpy(dY).cuda().to(torch.bfloat16)
    Wtd = torch.from_numpy(np.ascontiguousarray(W.T)).cuda().to(torch.bfloat16)
    Xd = torch.from_numpy(X).cuda().to(torch.bfloat16)
    Zd = torch.from_numpy(Zp).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    # data gradient
    dX1 = torch.empty((M, K), dtype=torch.bfloat16, device="cuda")
    dX2 = torch.empty_like(dX1)
    assert L.aqua_gnn_linear_dgrad_tc(M, N, K, Lm._p(dYd), N, Lm._p(Wtd),
                                      Lm._p(Zd), K, 1, Lm._p(dX1), K,
                                      Lm._p(err), None) == 0
    assert L.aqua_gnn_linear_dgrad(M, N, K, Lm._p(dYd), N, Lm._p(Wtd),
                                   Lm._p(Zd), K, 1, Lm._p(dX2), K, None) == 0
    # weight and bias gradients (accumulated onto nonzero starting values)
    dW0 = rng.normal(0, 1, (N, K)).astype(np.float32)
    db0 = rng.normal(0, 1, N).astype(np.float32)
    dW1, dW2 = torch.from_numpy(dW0).cuda(), torch.from_numpy(dW0).cuda()
    db1, db2 = torch.from_numpy(db0).cuda(), torch.from_numpy(db0).cuda()
    assert L.aqua_gnn_linear_wgrad_tc(M, N, K, Lm._p(dYd), N, Lm._p(Xd), K,
                                      Lm._p(dW1), Lm._p(db1), Lm._p(err),
                                      None) == 0
    assert L.aqua_gnn_linear_wgrad(M, N, K, Lm._p(dYd), N, Lm._p(Xd), K,
                                   Lm._p(dW2), Lm._p(db2), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    dy64, w64, x64, z64 = (a.astype(np.float64) for a in (dY, W, X, Zp))
    sg = 1.0 / (1.0 + np.exp(-z64))
    dx_ref = (dy64 @ w64) * sg * (1.0 + z64 * (1.0 - sg))
    a1 = dX1.float().cpu().numpy()
    a2 = dX2.float().cpu().numpy()
    scale = max(np.abs(dx_ref).max(), 1e-30)
    # one bf16 rounding of the output, plus f32 accumulation and SiLU'
    assert np.abs(a1 - dx_ref).max() <= 2.0 ** -7 * scale
    assert np.abs(a1 - a2).max() <= 2.0 ** -7 * scale
    dw_ref = dW0 + dy64.T @ x64
    db_ref = db0 + dy64.sum(0)
    assert rel(dW1.cpu().numpy(), dw_ref) < 1e-5
    assert rel(db1.cpu().numpy(), db_ref) < 1e-5
    assert rel(dW1.cpu().numpy(), dW2.cpu().numpy()) < 1e-5
    assert rel(db1.cpu().numpy(), db2.cpu().numpy()) < 1e-5
