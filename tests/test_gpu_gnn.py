"""The learned proposal's GPU kernels against the CPU oracle
(oracle/gnn_oracle.py): dense layers (forward, data and weight gradients),
the neighbour graph, the whole two-round network forward and backward,
training and the proposal/judge/rollback loop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import gnn_oracle as G
from aquagpusph_gb300 import case as cases


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def to_bf16(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda().to(torch.bfloat16)


def from_bf16(t):
    return t.float().cpu().numpy()


@pytest.mark.parametrize("M,K,N", [(1000, 16, 64), (333, 64, 64), (70, 80, 64),
                                   (129, 144, 64), (517, 64, 16)])
def test_linear_layers_match_numpy(torch, M, K, N):
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(M + K + N)
    X = G.bf16(rng.normal(0, 1, (M, K)).astype(np.float32))
    W = G.bf16(rng.normal(0, 0.2, (N, K)).astype(np.float32))
    b = rng.normal(0, 0.1, N).astype(np.float32)
    Xd, Wd = to_bf16(torch, X), to_bf16(torch, W)
    bd = torch.from_numpy(b).cuda()
    Z = torch.empty((M, N), dtype=torch.float32, device="cuda")
    Y = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_linear_fwd(M, K, N, Lm._p(Xd), K, Lm._p(Wd), Lm._p(bd),
                                 Lm._p(Z), N, Lm._p(Y), N, 1, None) == 0
    zref = X.astype(np.float64) @ W.T.astype(np.float64) + b
    assert rel(Z.cpu().numpy(), zref) < 1e-5
    assert rel(from_bf16(Y), G.silu(zref)) < 1e-2
    # data gradient through silu of a previous layer
    dY = G.bf16(rng.normal(0, 1, (M, N)).astype(np.float32))
    Zp = rng.normal(0, 1, (M, K)).astype(np.float32)
    Wt = torch.empty((K, N), dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_transpose(N, K, Lm._p(Wd), Lm._p(Wt), None) == 0
    dX = torch.empty((M, K), dtype=torch.bfloat16, device="cuda")
    Zpd = torch.from_numpy(Zp).cuda()
    dYd = to_bf16(torch, dY)
    assert L.aqua_gnn_linear_dgrad(M, N, K, Lm._p(dYd), N, Lm._p(Wt), Lm._p(Zpd),
                                   K, 1, Lm._p(dX), K, None) == 0
    dref = (dY.astype(np.float64) @ W.astype(np.float64)) * G.silu_grad(Zp)
    assert rel(from_bf16(dX), dref) < 1e-2
    # weight gradient (accumulating)
    dW = torch.full((N, K), 0.5, dtype=torch.float32, device="cuda")
    db = torch.zeros(N, dtype=torch.float32, device="cuda")
    assert L.aqua_gnn_linear_wgrad(M, N, K, Lm._p(dYd), N, Lm._p(Xd), K,
                                   Lm._p(dW), Lm._p(db), None) == 0
    wref = dY.astype(np.float64).T @ X.astype(np.float64) + 0.5
    assert rel(dW.cpu().numpy(), wref) < 1e-5
    assert rel(db.cpu().numpy(), dY.sum(0)) < 1e-5


def small_batch(n=2, seed=5):
    return cases.sloshing_batch_2d(n_cases=n, seed=seed, dx=0.02)


def test_graph_matches_oracle(torch):
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    b = small_batch(3)
    c = b.case
    sv = Solver(c.params, capacity=c.N)
    r = torch.from_numpy(c.r).cuda()
    im = torch.from_numpy(c.imove).cuda()
    cid = Lm.case_ids(b)
    radius = float(c.params.support * c.params.h)
    g = Lm.Graph(sv, 2, r, im, cid, c.N, radius)
    recv, send, off, nodes = G.neighbours(2, c.r, c.imove, cid.cpu().numpy(), radius)
    assert g.n_nodes == len(nodes) and g.n_edges == len(recv)
    perm = g.perm.cpu().numpy()[: g.n_nodes]
    gr = perm[g.receivers.cpu().numpy()[: g.n_edges]]
    gs = perm[g.senders.cpu().numpy()[: g.n_edges]]
    assert set(zip(gr.tolist(), gs.tolist())) == \
        set(zip(nodes[recv].tolist(), nodes[send].tolist()))
    sv.close()


def network_inputs(torch, b, seed=0):
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    c = b.case
    rng = np.random.default_rng(seed)
    u = (rng.normal(0, 0.05, (c.N, 2))).astype(np.float32)
    dudt = rng.normal(0, 0.5, (c.N, 2)).astype(np.float32)
    drhodt = rng.normal(0, 5, c.N).astype(np.float32)
    rho = c.rho + rng.normal(0, 0.5, c.N).astype(np.float32)
    sv = Solver(c.params, capacity=c.N)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    r, im = dev(c.r), dev(c.imove)
    cid = Lm.case_ids(b)
    radius = float(c.params.support * c.params.h)
    g = Lm.Graph(sv, 2, r, im, cid, c.N, radius)
    x = Lm.Inputs(g, r, dev(u), dev(rho), dev(dudt), dev(drhodt), im,
                  dev(c.normal))
    host = dict(u=u, rho=rho, dudt=dudt, drhodt=drhodt)
    return sv, g, x, host


@pytest.mark.parametrize("tcgen05", [False, True])
def test_network_forward_backward_match_oracle(torch, tcgen05):
    from aquagpusph_gb300 import learned as Lm
    b = small_batch(2)
    c = b.case
    sv, g, x, host = network_inputs(torch, b)
    params = Lm.init_params(7)
    rng = np.random.default_rng(8)
    params = {k: (w, rng.normal(0, 0.05, len(bb)).astype(np.float32))
              for k, (w, bb) in params.items()}
    model = Lm.Model(2, params)
    sc = (float(c.params.h), 0.05, 0.5, 0.5, 5.0, 998.0)
    model.scales.copy_(torch.tensor(sc))
    net = Lm.Network(model, g, x, tcgen05=tcgen05)
    out = net.forward(train=True)
    n = g.n_nodes
    target = rng.normal(0, 1, (n, 3)).astype(np.float32)
    mask = (x.imove.cpu().numpy() == 1).astype(np.int32)
    loss, dout = Lm.mse_loss(out, torch.from_numpy(target).cuda(),
                             torch.from_numpy(mask).cuda())
    model.grad.zero_()
    net.backward(dout)
    # the oracle on the same graph (node order and edges of the GPU graph)
    perm = g.perm.cpu().numpy()[:n]
    recv = g.receivers.cpu().numpy()[: g.n_edges].astype(np.int64)
    send = g.senders.cpu().numpy()[: g.n_edges].astype(np.int64)
    off = g.offsets.cpu().numpy().astype(np.int64)
    im = c.imove[perm]
    F = G.node_features(2, host["u"][perm], host["rho"][perm], host["dudt"][perm],
                        host["drhodt"][perm], im, c.normal[perm], sc)
    E0 = G.edge_features(2, recv, send, c.r[perm], host["u"][perm],
                         host["rho"][perm], im, c.normal[perm], sc)
    onet = G.Net(params, "bf16", Lm.AGG_SCALE)
    oout, cache = onet.forward(F.astype(np.float32), E0.astype(np.float32),
                               recv, send, off)
    assert rel(out.cpu().numpy()[:, :3], oout[:, :3]) < 2e-2
    oloss, odout = G.mse(oout, target.astype(np.float64), mask.astype(bool))
    assert abs(float(loss.item()) - oloss) <= 2e-2 * oloss
    grads = onet.backward(cache, odout, recv, send, off)
    got = model.grads()
    for name in grads:
        assert rel(got[name][0], grads[name][0]) < 5e-2, name
        assert rel(got[name][1], grads[name][1]) < 5e-2, name
    sv.close()


def test_training_reduces_the_loss(torch):
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    b = small_batch(4, seed=9)
    c = b.case
    k = 8
    pairs, dts = Lm.collect_pairs(b, k, n_pairs=6, gap=40, warm=200, fast=True)
    model = Lm.Model(2, seed=1)
    Lm.fit_scales(model, pairs, dts, k, c.params, Lm.case_ids(b))
    sv = Solver(c.params, capacity=c.N)
    tr = Lm.Trainer(model, sv, b, k, lr=2e-3, cases_per_step=4)
    first = [float(tr.batch_loss(pairs[i], dts[i], 0, 4, train=False)[1].item())
             for i in range(len(pairs))]
    for _ in range(60):
        tr.step(pairs, dts)
    after = [float(tr.batch_loss(pairs[i], dts[i], 0, 4, train=False)[1].item())
             for i in range(len(pairs))]
    assert np.isfinite(after).all()
    assert np.mean(after) < 0.8 * np.mean(first), (first, after)
    sv.close()


def test_online_training_over_generations(torch):
    """The online trainer steps three generations of two tanks each through
    a ring of three snapshot pairs (more pairs than it holds), takes the
    configured Adam steps and lowers the loss."""
    from aquagpusph_gb300 import learned as Lm
    k = 8
    model = Lm.Model(2, seed=1)
    st = Lm.online_train(model, k, lambda n, g: small_batch(n, seed=20 + g),
                         n_runs=6, runs_per_gen=2, capacity=3, warm=100, gap=20,
                         pairs_per_gen=2, iters_per_pair=15, fit_pairs=2,
                         cases_per_step=2, lr=2e-3, seed=0)
    assert st["runs"] == 6 and st["generations"] == 3
    assert st["pairs_pushed"] == 6 and st["iterations"] == 3 * 2 * 15 - 15
    assert np.isfinite(st["loss_last10"])
    assert st["loss_last10"] < st["loss_first"], st


def test_proposal_judge_and_rollback(torch):
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    b = small_batch(4, seed=3)
    c = b.case
    k = 8
    sv = Solver(c.params, capacity=c.N,
                ihoc_capacity=b.n_cases * c.params.max_cells())
    sv.set_precision(True)
    sv.set_batch(b)
    sv.step(100, graph=True)
    t0 = sv.case_scalars()
    model = Lm.Model(2, seed=2)          # untrained: a poor proposal
    pairs, dts = Lm.collect_pairs(b, k, 2, 10, 100)
    Lm.fit_scales(model, pairs, dts, k, c.params, Lm.case_ids(b))
    run = Lm.ProposalRunner(sv, b, model, k=k, judge_fraction=0.5, tol=0.02)
    for _ in range(3):
        p_err, rho_err, judged = run.advance()
        assert len(judged) == 2 and np.isfinite(p_err).all()
    t1 = sv.case_scalars()
    for a, bb in zip(t0, t1):
        assert bb["iter"] == a["iter"] + 3 * k
        assert bb["t"] > a["t"]
    # the plain step continues from the proposed state
    sv.step(20, graph=True)
    sv.check()
    st = run.stats
    assert st["proposals"] == 3 and st["judged"] == 6
    assert 0 <= st["rolled_back"] <= 6
    sv.close()


def test_fused_edge_mlps_equal_the_layer_by_layer_forward(torch):
    """Inference with each edge MLP as one fused tcgen05 kernel, with or
    without the receiver sums fused in, gives the layer-by-layer tcgen05
    forward bit for bit."""
    from aquagpusph_gb300 import learned as Lm
    b = small_batch(3)
    sv, g, x, host = network_inputs(torch, b)
    params = Lm.init_params(11)
    model = Lm.Model(2, params)
    model.scales.copy_(torch.tensor((float(b.case.params.h), 0.05, 0.5, 0.5,
                                     5.0, 998.0)))
    outs = []
    for fused, summed in ((False, False), (True, False), (True, True)):
        net = Lm.Network(model, g, x, tcgen05=True, fused=fused,
                         fused_sum=summed)
        outs.append(net.forward(train=False).clone())
    assert torch.equal(outs[0], outs[1])
    # the edge outputs summed into the receivers on chip: the same bits
    assert torch.equal(outs[0], outs[2])
    sv.close()
