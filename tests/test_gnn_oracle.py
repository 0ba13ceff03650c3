"""The CPU restatement of the learned proposal's network (oracle/
gnn_oracle.py): its backward pass against central finite differences in
float64, on a small random graph.  (The GPU kernels are compared with this
oracle in tests/test_gpu_gnn.py.)"""
import numpy as np

import gnn_oracle as G


def small_graph(seed=0, n=40, dims=2):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0, 0.1, (n, 4)).astype(np.float32)
    imove = np.ones(n, np.int32)
    imove[:6] = -3
    imove[6] = 0
    cid = np.zeros(n, np.int32)
    cid[n // 2:] = 1
    recv, send, off, nodes = G.neighbours(dims, r, imove, cid, 0.04)
    u = rng.normal(0, 0.1, (n, 4))
    rho = 1000 + rng.normal(0, 1, n)
    dudt = rng.normal(0, 1, (n, 4))
    drhodt = rng.normal(0, 1, n)
    normal = rng.normal(0, 1, (n, 4))
    sc = (0.01, 0.1, 1.0, 1.0, 1.0, 1000.0)
    F = G.node_features(dims, u[nodes], rho[nodes], dudt[nodes], drhodt[nodes],
                        imove[nodes], normal[nodes], sc)
    E0 = G.edge_features(dims, recv, send, r[nodes], u[nodes], rho[nodes],
                         imove[nodes], normal[nodes], sc)
    return F, E0, recv, send, off, imove[nodes]


def loss_of(params, F, E0, recv, send, off, target, mask):
    net = G.Net(params, "f64")
    out, c = net.forward(F, E0, recv, send, off)
    return G.mse(out, target, mask)[0]


def test_graph_is_symmetric_and_excludes_probes():
    F, E0, recv, send, off, imove = small_graph()
    pairs = set(zip(recv.tolist(), send.tolist()))
    assert all((j, i) in pairs for i, j in pairs)
    assert len(off) - 1 == len(imove) and (imove != 0).all()
    assert len(recv) > 50


def test_backward_matches_finite_differences():
    F, E0, recv, send, off, imove = small_graph(1)
    rng = np.random.default_rng(2)
    params = G.init_params(3)
    # non-trivial biases
    params = {k: (w, rng.normal(0, 0.1, len(b)).astype(np.float32))
              for k, (w, b) in params.items()}
    n = len(F)
    target = rng.normal(0, 1, (n, 3))
    mask = imove == 1
    net = G.Net(params, "f64")
    out, c = net.forward(F, E0, recv, send, off)
    loss, dout = G.mse(out, target, mask)
    grads = net.backward(c, dout, recv, send, off)
    eps = 1e-6
    for name in ("e1_0", "e1_2", "n1_0", "e2_0", "e2_1", "n2_0", "n2_2"):
        w, b = params[name]
        for (a, i) in [(0, 0), (1, 3), (w.shape[0] - 1, w.shape[1] - 1)]:
            p2 = {k: (v[0].astype(np.float64), v[1].astype(np.float64))
                  for k, v in params.items()}
            wp = p2[name][0].copy()
            wp[a, i] += eps
            lp = loss_of({**p2, name: (wp, p2[name][1])}, F, E0, recv, send, off,
                         target, mask)
            wm = p2[name][0].copy()
            wm[a, i] -= eps
            lm = loss_of({**p2, name: (wm, p2[name][1])}, F, E0, recv, send, off,
                         target, mask)
            fd = (lp - lm) / (2 * eps)
            an = grads[name][0][a, i]
            assert abs(fd - an) <= 1e-6 + 1e-4 * abs(fd), (name, a, i, fd, an)
        bp = p2[name][1].copy()
        bp[0] += eps
        lp = loss_of({**p2, name: (p2[name][0], bp)}, F, E0, recv, send, off,
                     target, mask)
        bm = p2[name][1].copy()
        bm[0] -= eps
        lm = loss_of({**p2, name: (p2[name][0], bm)}, F, E0, recv, send, off,
                     target, mask)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grads[name][1][0]) <= 1e-6 + 1e-4 * abs(fd), name


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e38], np.float32)
    y = G.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.015625 and y[3] == -2.5
