"""CPU restatement of the learned proposal's network (TEST INFRASTRUCTURE
ONLY: tests/ import it to check the GPU kernels of
aquagpusph_gb300/csrc/gnn.cu; the product never does).

The network has no counterpart in the reference.  This module states the
same computation as the GPU path in numpy, in two precisions:

* ``"bf16"`` -- the GPU's rounding points: features, weights, activations
  and gradients rounded to bfloat16 (round to nearest even) where the GPU
  stores them, products accumulated in float64 then rounded to float32 (the
  GPU accumulates in float32 in another order, so results agree to a few
  bf16 ulps, not bit for bit);
* ``"f64"`` -- no rounding at all, for finite-difference checks of the
  backward formulas.

Graph: nodes are the non-probe particles; node i receives from every node j
of the same case with |r_j - r_i| < radius, j != i.
"""
from __future__ import annotations

import numpy as np

LATENT = 64
FEAT = 16

# (name, out N, in K, activation of the output)
LAYERS = [
    ("e1_0", 64, 16, "silu"), ("e1_1", 64, 64, "silu"), ("e1_2", 64, 64, None),
    ("n1_0", 64, 80, "silu"), ("n1_1", 64, 64, "silu"), ("n1_2", 64, 64, None),
    ("e2_0", 64, 144, "silu"), ("e2_1", 64, 64, "silu"), ("e2_2", 64, 64, None),
    ("n2_0", 64, 144, "silu"), ("n2_1", 64, 64, "silu"), ("n2_2", 16, 64, None),
]


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).reshape(a.shape)
    nan = np.isnan(a)
    if nan.any():
        out = out.copy()
        out[nan] = np.nan
    return out


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def silu_grad(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def init_params(seed=0):
    """He-style initialisation: {name: (W (N x K), b (N))} float32."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, n, k, act in LAYERS:
        std = np.sqrt(2.0 / k) if act else np.sqrt(1.0 / k)
        if name == "n2_2":
            std *= 0.1
        p[name] = (rng.normal(0, std, (n, k)).astype(np.float32),
                   np.zeros(n, np.float32))
    return p


def wendland_shape(q):
    a = 1.0 - 0.5 * q
    return np.where(q < 2.0, (1.0 + 2.0 * q) * a * a * a * a, 0.0)


def node_features(dims, u, rho, dudt, drhodt, imove, normal, scales):
    h, U, R, A, Rd, rho0 = scales
    n = len(rho)
    f = np.zeros((n, FEAT), np.float64)
    k = 0
    f[:, k:k + dims] = u[:, :dims] / U
    k += dims
    f[:, k] = (rho - rho0) / R
    k += 1
    f[:, k:k + dims] = dudt[:, :dims] / A
    k += dims
    f[:, k] = drhodt / Rd
    k += 1
    f[:, k] = imove == 1
    f[:, k + 1] = imove < 0
    k += 2
    f[:, k:k + dims] = np.where((imove < 0)[:, None], normal[:, :dims], 0.0)
    return f


def edge_features(dims, recv, send, r, u, rho, imove, normal, scales):
    h, U, R = scales[0], scales[1], scales[2]
    d = (r[send, :dims] - r[recv, :dims])
    f = np.zeros((len(recv), FEAT), np.float64)
    k = 0
    f[:, k:k + dims] = d / h
    k += dims
    q = np.sqrt((d * d).sum(1)) / h
    f[:, k] = q
    k += 1
    f[:, k:k + dims] = (u[send, :dims] - u[recv, :dims]) / U
    k += dims
    f[:, k] = (rho[send] - rho[recv]) / R
    k += 1
    f[:, k] = wendland_shape(q)
    k += 1
    wall = imove[send] < 0
    f[:, k] = wall
    k += 1
    f[:, k:k + dims] = np.where(wall[:, None], normal[send, :dims], 0.0)
    return f


def neighbours(dims, r, imove, cid, radius):
    """(receivers, senders, offsets, nodes): nodes = non-probe particle
    indices in ascending order; edges receiver-major, senders ascending."""
    nodes = np.nonzero(imove != 0)[0]
    pos = np.asarray(r, np.float32)[nodes, :dims]
    # float32, one rounding per operation, as the GPU kernel computes it
    r2 = np.float32(radius) * np.float32(radius)
    recv, send, off = [], [], [0]
    c = cid[nodes]
    for a in range(len(nodes)):
        same = c == c[a]
        d = pos - pos[a]
        dd = np.zeros(len(pos), np.float32)
        for k in range(dims):
            dd = dd + d[:, k] * d[:, k]
        js = np.nonzero(same & (dd < r2))[0]
        js = js[js != a]
        recv.extend([a] * len(js))
        send.extend(js.tolist())
        off.append(len(send))
    return (np.array(recv, np.int64), np.array(send, np.int64),
            np.array(off, np.int64), nodes)


class Net:
    """Forward and backward of the two-round message-passing network."""

    def __init__(self, params, precision="bf16", agg_scale=1.0 / 32.0):
        self.p = params
        self.prec = precision
        self.scale = agg_scale

    def q(self, x):
        return bf16(x) if self.prec == "bf16" else np.asarray(x, np.float64)

    def W(self, name):
        w, b = self.p[name]
        return self.q(w).astype(np.float64), np.asarray(b, np.float64)

    def z32(self, z):
        return z.astype(np.float32).astype(np.float64) if self.prec == "bf16" else z

    def mlp_fwd(self, prefix, x):
        acts = [x]
        zs = []
        for k in range(3):
            w, b = self.W(f"{prefix}_{k}")
            z = self.z32(acts[-1] @ w.T + b)
            zs.append(z)
            acts.append(self.q(silu(z)) if k < 2 else self.q(z))
        return acts, zs

    def segsum(self, y, off):
        out = np.zeros((len(off) - 1, y.shape[1]))
        for s in range(len(off) - 1):
            out[s] = y[off[s]:off[s + 1]].sum(0)
        return self.q(out * self.scale)

    def forward(self, F, E0, recv, send, off):
        """F: node features (n x 16), E0: edge features (E x 16)."""
        c = {"F": self.q(F), "E0": self.q(E0)}
        a, z = self.mlp_fwd("e1", c["E0"])
        c["e1"] = (a, z)
        agg1 = self.segsum(a[-1], off)
        c["n1_in"] = np.concatenate([agg1, c["F"]], 1)
        a, z = self.mlp_fwd("n1", c["n1_in"])
        c["n1"] = (a, z)
        H = a[-1]
        c["X2"] = np.concatenate([H[recv], H[send], c["E0"]], 1)
        a, z = self.mlp_fwd("e2", c["X2"])
        c["e2"] = (a, z)
        agg2 = self.segsum(a[-1], off)
        c["n2_in"] = np.concatenate([agg2, H, c["F"]], 1)
        acts = [c["n2_in"]]
        zs = []
        for k in range(3):
            w, b = self.W(f"n2_{k}")
            zz = self.z32(acts[-1] @ w.T + b)
            zs.append(zz)
            acts.append(self.q(silu(zz)) if k < 2 else zz)
        c["n2"] = (acts, zs)
        c["out"] = zs[-1]
        return c["out"], c

    def mlp_bwd(self, prefix, cache, dy, grads, want_dx):
        acts, zs = cache
        for k in (2, 1, 0):
            w, b = self.W(f"{prefix}_{k}")
            grads[f"{prefix}_{k}"] = (dy.T @ acts[k], dy.sum(0))
            if k == 0 and not want_dx:
                return None
            dx = dy @ w
            if k > 0:
                dx = dx * silu_grad(zs[k - 1])
            dy = self.q(dx)
        return dy

    def backward(self, c, dout, recv, send, off):
        """dout: gradient of the loss w.r.t. out (n x 16).  Returns
        {layer: (dW, db)}."""
        g = {}
        dn2 = self.mlp_bwd("n2", c["n2"], self.q(dout), g, True)
        dagg2, dh_a = dn2[:, :64], dn2[:, 64:128]
        dy = self.q(dagg2[recv] * self.scale)
        dX2 = self.mlp_bwd("e2", c["e2"], dy, g, True)
        dH = np.zeros((len(off) - 1, 64))
        for s in range(len(off) - 1):
            dH[s] += dX2[off[s]:off[s + 1], :64].sum(0)
        np.add.at(dH, send, dX2[:, 64:128])
        if self.prec == "bf16":
            dH = dH.astype(np.float32).astype(np.float64)
        dh = self.q(dH + dh_a)
        dn1 = self.mlp_bwd("n1", c["n1"], dh, g, True)
        dagg1 = dn1[:, :64]
        dy = self.q(dagg1[recv] * self.scale)
        self.mlp_bwd("e1", c["e1"], dy, g, False)
        return g


def mse(out, target, mask):
    """Masked MSE over the first t columns and its gradient."""
    t = target.shape[1]
    cnt = float(mask.sum())
    d = np.zeros_like(out)
    diff = out[:, :t] - target
    loss = float((diff[mask] ** 2).sum() / cnt)
    d[mask, :t] = 2.0 * diff[mask] / cnt
    return loss, d
