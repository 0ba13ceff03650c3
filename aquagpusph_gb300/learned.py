"""Learned k-step proposal over batched cases.

A message-passing network over the particles' neighbour graph (two rounds
of edge and node MLPs, latent width 64, SiLU, BF16 weights with FP32
accumulation on the tensor cores) predicts how far the state k steps ahead
departs from the explicit extrapolation of the current rates:

    u(t + k dt)   = u + k dt dudt + su * out[0:dims]
    rho(t + k dt) = rho + k dt drhodt + srho * out[dims]
    r(t + k dt)   = r + k dt (u + u(t + k dt)) / 2        (fluid particles)

It is trained on trajectories of the plain step (``Solver``) by the
library's own forward and backward kernels (include/aqua_learned.h) with
Adam.  ``ProposalRunner`` advances a batch: the network proposes k steps
for every case, the plain step re-runs a sampled subset of the cases from
the same state as the judge, and a case whose probe pressure departs by
more than a tolerance from the judge's is rolled back to the judge's state.

The learned component has no counterpart in the reference.  All GPU work
goes through ``libaqua_gb300.so``; PyTorch only allocates device memory.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib

LATENT = 64
FEAT = 16
# (name, out N, in K, activation)
LAYERS = [
    ("e1_0", 64, 16, 1), ("e1_1", 64, 64, 1), ("e1_2", 64, 64, 0),
    ("n1_0", 64, 80, 1), ("n1_1", 64, 64, 1), ("n1_2", 64, 64, 0),
    ("e2_0", 64, 144, 1), ("e2_1", 64, 64, 1), ("e2_2", 64, 64, 0),
    ("n2_0", 64, 144, 1), ("n2_1", 64, 64, 1), ("n2_2", 16, 64, 0),
]
AGG_SCALE = 1.0 / 32.0
# aqua_gnn_probes_pressure: probes per call and device scratch (floats)
MAX_PROBES = 8
PROBE_SCRATCH = 2 * MAX_PROBES * 256
# 64-wide layers run on tcgen05 (tensor memory) when True, on mma.sync
# otherwise (the 16-wide output layer always uses mma.sync)
USE_TCGEN05 = True
# inference runs each edge MLP as one fused tcgen05 kernel (inputs gathered
# and activations kept on chip) when True
FUSE_EDGE_MLP = True
# ... and sums its output into the receivers on chip as well (no E x 64
# intermediate) when True
FUSE_EDGE_SUM = True
# edge features read packed per-node records (aqua_gnn_node_records) when
# True, the separate node arrays otherwise; the features are the same
EDGE_RECORDS = True

_vp = C.c_void_p


def _torch():
    import torch
    return torch


def _p(t):
    return _vp(t.data_ptr()) if t is not None else _vp(0)


# entry points called (each launches at least one kernel); for accounting
CALLS = [0]


def _chk(name, st):
    CALLS[0] += 1
    _lib.check(name, st)


_u32, _i32, _f32 = C.c_uint32, C.c_int32, C.c_float
# argument types of every function of include/aqua_learned.h
SIGNATURES = {
    "aqua_gnn_cell_keys": [_u32, _i32, _vp, _vp, _vp, _f32, _vp, _vp, _vp, _vp,
                           _vp],
    "aqua_gnn_cell_ranges": [_u32, _vp, _u32, _vp, _vp, _vp],
    "aqua_gnn_neighbours": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _f32, _vp, _vp,
                            _vp, _vp, _vp],
    "aqua_gnn_bbox": [_u32, _i32, _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_exclusive_scan": [_u32, _vp, _vp, _vp, _vp],
    "aqua_gnn_gather32": [_u32, _vp, _vp, _u32, _u32, _vp, _vp],
    "aqua_gnn_scatter32": [_u32, _vp, _vp, _u32, _vp, _u32, _vp],
    "aqua_gnn_node_features": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _vp, _u32, _u32, _vp],
    "aqua_gnn_edge_features": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _vp, _vp, _vp],
    "aqua_gnn_node_records": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_edge_features_rec": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_linear_fwd": [_u32, _u32, _u32, _vp, _u32, _vp, _vp, _vp, _u32,
                            _vp, _u32, _i32, _vp],
    "aqua_gnn_linear_fwd_tc": [_u32, _u32, _u32, _vp, _u32, _vp, _vp, _vp,
                               _u32, _vp, _u32, _i32, _vp, _vp],
    "aqua_gnn_edge_mlp_tc": [_u32, _u32, _vp, _u32, _vp, _vp, _vp, _u32, _vp,
                             _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32,
                             _vp, _u32, _vp, _vp],
    "aqua_gnn_edge_mlp_sum_tc": [_u32, _u32, _u32, _vp, _u32, _vp, _vp, _vp,
                                 _vp, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _i32, _i32, _i32, _f32, _vp, _u32, _u32, _vp,
                                 _vp],
    "aqua_gnn_linear_dgrad": [_u32, _u32, _u32, _vp, _u32, _vp, _vp, _u32,
                              _i32, _vp, _u32, _vp],
    "aqua_gnn_linear_wgrad": [_u32, _u32, _u32, _vp, _u32, _vp, _u32, _vp, _vp,
                              _vp],
    "aqua_gnn_linear_dgrad_tc": [_u32, _u32, _u32, _vp, _u32, _vp, _vp, _u32,
                                 _i32, _vp, _u32, _vp, _vp],
    "aqua_gnn_linear_wgrad_tc": [_u32, _u32, _u32, _vp, _u32, _vp, _u32, _vp,
                                 _vp, _vp, _vp],
    "aqua_gnn_segment_sum": [_u32, _vp, _vp, _u32, _f32, _vp, _u32, _u32, _vp],
    "aqua_gnn_segment_bcast": [_u32, _vp, _vp, _u32, _u32, _f32, _vp, _u32,
                               _vp],
    "aqua_gnn_gather_pair": [_u32, _vp, _vp, _vp, _u32, _vp, _vp, _vp],
    "aqua_gnn_scatter_pair": [_u32, _u32, _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_add_to_bf16": [_u32, _vp, _vp, _u32, _u32, _vp, _u32, _u32, _vp],
    "aqua_gnn_mse": [_u32, _u32, _vp, _vp, _vp, _f32, _vp, _vp, _vp],
    "aqua_gnn_adam": [_u32, _vp, _vp, _vp, _vp, _f32, _f32, _f32, _f32, _u32,
                      _vp, _vp],
    "aqua_gnn_to_bf16": [_u32, _vp, _vp, _vp],
    "aqua_gnn_transpose": [_u32, _u32, _vp, _vp, _vp],
    "aqua_gnn_apply": [_u32, _i32, _vp, _vp, _vp, _vp, _u32, _f32, _f32, _vp,
                       _vp, _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_targets": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                         _vp, _u32, _f32, _f32, _vp, _vp, _vp, _vp],
    "aqua_gnn_roll": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                      _vp, _vp, _vp, _vp, _vp],
    "aqua_gnn_probe_pressure": [_u32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                _vp],
    "aqua_gnn_probes_pressure": [_u32, _i32, _vp, _vp, _vp, _vp, _u32, _vp, _vp,
                                 _vp, _vp, _vp],
    "aqua_gnn_sample_max_diff": [_u32, _vp, _vp, _vp, _u32, _f32, _f32, _vp,
                                 _vp],
    "aqua_gnn_case_max_diff": [_u32, _vp, _vp, _vp, _vp, _f32, _vp, _vp],
    "aqua_gnn_judge_density": [_u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _f32, _f32, _f32, _u32, _vp, _vp, _vp],
}


def _bind(lib):
    if getattr(lib, "_gnn_bound", False):
        return lib
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib._gnn_bound = True
    return lib


def lib():
    return _bind(_lib.load())


# ------------------------------------------------------------------ graph ----

class Graph:
    """Neighbour graph of the non-probe particles of a batch (device).

    Node s is particle ``perm[s]``; edges are receiver-major (``offsets``)
    with ``receivers`` / ``senders`` as node indices.  Cases never connect:
    the cell key carries the case id."""

    def __init__(self, solver, dims, r, imove, cid, n, radius, stream=None):
        torch = _torch()
        L = lib()
        dev = r.device
        s = _vp(stream or 0)
        self.dims, self.n, self.radius = dims, n, float(radius)
        box = (C.c_float * 6)()
        scratch = torch.empty(8, dtype=torch.int32, device=dev)
        _chk("aqua_gnn_bbox", L.aqua_gnn_bbox(n, dims, _p(r), _p(imove),
                                               _p(scratch), box, s))
        cell = float(radius)
        lo = np.array(box[0:3], np.float64) - cell
        hi = np.array(box[3:6], np.float64) + cell
        if dims == 2 or n == 0:
            lo[dims:] = 0.0
            hi[dims:] = 0.0
        if n == 0:
            lo[:] = hi[:] = 0.0
        nc = np.maximum(np.ceil((hi - lo) / cell).astype(np.int64) + 1, 1)
        if dims == 2:
            nc[2] = 1
        n_cases = int(cid.max().item()) + 1 if n else 1
        per_case = int(np.prod(nc))
        n_keys = per_case * n_cases
        if n_keys >= 0xFFFFFFFF:
            raise ValueError("cell grid too large for 32-bit keys")
        origin = (C.c_float * 3)(*lo.astype(np.float32))
        ncell = (C.c_uint32 * 3)(*nc.astype(np.uint32))
        self.keys = torch.empty(n, dtype=torch.int32, device=dev)
        self.perm = torch.empty(n, dtype=torch.int32, device=dev)
        _chk("aqua_gnn_cell_keys", L.aqua_gnn_cell_keys(
            n, dims, _p(r), _p(imove), _p(cid), cell, origin, ncell,
            _p(self.keys), _p(self.perm), s))
        # probes carry key 0xffffffff: all 32 bits take part in the sort
        solver.radix_sort(self.keys.data_ptr(), self.perm.data_ptr(), 0, n, 32,
                          stream)
        self.n_nodes = int((imove != 0).sum().item())
        cstart = torch.empty(n_keys, dtype=torch.int32, device=dev)
        cend = torch.empty(n_keys, dtype=torch.int32, device=dev)
        _chk("aqua_gnn_cell_ranges", L.aqua_gnn_cell_ranges(
            n, _p(self.keys), n_keys, _p(cstart), _p(cend), s))
        nn = self.n_nodes
        vs = 4 if dims == 3 else 2
        self.rs = torch.empty((nn, vs), dtype=torch.float32, device=dev)
        _chk("aqua_gnn_gather32", L.aqua_gnn_gather32(
            nn, _p(self.perm), _p(r), vs, vs, _p(self.rs), s))
        deg = torch.empty(nn, dtype=torch.int32, device=dev)
        _chk("aqua_gnn_neighbours", L.aqua_gnn_neighbours(
            nn, dims, _p(self.rs), _p(self.keys), ncell, _p(cstart), _p(cend),
            radius, _p(deg), _vp(0), _vp(0), _vp(0), s))
        # 32-bit edge offsets (the kernels take E < 2^31)
        total = int(deg.sum(dtype=torch.int64).item()) if nn else 0
        if total >= 2 ** 31:
            raise ValueError(f"{total} edges: the graph needs E < 2^31 "
                             "(a smaller radius)")
        self.offsets = torch.empty(nn + 1, dtype=torch.int32, device=dev)
        scr = torch.empty(nn // 4096 + 4, dtype=torch.int32, device=dev)
        _chk("aqua_gnn_exclusive_scan", L.aqua_gnn_exclusive_scan(
            nn, _p(deg), _p(self.offsets), _p(scr), s))
        self.n_edges = int(self.offsets[nn].item())
        E = self.n_edges
        self.receivers = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
        self.senders = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
        _chk("aqua_gnn_neighbours", L.aqua_gnn_neighbours(
            nn, dims, _p(self.rs), _p(self.keys), ncell, _p(cstart), _p(cend),
            radius, _vp(0), _p(self.offsets), _p(self.receivers),
            _p(self.senders), s))
        self.ncell = nc
        self.origin = lo

    def gather(self, src, comps, stride=None, stream=None):
        """Node-ordered copy of a per-particle array (f32/i32, comps wide)."""
        torch = _torch()
        out = torch.empty((self.n_nodes, comps) if comps > 1 else self.n_nodes,
                          dtype=src.dtype, device=src.device)
        _chk("aqua_gnn_gather32", lib().aqua_gnn_gather32(
            self.n_nodes, _p(self.perm), _p(src), stride or comps, comps,
            _p(out), _vp(stream or 0)))
        return out


# ------------------------------------------------------------------ model ----

def init_params(seed=0):
    """He-style initial weights {name: (W (N x K), b (N))} (float32)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, n, k, act in LAYERS:
        std = math.sqrt(2.0 / k) if act else math.sqrt(1.0 / k)
        if name == "n2_2":
            std *= 0.1
        p[name] = (rng.normal(0, std, (n, k)).astype(np.float32),
                   np.zeros(n, np.float32))
    return p


class Model:
    """Parameters on the device: FP32 master copy, BF16 weights (and their
    transposes), Adam moments, gradients; one flat buffer each."""

    def __init__(self, dims, params=None, seed=0, device="cuda"):
        torch = _torch()
        self.dims = dims
        self.offs = {}
        o = 0
        for name, n, k, act in LAYERS:
            self.offs[name] = (o, o + n * k, n, k, act)
            o += n * k + n
        self.size = o
        self.flat = torch.zeros(o, dtype=torch.float32, device=device)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.wbf = torch.zeros(o, dtype=torch.bfloat16, device=device)
        self.wt = {name: torch.zeros(k * n, dtype=torch.bfloat16, device=device)
                   for name, n, k, act in LAYERS}
        self.step_count = 0
        # feature scales: h, U, R, A, Rd, rho0; output scales su, srho
        self.scales = torch.ones(6, dtype=torch.float32, device=device)
        self.out_scale = (1.0, 1.0)
        self.set_params(params or init_params(seed))

    def set_params(self, params):
        torch = _torch()
        host = np.zeros(self.size, np.float32)
        for name, (o, ob, n, k, act) in self.offs.items():
            w, b = params[name]
            host[o:o + n * k] = np.asarray(w, np.float32).ravel()
            host[ob:ob + n] = np.asarray(b, np.float32)
        self.flat.copy_(torch.from_numpy(host))
        self._refresh()

    def params(self):
        host = self.flat.cpu().numpy()
        return {name: (host[o:o + n * k].reshape(n, k).copy(), host[ob:ob + n].copy())
                for name, (o, ob, n, k, act) in self.offs.items()}

    def grads(self):
        host = self.grad.cpu().numpy()
        return {name: (host[o:o + n * k].reshape(n, k).copy(), host[ob:ob + n].copy())
                for name, (o, ob, n, k, act) in self.offs.items()}

    def _refresh(self, stream=None):
        L = lib()
        s = _vp(stream or 0)
        _chk("aqua_gnn_to_bf16", L.aqua_gnn_to_bf16(self.size, _p(self.flat),
                                                     _p(self.wbf), s))
        self._transpose(s)

    def _transpose(self, s):
        L = lib()
        for name, (o, ob, n, k, act) in self.offs.items():
            _chk("aqua_gnn_transpose", L.aqua_gnn_transpose(
                n, k, _vp(self.wbf.data_ptr() + 2 * o), _p(self.wt[name]), s))

    def W(self, name):
        return _vp(self.wbf.data_ptr() + 2 * self.offs[name][0])

    def b(self, name):
        return _vp(self.flat.data_ptr() + 4 * self.offs[name][1])

    def dW(self, name):
        return _vp(self.grad.data_ptr() + 4 * self.offs[name][0])

    def db(self, name):
        return _vp(self.grad.data_ptr() + 4 * self.offs[name][1])

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        self.step_count += 1
        s = _vp(stream or 0)
        _chk("aqua_gnn_adam", lib().aqua_gnn_adam(
            self.size, _p(self.flat), _p(self.grad), _p(self.m), _p(self.v),
            lr, beta1, beta2, eps, self.step_count, _p(self.wbf), s))
        self._transpose(s)

    def save(self, path):
        np.savez(path, flat=self.flat.cpu().numpy(),
                 scales=self.scales.cpu().numpy(),
                 out_scale=np.array(self.out_scale, np.float32),
                 dims=np.int32(self.dims))

    @classmethod
    def load(cls, path, device="cuda"):
        torch = _torch()
        d = np.load(path)
        m = cls(int(d["dims"]), device=device)
        m.flat.copy_(torch.from_numpy(d["flat"]))
        m.scales.copy_(torch.from_numpy(d["scales"]))
        m.out_scale = tuple(float(x) for x in d["out_scale"])
        m._refresh()
        return m


class Inputs:
    """Node-ordered particle arrays of one graph (device f32 / i32)."""

    def __init__(self, graph, r, u, rho, dudt, drhodt, imove, normal,
                 stream=None):
        vs = 4 if graph.dims == 3 else 2
        g = graph
        self.r = g.rs
        self.u = g.gather(u, vs, stream=stream)
        self.rho = g.gather(rho, 1, stream=stream)
        self.dudt = g.gather(dudt, vs, stream=stream)
        self.drhodt = g.gather(drhodt, 1, stream=stream)
        self.imove = g.gather(imove, 1, stream=stream)
        self.normal = g.gather(normal, vs, stream=stream)


class Network:
    """Forward (and, with ``train``, backward) of the model on one graph."""

    def __init__(self, model: Model, graph: Graph, inputs: Inputs, stream=None,
                 tcgen05=None, fused=None, fused_sum=None):
        torch = _torch()
        self.model, self.g, self.x = model, graph, inputs
        self.s = _vp(stream or 0)
        self.stream = stream
        self.tc = USE_TCGEN05 if tcgen05 is None else bool(tcgen05)
        self.fused = self.tc and (FUSE_EDGE_MLP if fused is None else bool(fused))
        self.fused_sum = self.fused and (FUSE_EDGE_SUM if fused_sum is None
                                         else bool(fused_sum))
        self.err = torch.zeros(1, dtype=torch.int32, device=graph.rs.device)

    def _buf(self, shape, dtype):
        torch = _torch()
        return torch.empty(shape, dtype=dtype, device=self.g.rs.device)

    def _lin(self, name, X, ldx, M, Z=None, ldz=0, Y=None, ldy=0):
        o, ob, n, k, act = self.model.offs[name]
        if self.tc and n == 64:
            _chk("aqua_gnn_linear_fwd_tc", lib().aqua_gnn_linear_fwd_tc(
                M, k, n, X, ldx, self.model.W(name), self.model.b(name),
                Z, ldz, Y, ldy, act, _p(self.err), self.s))
            return
        _chk("aqua_gnn_linear_fwd", lib().aqua_gnn_linear_fwd(
            M, k, n, X, ldx, self.model.W(name), self.model.b(name),
            Z, ldz, Y, ldy, act, self.s))

    def _mlp(self, prefix, X, ldx, M, keep, out=None, ldo=64):
        """Three layers; returns (A list (bf16), Z list (f32)); the last
        layer's bf16 output goes to ``out`` (rows ldo apart) if given."""
        torch = _torch()
        A, Z = [], []
        cur, ldc = X, ldx
        for k in range(3):
            name = f"{prefix}_{k}"
            n = self.model.offs[name][2]
            z = self._buf((M, n), torch.float32) if (keep and k < 2) else None
            if k < 2:
                y = self._buf((M, n), torch.bfloat16)
                self._lin(name, cur, ldc, M, _p(z) if z is not None else _vp(0), n,
                          _p(y), n)
                A.append(y)
                Z.append(z)
                cur, ldc = _p(y), n
            else:
                if out is None:
                    y = self._buf((M, n), torch.bfloat16)
                    self._lin(name, cur, ldc, M, _vp(0), 0, _p(y), n)
                    A.append(y)
                else:
                    self._lin(name, cur, ldc, M, _vp(0), 0, out, ldo)
        return A, Z

    def _edge_mlp_fused(self, prefix, E, X=None, ldx=0, H=None, ldh=0, Ef=None,
                        out=None, ldo=64):
        """The three layers of an edge MLP in one tcgen05 kernel (inference:
        no activations kept); returns the E x 64 bf16 output, or writes it
        to ``out`` (rows ``ldo`` apart) if given.  The first node MLP (n1,
        80-wide rows) runs through the same kernel."""
        torch = _torch()
        m = self.model
        y = self._buf((max(E, 1), 64), torch.bfloat16) if out is None else None
        names = [f"{prefix}_{k}" for k in range(3)]
        acts = [m.offs[nm][4] for nm in names]
        k1 = m.offs[names[0]][3]
        g = self.g
        _chk("aqua_gnn_edge_mlp_tc", lib().aqua_gnn_edge_mlp_tc(
            E, k1, X or _vp(0), ldx,
            _p(g.receivers) if H is not None else _vp(0),
            _p(g.senders) if H is not None else _vp(0),
            H or _vp(0), ldh, Ef or _vp(0),
            m.W(names[0]), m.b(names[0]), m.W(names[1]), m.b(names[1]),
            m.W(names[2]), m.b(names[2]), acts[0], acts[1], acts[2],
            _p(y) if out is None else out, 64 if out is None else ldo,
            _p(self.err), self.s))
        return y

    def _edge_mlp_sum(self, prefix, out, ld, X=None, ldx=0, H=None, ldh=0,
                      Ef=None):
        """The fused edge MLP summed into the receivers: AGG_SCALE times the
        sum of each node's edge outputs, bf16 at column 0 of ``out`` (rows
        ``ld`` apart)."""
        m = self.model
        names = [f"{prefix}_{k}" for k in range(3)]
        acts = [m.offs[nm][4] for nm in names]
        k1 = m.offs[names[0]][3]
        g = self.g
        _chk("aqua_gnn_edge_mlp_sum_tc", lib().aqua_gnn_edge_mlp_sum_tc(
            g.n_nodes, g.n_edges, k1, X or _vp(0), ldx, _p(g.offsets),
            _p(g.receivers), _p(g.senders) if H is not None else _vp(0),
            H or _vp(0), ldh, Ef or _vp(0),
            m.W(names[0]), m.b(names[0]), m.W(names[1]), m.b(names[1]),
            m.W(names[2]), m.b(names[2]), acts[0], acts[1], acts[2],
            AGG_SCALE, _p(out), ld, 0, _p(self.err), self.s))

    def forward(self, train=False):
        torch = _torch()
        L = lib()
        m, g, x = self.model, self.g, self.x
        n, E, dims = g.n_nodes, g.n_edges, g.dims
        s = self.s
        c = {}
        E0 = self._buf((max(E, 1), FEAT), torch.bfloat16)
        if EDGE_RECORDS:
            rec = self._buf((max(n, 1), 12 if dims == 3 else 8), torch.float32)
            _chk("aqua_gnn_node_records", L.aqua_gnn_node_records(
                n, dims, _p(x.r), _p(x.u), _p(x.rho), _p(x.imove),
                _p(x.normal), _p(rec), s))
            _chk("aqua_gnn_edge_features_rec", L.aqua_gnn_edge_features_rec(
                E, dims, _p(g.receivers), _p(g.senders), _p(rec), _p(m.scales),
                _p(E0), s))
            del rec
        else:
            _chk("aqua_gnn_edge_features", L.aqua_gnn_edge_features(
                E, dims, _p(g.receivers), _p(g.senders), _p(x.r), _p(x.u),
                _p(x.rho), _p(x.imove), _p(x.normal), _p(m.scales), _p(E0), s))
        c["E0"] = E0
        fused = self.fused and not train
        summed = self.fused_sum and not train
        n1_in = self._buf((n, 80), torch.bfloat16)
        if summed:
            self._edge_mlp_sum("e1", n1_in, 80, X=_p(E0), ldx=FEAT)
        else:
            if fused:
                A, Z = [self._edge_mlp_fused("e1", E, X=_p(E0), ldx=FEAT)], []
            else:
                A, Z = self._mlp("e1", _p(E0), FEAT, E, train)
            c["e1"] = (A, Z)
            _chk("aqua_gnn_segment_sum", L.aqua_gnn_segment_sum(
                n, _p(g.offsets), _p(A[-1]), 64, AGG_SCALE, _p(n1_in), 80, 0, s))
            del A, Z
        _chk("aqua_gnn_node_features", L.aqua_gnn_node_features(
            n, dims, _p(x.u), _p(x.rho), _p(x.dudt), _p(x.drhodt), _p(x.imove),
            _p(x.normal), _p(m.scales), _p(n1_in), 80, 64, s))
        c["n1_in"] = n1_in
        n2_in = self._buf((n, 144), torch.bfloat16)
        H = _vp(n2_in.data_ptr() + 2 * 64)
        if fused:
            self._edge_mlp_fused("n1", n, X=_p(n1_in), ldx=80, out=H, ldo=144)
            c["n1"] = ([], [])
        else:
            A, Z = self._mlp("n1", _p(n1_in), 80, n, train, out=H, ldo=144)
            c["n1"] = (A, Z)
        if summed:
            self._edge_mlp_sum("e2", n2_in, 144, H=H, ldh=144, Ef=_p(E0))
        else:
            if fused:
                # the pair inputs are gathered on chip: X2 is never built
                A, Z = [self._edge_mlp_fused("e2", E, H=H, ldh=144,
                                             Ef=_p(E0))], []
            else:
                X2 = self._buf((max(E, 1), 144), torch.bfloat16)
                _chk("aqua_gnn_gather_pair", L.aqua_gnn_gather_pair(
                    E, _p(g.receivers), _p(g.senders), H, 144, _p(E0), _p(X2),
                    s))
                c["X2"] = X2
                A, Z = self._mlp("e2", _p(X2), 144, E, train)
            c["e2"] = (A, Z)
            _chk("aqua_gnn_segment_sum", L.aqua_gnn_segment_sum(
                n, _p(g.offsets), _p(A[-1]), 64, AGG_SCALE, _p(n2_in), 144, 0,
                s))
            del A, Z
        _chk("aqua_gnn_node_features", L.aqua_gnn_node_features(
            n, dims, _p(x.u), _p(x.rho), _p(x.dudt), _p(x.drhodt), _p(x.imove),
            _p(x.normal), _p(m.scales), _p(n2_in), 144, 128, s))
        c["n2_in"] = n2_in
        A2, Z2 = [], []
        cur, ldc = _p(n2_in), 144
        for k in range(2):
            name = f"n2_{k}"
            z = self._buf((n, 64), torch.float32) if train else None
            y = self._buf((n, 64), torch.bfloat16)
            self._lin(name, cur, ldc, n, _p(z) if z is not None else _vp(0), 64,
                      _p(y), 64)
            A2.append(y)
            Z2.append(z)
            cur, ldc = _p(y), 64
        out = self._buf((n, 16), torch.float32)
        self._lin("n2_2", cur, ldc, n, _p(out), 16, None, 0)
        c["n2"] = (A2, Z2)
        self.cache = c
        self.out = out
        if self.tc and int(self.err.item()):
            raise _lib.AquaError("aqua_gnn_linear_fwd_tc (wait timed out)",
                                 _lib.AQUA_ERR_CUDA)
        return out

    def _mlp_bwd(self, prefix, X, ldx, A, Z, dY, M, want_dx, dx_ld=None):
        """Backward through three layers (A[0], A[1] bf16 activations, Z[0],
        Z[1] their pre-activations, X the input).  dY: bf16 M x N of the last
        layer.  Returns dX (bf16, M x K0) or None."""
        torch = _torch()
        L = lib()
        m = self.model
        s = self.s
        ins = [(X, ldx), (_p(A[0]), 64), (_p(A[1]), 64)]
        for k in (2, 1, 0):
            name = f"{prefix}_{k}"
            o, ob, n, kk, act = m.offs[name]
            xin, ldin = ins[k]
            # weight and data gradients on the tensor cores (tcgen05) or on
            # mma.sync
            if self.tc:
                _chk("aqua_gnn_linear_wgrad_tc", L.aqua_gnn_linear_wgrad_tc(
                    M, n, kk, _p(dY), n, xin, ldin, m.dW(name), m.db(name),
                    _p(self.err), s))
            else:
                _chk("aqua_gnn_linear_wgrad", L.aqua_gnn_linear_wgrad(
                    M, n, kk, _p(dY), n, xin, ldin, m.dW(name), m.db(name), s))
            if k == 0 and not want_dx:
                return None
            dX = self._buf((M, kk), torch.bfloat16)
            zp = _p(Z[k - 1]) if k > 0 else _vp(0)
            if self.tc:
                _chk("aqua_gnn_linear_dgrad_tc", L.aqua_gnn_linear_dgrad_tc(
                    M, n, kk, _p(dY), n, _p(m.wt[name]), zp,
                    kk if k > 0 else 0, 1 if k > 0 else 0, _p(dX), kk,
                    _p(self.err), s))
            else:
                _chk("aqua_gnn_linear_dgrad", L.aqua_gnn_linear_dgrad(
                    M, n, kk, _p(dY), n, _p(m.wt[name]), zp,
                    kk if k > 0 else 0, 1 if k > 0 else 0, _p(dX), kk, s))
            dY = dX
        return dY

    def backward(self, dout):
        """dout: bf16 n x 16 gradient of the loss; accumulates into
        model.grad."""
        torch = _torch()
        L = lib()
        g, c, s = self.g, self.cache, self.s
        n, E = g.n_nodes, g.n_edges
        A2, Z2 = c["n2"]
        dn2 = self._mlp_bwd("n2", _p(c["n2_in"]), 144, A2, Z2, dout, n, True)
        # dn2: n x 144 = [d agg2, d h, d features]
        dy = self._buf((max(E, 1), 64), torch.bfloat16)
        _chk("aqua_gnn_segment_bcast", L.aqua_gnn_segment_bcast(
            E, _p(g.receivers), _p(dn2), 144, 0, AGG_SCALE, _p(dy), 64, s))
        A, Z = c["e2"]
        dX2 = self._mlp_bwd("e2", _p(c["X2"]), 144, A, Z, dy, E, True)
        dH = torch.zeros((n, 64), dtype=torch.float32, device=g.rs.device)
        _chk("aqua_gnn_scatter_pair", L.aqua_gnn_scatter_pair(
            n, E, _p(g.offsets), _p(g.senders), _p(dX2), _p(dH), s))
        dh = self._buf((n, 64), torch.bfloat16)
        _chk("aqua_gnn_add_to_bf16", L.aqua_gnn_add_to_bf16(
            n, _p(dH), _p(dn2), 144, 64, _p(dh), 64, 0, s))
        A, Z = c["n1"]
        dn1 = self._mlp_bwd("n1", _p(c["n1_in"]), 80, A, Z, dh, n, True)
        _chk("aqua_gnn_segment_bcast", L.aqua_gnn_segment_bcast(
            E, _p(g.receivers), _p(dn1), 80, 0, AGG_SCALE, _p(dy), 64, s))
        A, Z = c["e1"]
        self._mlp_bwd("e1", _p(c["E0"]), FEAT, A, Z, dy, E, False)
        if self.tc and int(self.err.item()):
            raise _lib.AquaError("tensor-core backward (wait timed out)",
                                 _lib.AQUA_ERR_CUDA)


def mse_loss(out, target, mask, stream=None):
    """Masked MSE (device) -> (loss tensor (1,), dOut bf16 n x 16)."""
    torch = _torch()
    n, t = target.shape
    loss = torch.zeros(1, dtype=torch.float32, device=out.device)
    dout = torch.empty((n, 16), dtype=torch.bfloat16, device=out.device)
    cnt = float(max(int(mask.sum().item()), 1))
    _chk("aqua_gnn_mse", lib().aqua_gnn_mse(
        n, t, _p(out), _p(target), _p(mask), cnt, _p(loss), _p(dout),
        _vp(stream or 0)))
    return loss, dout


# ------------------------------------------------------- batch snapshots ----

STATE_FIELDS = ("id", "iset", "imove", "r", "normal", "tangent", "binormal",
                "u", "dudt", "rho", "drhodt", "m", "p")
_VEC = ("r", "normal", "tangent", "binormal", "u", "dudt")
_U32 = ("id", "iset")


class Snapshot:
    """The particle Variables of a solver's resident batch, in original
    particle order (device tensors)."""

    def __init__(self, n, dims, device="cuda"):
        torch = _torch()
        vs = 4 if dims == 3 else 2
        self.n, self.dims = n, dims
        self.a = {}
        for f in STATE_FIELDS:
            shape = (n, vs) if f in _VEC else (n,)
            dt = torch.int32 if f in _U32 or f == "imove" else torch.float32
            self.a[f] = torch.empty(shape, dtype=dt, device=device)

    def __getitem__(self, k):
        return self.a[k]

    def ptrs(self):
        return {k: v.data_ptr() for k, v in self.a.items()}

    @classmethod
    def capture(cls, solver, dims, stream=None):
        """Reads the resident state and reorders it by particle id."""
        n = solver.N
        raw = cls(n, dims)
        solver.get_state_raw(raw.ptrs(), False, stream)
        out = cls(n, dims)
        L = lib()
        vs = 4 if dims == 3 else 2
        for f in STATE_FIELDS:
            comps = vs if f in _VEC else 1
            _chk("aqua_gnn_scatter32", L.aqua_gnn_scatter32(
                n, _p(raw["id"]), _p(raw[f]), comps, _p(out[f]), comps,
                _vp(stream or 0)))
        return out

    def clone(self):
        c = Snapshot.__new__(Snapshot)
        c.n, c.dims = self.n, self.dims
        c.a = {k: v.clone() for k, v in self.a.items()}
        return c


def case_ids(batch, device="cuda"):
    torch = _torch()
    sizes = np.diff(np.asarray(batch.offsets, np.int64))
    cid = np.repeat(np.arange(len(sizes), dtype=np.int32), sizes)
    return torch.from_numpy(cid).to(device)


# --------------------------------------------------------------- training ----

def collect_pairs(batch, k, n_pairs, gap, warm, fast=True, stream=None):
    """Trajectories of the plain step: ``n_pairs`` snapshot pairs
    (state at t, state at t + k steps), ``gap`` steps apart after ``warm``
    steps.  Returns (pairs, per-pair per-case dt arrays)."""
    from .solver import Solver
    torch = _torch()
    c = batch.case
    sv = Solver(c.params, capacity=c.N,
                ihoc_capacity=batch.n_cases * c.params.max_cells())
    sv.set_precision(fast)
    sv.set_batch(batch)
    if warm:
        sv.step(warm, graph=True, stream=stream)
    pairs, dts = [], []
    for _ in range(n_pairs):
        s0 = Snapshot.capture(sv, c.dims, stream)
        dt = torch.tensor([x["dt"] for x in sv.case_scalars(stream)],
                          dtype=torch.float32, device="cuda")
        sv.step(k, graph=True, stream=stream)
        s1 = Snapshot.capture(sv, c.dims, stream)
        pairs.append((s0, s1))
        dts.append(dt)
        if gap:
            sv.step(gap, graph=True, stream=stream)
    sv.check(stream)
    sv.close()
    return pairs, dts


def fit_scales(model, pairs, dts, k, params, cid):
    """Feature and target scales from the training snapshots (standard
    deviations over fluid particles); ``cid`` = case of each particle."""
    torch = _torch()
    dims = model.dims
    cid = cid.long()
    us, rs, accs, rds, du, dr = [], [], [], [], [], []
    for (s0, s1), dt in zip(pairs[:8], dts[:8]):
        fl = s0["imove"] == 1
        T = (float(k) * dt[cid])[fl]
        u0, u1 = s0["u"][fl, :dims], s1["u"][fl, :dims]
        a0 = s0["dudt"][fl, :dims]
        us.append(u0)
        rs.append(s0["rho"][fl])
        accs.append(a0)
        rds.append(s0["drhodt"][fl])
        du.append(u1 - u0 - T[:, None] * a0)
        dr.append(s1["rho"][fl] - s0["rho"][fl] - T * s0["drhodt"][fl])
    rho0 = float(params.refd[0])

    def sd(xs, floor):
        return max(float(torch.cat([x.reshape(-1) for x in xs]).std().item()), floor)
    h = float(params.h)
    U = sd(us, 1e-3)
    R = max(float(torch.cat(rs).sub(rho0).abs().mean().item()), 1e-3)
    A = sd(accs, 1e-3)
    Rd = sd(rds, 1e-3)
    model.scales.copy_(torch.tensor([h, U, R, A, Rd, rho0], dtype=torch.float32))
    model.out_scale = (sd(du, 1e-9), sd(dr, 1e-9))
    return model.scales.cpu().numpy(), model.out_scale


class Trainer:
    """Adam on the masked MSE of the normalised residual targets."""

    def __init__(self, model, solver, batch, k, lr=1e-3, cases_per_step=16,
                 seed=0, radius=None):
        self.model, self.sv, self.batch, self.k = model, solver, batch, k
        self.lr = lr
        self.cases = cases_per_step
        self.rng = np.random.default_rng(seed)
        self.cid = case_ids(batch)
        self.offsets = np.asarray(batch.offsets, np.int64)
        p = batch.case.params
        # graph radius: the kernel support 2h unless given
        self.radius = float(radius) if radius else float(p.support * p.h)
        self.history = []

    def _slice(self, snap, a, b):
        lo, hi = int(self.offsets[a]), int(self.offsets[b])
        return {f: v[lo:hi] for f, v in snap.a.items()}, lo, hi

    def batch_loss(self, pair, dt, a, b, train=True):
        torch = _torch()
        L = lib()
        dims = self.model.dims
        s0, lo, hi = self._slice(pair[0], a, b)
        s1, _, _ = self._slice(pair[1], a, b)
        n = hi - lo
        cid = self.cid[lo:hi]
        g = Graph(self.sv, dims, s0["r"], s0["imove"], cid, n, self.radius)
        x = Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                   s0["imove"], s0["normal"])
        tgt = torch.empty((g.n_nodes, dims + 1), dtype=torch.float32,
                          device=g.rs.device)
        mask = torch.empty(g.n_nodes, dtype=torch.int32, device=g.rs.device)
        su, srho = self.model.out_scale
        _chk("aqua_gnn_targets", L.aqua_gnn_targets(
            g.n_nodes, dims, _p(g.perm), _p(s0["u"]), _p(s0["rho"]),
            _p(s0["dudt"]), _p(s0["drhodt"]), _p(s1["u"]), _p(s1["rho"]),
            _p(cid), _p(dt), self.k, su, srho, _p(s0["imove"]), _p(tgt),
            _p(mask), _vp(0)))
        net = Network(self.model, g, x)
        out = net.forward(train=train)
        loss, dout = mse_loss(out, tgt, mask)
        return net, loss, dout, g

    def step(self, pairs, dts):
        i = int(self.rng.integers(len(pairs)))
        nc = len(self.offsets) - 1
        a = int(self.rng.integers(0, max(nc - self.cases, 0) + 1))
        b = min(a + self.cases, nc)
        net, loss, dout, g = self.batch_loss(pairs[i], dts[i], a, b)
        self.model.grad.zero_()
        net.backward(dout)
        self.model.adam(self.lr)
        v = float(loss.item())
        self.history.append(v)
        return v


class PairRing:
    """A fixed-capacity ring of plain-step snapshot pairs on the device.
    Each entry is (s0, s1, dt, offsets, cid): the states k steps apart, the
    per-case time steps at s0, and the layout of the batch the pair came
    from (case offsets, case of each particle).  A push past the capacity
    overwrites the oldest entry."""

    def __init__(self, capacity):
        if capacity < 1:
            raise ValueError("ring capacity must be >= 1")
        self.capacity = int(capacity)
        self.items = []
        self.next = 0
        self.pushed = 0

    def __len__(self):
        return len(self.items)

    def push(self, item):
        if len(self.items) < self.capacity:
            self.items.append(item)
        else:
            self.items[self.next] = item
        self.next = (self.next + 1) % self.capacity
        self.pushed += 1

    def sample(self, rng):
        return self.items[int(rng.integers(len(self.items)))]


def online_train(model, k, make_batch, n_runs=256, runs_per_gen=64,
                 capacity=16, warm=20000, gap=300, pairs_per_gen=8,
                 iters_per_pair=10, fit_pairs=4, cases_per_step=16, lr=1e-3,
                 seed=0, fast=True, stream=None):
    """Online training over many plain-solver runs.

    Generations of ``runs_per_gen`` tanks (``make_batch(n_cases, g)`` gives
    generation g's batch; n_runs / runs_per_gen generations) are stepped by
    the plain solver.  After ``warm`` steps each generation emits
    ``pairs_per_gen`` snapshot pairs k steps apart, ``gap`` steps apart,
    into a PairRing of ``capacity`` pairs.  After each emission the trainer
    takes ``iters_per_pair`` Adam steps, each on a pair drawn from the ring
    and ``cases_per_step`` consecutive tanks of it.  The feature and target
    scales are fitted on generation 0's first ``fit_pairs`` pairs before
    the first step.  Returns the statistics of the run."""
    from .solver import Solver
    torch = _torch()
    rng = np.random.default_rng(seed)
    ring = PairRing(capacity)
    gens = max(1, int(n_runs) // int(runs_per_gen))
    tr = None
    sv_graph = None
    graph_cap = 0
    iters = 0
    losses = []
    t_gen = t_train = 0.0
    for gi in range(gens):
        t0 = time.perf_counter()
        batch = make_batch(runs_per_gen, gi)
        c = batch.case
        sv = Solver(c.params, capacity=c.N,
                    ihoc_capacity=batch.n_cases * c.params.max_cells())
        sv.set_precision(fast)
        sv.set_batch(batch)
        if warm:
            sv.step(warm, graph=True, stream=stream)
        offsets = np.asarray(batch.offsets, np.int64)
        cid = case_ids(batch)
        pending = []
        for pi in range(pairs_per_gen):
            s0 = Snapshot.capture(sv, c.dims, stream)
            dt = torch.tensor([x["dt"] for x in sv.case_scalars(stream)],
                              dtype=torch.float32, device="cuda")
            sv.step(k, graph=True, stream=stream)
            s1 = Snapshot.capture(sv, c.dims, stream)
            item = (s0, s1, dt, offsets, cid)
            ring.push(item)
            if gap and pi + 1 < pairs_per_gen:
                sv.step(gap, graph=True, stream=stream)
            if tr is None:
                # the scales from generation 0's first pairs, then training
                pending.append(item)
                if len(pending) < min(fit_pairs, pairs_per_gen):
                    continue
                fit_scales(model, [(a, b) for a, b, _, _, _ in pending],
                           [d for _, _, d, _, _ in pending], k, c.params, cid)
                # the graph context (grown when a slice does not fit)
                graph_cap = c.N
                sv_graph = Solver(c.params, capacity=graph_cap)
                tr = Trainer(model, sv_graph, batch, k, lr=lr,
                             cases_per_step=cases_per_step, seed=seed)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            t_gen += t1 - t0
            for _ in range(iters_per_pair):
                s0_, s1_, dt_, off_, cid_ = ring.sample(rng)
                tr.offsets, tr.cid = off_, cid_
                nc = len(off_) - 1
                a = int(rng.integers(0, max(nc - cases_per_step, 0) + 1))
                b = min(a + cases_per_step, nc)
                n_slice = int(off_[b] - off_[a])
                if n_slice > graph_cap:
                    # a larger slice than any before: a larger graph context
                    sv_graph.close()
                    graph_cap = n_slice + n_slice // 4
                    sv_graph = Solver(c.params, capacity=graph_cap)
                    tr.sv = sv_graph
                net, loss, dout, _ = tr.batch_loss((s0_, s1_), dt_, a, b)
                model.grad.zero_()
                net.backward(dout)
                model.adam(lr)
                losses.append(float(loss.item()))
                iters += 1
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            t_train += t0 - t1
        sv.check(stream)
        sv.close()
        t_gen += time.perf_counter() - t0
    if sv_graph is not None:
        sv_graph.close()
    return {"runs": gens * int(runs_per_gen), "generations": gens,
            "runs_per_generation": int(runs_per_gen), "ring_capacity": capacity,
            "pairs_pushed": ring.pushed, "iterations": iters,
            "warm_steps": warm, "gap_steps": gap, "cases_per_step": cases_per_step,
            "loss_first": losses[0] if losses else None,
            "loss_last10": float(np.mean(losses[-10:])) if losses else None,
            "generate_s": t_gen, "train_s": t_train}


# ---------------------------------------------------------------- proposal ----

class ProposalRunner:
    """Advances a resident batch by learned k-step proposals with a plain
    judge on a sampled subset of the cases.

    Each ``advance()``: the network proposes the state k plain steps ahead
    for every case (walls and probes follow the prescribed roll); a
    fraction ``judge_fraction`` of the cases, sampled anew each time, is
    re-run from the same state by the plain step; a judged case whose probe
    pressure departs from the plain one by more than ``tol`` of
    max(|p_plain|, p_floor), or whose fluid density departs by more than
    ``tol`` of refd anywhere, takes the plain state instead (rollback)."""

    def __init__(self, solver, batch, model, k=8, judge_fraction=0.25,
                 tol=0.02, p_floor=None, seed=0, fast=True):
        from .solver import Solver
        torch = _torch()
        self.sv, self.batch, self.model, self.k = solver, batch, model, k
        self.dims = batch.case.dims
        self.frac, self.tol = judge_fraction, tol
        self.rng = np.random.default_rng(seed)
        p = batch.case.params
        self.params = p
        self.radius = float(p.support * p.h)
        self.refd = float(p.refd[0])
        g = abs(float(np.asarray(p.g)[1 if self.dims == 2 else 2]))
        self.p_floor = p_floor if p_floor is not None else self.refd * g * 4 * p.h
        self.cid = case_ids(batch)
        self.offsets = np.asarray(batch.offsets, np.int64)
        self.off_dev = torch.from_numpy(self.offsets.astype(np.int32)).cuda()
        # host array: the constants are kernel arguments
        self.consts = (C.c_float * 6)(p.H, p.CONW, p.SUPPORT, p.cs, p.p0,
                                      self.refd)
        n_cases = len(self.offsets) - 1
        self.n_judge = max(1, int(round(judge_fraction * n_cases)))
        sizes = np.diff(self.offsets)
        cap = int(np.sort(sizes)[-self.n_judge:].sum())
        self.judge = Solver(p, capacity=cap,
                            ihoc_capacity=self.n_judge * p.max_cells())
        self.judge.set_precision(fast)
        self.stats = {"proposals": 0, "judged": 0, "rolled_back": 0,
                      "p_err": [], "rho_err": []}

    def close(self):
        self.judge.close()

    def _motion_arrays(self, scal, T):
        torch = _torch()
        n = len(self.batch.motions)
        en = np.zeros(n, np.int32)
        iset = np.zeros(n, np.uint32)
        p0 = np.zeros(n, np.float32)
        p1 = np.zeros(n, np.float32)
        w1 = np.zeros(n, np.float32)
        cen = np.zeros((n, 4), np.float32)
        for c, m in enumerate(self.batch.motions):
            if m is None:
                continue
            t0 = float(scal[c]["t"])
            t1 = t0 + float(T[c])
            en[c] = 1
            iset[c] = m.iset
            p0[c] = m.amplitude * math.sin(m.angular_freq * t0)
            p1[c] = m.amplitude * math.sin(m.angular_freq * t1)
            w1[c] = m.amplitude * m.angular_freq * math.cos(m.angular_freq * t1)
            cen[c, :len(m.center)] = m.center
        dev = lambda a: torch.from_numpy(a).cuda()
        return (dev(en), dev(iset.view(np.int32)), dev(p0), dev(p1), dev(w1),
                dev(cen))

    def advance(self):
        """One proposal of k steps for the whole batch (synchronises)."""
        torch = _torch()
        L = lib()
        dims, k = self.dims, self.k
        vs = 4 if dims == 3 else 2
        scal = self.sv.case_scalars()
        dt = torch.tensor([x["dt"] for x in scal], dtype=torch.float32,
                          device="cuda")
        T = np.array([k * x["dt"] for x in scal], np.float64)
        s0 = Snapshot.capture(self.sv, dims)
        n = s0.n
        # ---- proposal for every case
        g = Graph(self.sv, dims, s0["r"], s0["imove"], self.cid, n, self.radius)
        x = Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                   s0["imove"], s0["normal"])
        out = Network(self.model, g, x).forward(train=False)
        s1 = s0.clone()
        su, srho = self.model.out_scale
        _chk("aqua_gnn_apply", L.aqua_gnn_apply(
            g.n_nodes, dims, _p(g.perm), _p(out), _p(self.cid), _p(dt), k, su,
            srho, _p(s1["r"]), _p(s1["u"]), _p(s1["rho"]), _p(s0["dudt"]),
            _p(s0["drhodt"]), _p(s0["imove"]), _vp(0)))
        en, iset, p0, p1, w1, cen = self._motion_arrays(scal, T)
        _chk("aqua_gnn_roll", L.aqua_gnn_roll(
            n, dims, _p(self.cid), _p(s1["iset"]), _p(s1["imove"]), _p(en),
            _p(iset), _p(p0), _p(p1), _p(w1), _p(cen), _p(s1["r"]),
            _p(s1["normal"]), _p(s1["tangent"]), _p(s1["u"]), _vp(0)))
        # ---- plain judge on a sampled subset of the cases
        n_cases = len(self.offsets) - 1
        judged = np.sort(self.rng.choice(n_cases, self.n_judge, replace=False))
        idx = np.concatenate([np.arange(self.offsets[c], self.offsets[c + 1])
                              for c in judged]).astype(np.int32)
        sub_sizes = np.array([self.offsets[c + 1] - self.offsets[c]
                              for c in judged], np.int64)
        sub_off = np.concatenate([[0], np.cumsum(sub_sizes)]).astype(np.int64)
        perm = torch.from_numpy(idx).cuda()
        m = len(idx)
        packed = Snapshot(m, dims)
        for f in STATE_FIELDS:
            comps = vs if f in _VEC else 1
            _chk("aqua_gnn_gather32", L.aqua_gnn_gather32(
                m, _p(perm), _p(s0[f]), comps, comps, _p(packed[f]), _vp(0)))
        packed["id"].copy_(torch.arange(m, dtype=torch.int32, device="cuda"))
        from .case import Batch
        sub = Batch.__new__(Batch)
        sub.offsets = sub_off
        sub.motions = [self.batch.motions[c] for c in judged]
        self.judge.set_state_raw(m, packed.ptrs(), False, scal[judged[0]]["t"],
                                 scal[judged[0]]["dt"], scal[judged[0]]["iter"])
        self._set_cases(self.judge, sub, [scal[c] for c in judged])
        self.judge.step(k, graph=True)
        self.judge.check()
        plain = Snapshot.capture(self.judge, dims)
        # proposal restricted to the judged cases, same packed order
        prop = Snapshot(m, dims)
        for f in ("r", "rho", "m", "imove"):
            comps = vs if f in _VEC else 1
            _chk("aqua_gnn_gather32", L.aqua_gnn_gather32(
                m, _p(perm), _p(s1[f]), comps, comps, _p(prop[f]), _vp(0)))
        so = torch.from_numpy(sub_off.astype(np.int32)).cuda()
        pp = torch.empty(len(judged), dtype=torch.float32, device="cuda")
        pj = torch.empty_like(pp)
        er = torch.empty_like(pp)
        _chk("aqua_gnn_probe_pressure", L.aqua_gnn_probe_pressure(
            len(judged), dims, _p(so), _p(prop["r"]), _p(prop["rho"]),
            _p(prop["m"]), _p(prop["imove"]), self.consts, _p(pp), _vp(0)))
        _chk("aqua_gnn_probe_pressure", L.aqua_gnn_probe_pressure(
            len(judged), dims, _p(so), _p(plain["r"]), _p(plain["rho"]),
            _p(plain["m"]), _p(plain["imove"]), self.consts, _p(pj), _vp(0)))
        _chk("aqua_gnn_case_max_diff", L.aqua_gnn_case_max_diff(
            len(judged), _p(so), _p(prop["rho"]), _p(plain["rho"]),
            _p(prop["imove"]), 1.0 / self.refd, _p(er), _vp(0)))
        pp, pj, er = pp.cpu().numpy(), pj.cpu().numpy(), er.cpu().numpy()
        p_err = np.abs(pp - pj) / np.maximum(np.abs(pj), self.p_floor)
        bad = (p_err > self.tol) | (er > self.tol)
        # ---- rollback: judged cases that failed take the plain state
        for j, c in enumerate(judged):
            if not bad[j]:
                continue
            lo, hi = int(sub_off[j]), int(sub_off[j + 1])
            glo = int(self.offsets[c])
            for f in STATE_FIELDS:
                if f == "id":
                    continue
                s1[f][glo:glo + (hi - lo)].copy_(plain[f][lo:hi])
        self.stats["proposals"] += 1
        self.stats["judged"] += len(judged)
        self.stats["rolled_back"] += int(bad.sum())
        self.stats["p_err"].extend(p_err.tolist())
        self.stats["rho_err"].extend(er.tolist())
        # ---- the proposal (with rollbacks) becomes the resident state
        s1["id"].copy_(torch.arange(n, dtype=torch.int32, device="cuda"))
        self.sv.set_state_raw(n, s1.ptrs(), False, scal[0]["t"] + T[0],
                              scal[0]["dt"], scal[0]["iter"] + k)
        new = [dict(x) for x in scal]
        for c, x in enumerate(new):
            x["t"] = float(x["t"]) + T[c]
            x["iter"] = int(x["iter"]) + k
        self._set_cases(self.sv, self.batch, new)
        return p_err, er, judged

    @staticmethod
    def _set_cases(solver, batch, scal):
        """aqua_set_cases with explicit per-case scalars."""
        n = len(batch.offsets) - 1
        offs = np.ascontiguousarray(batch.offsets, np.uint32)
        arr = (_lib.AquaCase * n)()
        for c, m in enumerate(batch.motions):
            a = arr[c]
            a.t, a.dt, a.iter = scal[c]["t"], scal[c]["dt"], scal[c]["iter"]
            if m is not None:
                a.roll_enabled = 1
                a.roll_iset = m.iset
                a.roll_amplitude = m.amplitude
                a.roll_angular_freq = m.angular_freq
                a.roll_center[:] = (list(m.center) + [0.0] * 4)[:4]
        _lib.check("aqua_set_cases", solver.lib.aqua_set_cases(
            solver.ctx, n, offs.ctypes.data_as(_lib._U), arr, _vp(0)))
        solver.n_cases = n


class FieldProposalRunner:
    """Advances one large case by learned k-step proposals, each judged by
    the plain method on a 10% sample.

    Each ``advance()``: the network proposes the state k plain steps ahead
    (graph radius ``radius``, default 0.9 h: with h = 2 dx, the 26 nearest
    lattice neighbours).  The judge evaluates the plain rates (one step of
    the plain pipeline, cfd/Rates.cl:55-77 with basic/deltaSPH.cl:330-350)
    at the start state and at the proposed state, each on the same hashed
    sample of the cells (a fraction ``rho_sample`` of them, drawn anew each
    proposal, plus every cell around a probe: ``aqua_set_rate_sample``), in
    a second solver context.  Over the k steps the plain continuity
    equation gives each sampled particle the density rho0 + k dt (drho/dt0
    + drho/dt1) / 2 (trapezoidal rule); the proposal fails where a sampled
    fluid particle's proposed density departs from it by more than ``tol``
    of refd, or where a probe's pressure (Shepard-interpolated,
    ``aqua_gnn_probes_pressure``) from the proposed densities departs by
    more than ``tol`` of max(|p|, p_floor) from the same interpolation of
    the plain densities.  A failed proposal is rolled back: the resident
    state, still the start state, is advanced by k plain steps instead."""

    def __init__(self, solver, case, model, k=8, radius=None, rho_sample=0.1,
                 tol=0.02, p_floor=None, seed=0, fast=True):
        from .solver import Solver
        torch = _torch()
        self.sv, self.model, self.k = solver, model, k
        self.dims = case.dims
        p = case.params
        self.params = p
        self.radius = float(radius) if radius else 0.9 * float(p.h)
        self.tol = tol
        self.rng = np.random.default_rng(seed)
        self.refd = float(p.refd[0])
        g = abs(float(np.asarray(p.g)[1 if self.dims == 2 else 2]))
        self.p_floor = p_floor if p_floor is not None else self.refd * g * 4 * p.h
        self.n = case.N
        self.cid = torch.zeros(case.N, dtype=torch.int32, device="cuda")
        self.consts = (C.c_float * 6)(p.H, p.CONW, p.SUPPORT, p.cs, p.p0,
                                      self.refd)
        # particles in original order (= id): the probes
        imove = np.asarray(case.imove)
        probes = np.nonzero(imove == 0)[0].astype(np.int32)
        if len(probes) > MAX_PROBES:
            raise ValueError(f"at most {MAX_PROBES} probes")
        self.probes = torch.from_numpy(probes).cuda()
        self.rho_sample = float(rho_sample)
        self.scratch = torch.empty(PROBE_SCRATCH, dtype=torch.float32,
                                   device="cuda")
        self.judge = Solver(p, capacity=case.N)
        self.judge.set_precision(fast)
        n = case.N
        self._icell = torch.empty(n, dtype=torch.int32, device="cuda")
        self._raw = Snapshot(n, self.dims)
        self._icell0 = torch.empty(n, dtype=torch.int32, device="cuda")
        self._drho0 = torch.empty(n, dtype=torch.float32, device="cuda")
        self._rho_j = torch.empty(n, dtype=torch.float32, device="cuda")
        self._res = torch.empty(1, dtype=torch.float32, device="cuda")
        self.stats = {"proposals": 0, "rolled_back": 0, "p_err": [],
                      "rho_err": [], "n_edges": 0, "phase_s": {}}

    def _phase(self, name, t0):
        torch = _torch()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ph = self.stats["phase_s"]
        ph[name] = ph.get(name, 0.0) + (t1 - t0)
        return t1

    def probe_pressures(self, snap, rho=None):
        """Pressure at every probe of a snapshot (device, one per probe),
        from the snapshot's densities or from `rho` (by particle id)."""
        torch = _torch()
        out = torch.empty(len(self.probes), dtype=torch.float32, device="cuda")
        _chk("aqua_gnn_probes_pressure", lib().aqua_gnn_probes_pressure(
            snap.n, self.dims, _p(snap["r"]), _p(snap["rho"] if rho is None else rho),
            _p(snap["m"]), _p(snap["imove"]), len(self.probes), _p(self.probes),
            self.consts, _p(self.scratch), _p(out), _vp(0)))
        return out

    def _plain_rates(self, snap, sc):
        """One plain step of the judge context from `snap` with the rate
        sample on; leaves its sorted state in self._raw and its cell keys in
        self._icell."""
        self.judge.set_state_raw(self.n, snap.ptrs(), False, sc["t"], sc["dt"],
                                 sc["iter"])
        self.judge.step(1, graph=False)
        self.judge.check()
        self.judge.get_state_raw(self._raw.ptrs(), False)
        self.judge.get_icell_raw(self._icell.data_ptr())

    def advance(self):
        """One proposal of k steps (synchronises)."""
        torch = _torch()
        L = lib()
        dims, k, n = self.dims, self.k, self.n
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = self.sv.scalars()
        dt = torch.tensor([sc["dt"]], dtype=torch.float32, device="cuda")
        s0 = Snapshot.capture(self.sv, dims)
        t0 = self._phase("snapshot", t0)
        # ---- proposal
        g = Graph(self.sv, dims, s0["r"], s0["imove"], self.cid, n, self.radius)
        self.stats["n_edges"] = g.n_edges
        t0 = self._phase("graph", t0)
        x = Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                   s0["imove"], s0["normal"])
        out = Network(self.model, g, x).forward(train=False)
        s1 = s0.clone()
        su, srho = self.model.out_scale
        _chk("aqua_gnn_apply", L.aqua_gnn_apply(
            g.n_nodes, dims, _p(g.perm), _p(out), _p(self.cid), _p(dt), k, su,
            srho, _p(s1["r"]), _p(s1["u"]), _p(s1["rho"]), _p(s0["dudt"]),
            _p(s0["drhodt"]), _p(s0["imove"]), _vp(0)))
        del x, out, g
        t0 = self._phase("network", t0)
        # ---- judge: plain rates at both ends on one cell sample
        seed = int(self.rng.integers(0, 2 ** 32))
        self.judge.set_rate_sample(self.rho_sample, seed)
        self._plain_rates(s0, sc)
        raw = self._raw
        _chk("aqua_gnn_scatter32", L.aqua_gnn_scatter32(
            n, _p(raw["id"]), _p(self._icell), 1, _p(self._icell0), 1, _vp(0)))
        _chk("aqua_gnn_scatter32", L.aqua_gnn_scatter32(
            n, _p(raw["id"]), _p(raw["drhodt"]), 1, _p(self._drho0), 1, _vp(0)))
        self._plain_rates(s1, sc)
        _chk("aqua_gnn_judge_density", L.aqua_gnn_judge_density(
            n, _p(raw["id"]), _p(self._icell), _p(raw["imove"]),
            _p(raw["drhodt"]), _p(self._icell0), _p(self._drho0),
            _p(s0["rho"]), _p(s1["rho"]), float(k * sc["dt"]), 1.0 / self.refd,
            self.rho_sample, seed, _p(self._rho_j), _p(self._res), _vp(0)))
        pp = self.probe_pressures(s1).cpu().numpy()
        pj = self.probe_pressures(s1, self._rho_j).cpu().numpy()
        p_err = np.abs(pp - pj) / np.maximum(np.abs(pj), self.p_floor)
        rho_err = float(self._res.item())
        bad = bool((p_err > self.tol).any() or rho_err > self.tol)
        t0 = self._phase("judge", t0)
        # ---- rollback (k plain steps from the start state, which is still
        # resident) or the proposal becomes resident
        if bad:
            self.sv.step(k, graph=True)
            self.sv.check()
            t0 = self._phase("rollback", t0)
        else:
            self.sv.set_state_raw(n, s1.ptrs(), False, sc["t"] + k * sc["dt"],
                                  sc["dt"], sc["iter"] + k)
            t0 = self._phase("set_state", t0)
        st = self.stats
        st["proposals"] += 1
        st["rolled_back"] += int(bad)
        st["p_err"].extend(p_err.tolist())
        st["rho_err"].append(rho_err)
        return p_err, rho_err, bad

    def close(self):
        self.judge.close()
