"""The learned proposal on one 3-D case, judged by the plain rates on a
cell sample (FieldProposalRunner): the multi-probe pressure kernel against
numpy, the 3-D network forward with the receiver sums fused in against the
unfused kernels, training on a 3-D trajectory, and the accept / rollback
decisions of the runner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from aquagpusph_gb300 import case as cases


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def small_3d():
    c = cases.dam_break_3d(dx=0.01, tank=(0.3, 0.1, 0.2), block=(0.12, 0.1, 0.1),
                           probes_z=(0.02, 0.06))
    c.dt = c.params.dt_fixed
    return c


def probes_numpy(c, r, rho, m, imove, probes):
    """Shepard-normalised pressure at each probe, float64."""
    p = c.params
    out = []
    fl = imove == 1
    rf, rhof, mf = r[fl, :3].astype(np.float64), rho[fl].astype(np.float64), m[fl]
    pj = p.p0 + p.cs ** 2 * (rhof - float(p.refd[0]))
    for k in probes:
        q = np.linalg.norm(rf - r[k, :3], axis=1) / p.H
        a = np.clip(2.0 - q, 0.0, None)
        w = 21.0 / (256.0 * np.pi) * (1 + 2 * q) * a ** 4 * p.CONW * mf / rhof
        w[q >= p.SUPPORT] = 0.0
        sw = w.sum()
        out.append((pj * w).sum() / (sw if sw >= 1e-6 else 1.0))
    return np.array(out)


def test_probes_pressure_matches_numpy(torch):
    from aquagpusph_gb300 import learned as Lm
    c = small_3d()
    rng = np.random.default_rng(3)
    n = c.N
    rho = (998.0 + rng.normal(0, 2.0, n)).astype(np.float32)
    probes = np.nonzero(c.imove == 0)[0]
    # a third probe inside the water, where the sums are full
    inner = int(np.nonzero(c.imove == 1)[0][len(probes) * 977 % 1000])
    imove = c.imove.copy()
    imove[inner] = 0
    probes = np.sort(np.append(probes, inner))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    r, rhod, m, im = dev(c.r), dev(rho), dev(c.m), dev(imove)
    pr = dev(probes.astype(np.int32))
    consts = (Lm.C.c_float * 6)(c.params.H, c.params.CONW, c.params.SUPPORT,
                                c.params.cs, c.params.p0, float(c.params.refd[0]))
    scratch = torch.empty(Lm.PROBE_SCRATCH, dtype=torch.float32, device="cuda")
    out = torch.empty(len(probes), dtype=torch.float32, device="cuda")
    L = Lm.lib()
    assert L.aqua_gnn_probes_pressure(n, 3, Lm._p(r), Lm._p(rhod), Lm._p(m),
                                      Lm._p(im), len(probes), Lm._p(pr), consts,
                                      Lm._p(scratch), Lm._p(out), None) == 0
    got = out.cpu().numpy()
    ref = probes_numpy(c, c.r, rho, c.m, imove, probes)
    assert np.all(np.abs(got - ref) <= 1e-4 * np.maximum(np.abs(ref), 100.0)), (got, ref)
    # deterministic: a second call gives the same bits
    out2 = torch.empty_like(out)
    assert L.aqua_gnn_probes_pressure(n, 3, Lm._p(r), Lm._p(rhod), Lm._p(m),
                                      Lm._p(im), len(probes), Lm._p(pr), consts,
                                      Lm._p(scratch), Lm._p(out2), None) == 0
    assert torch.equal(out, out2)
    # more probes than the kernel holds
    assert L.aqua_gnn_probes_pressure(n, 3, Lm._p(r), Lm._p(rhod), Lm._p(m),
                                      Lm._p(im), Lm.MAX_PROBES + 1, Lm._p(pr),
                                      consts, Lm._p(scratch), Lm._p(out),
                                      None) == -1


def lowbias32(x):
    x = np.asarray(x, np.uint64) & 0xffffffff
    x ^= x >> 16
    x = (x * 0x7feb352d) & 0xffffffff
    x ^= x >> 15
    x = (x * 0x846ca68b) & 0xffffffff
    x ^= x >> 16
    return x


@pytest.mark.parametrize("frac", [0.0, 0.1, 0.5, 1.0])
def test_sample_max_diff_matches_numpy(torch, frac):
    """The subsampled density check picks the particles whose hash of
    (index, seed) is below frac * 2^32 and returns their largest scaled
    difference; a NaN counts as infinite."""
    from aquagpusph_gb300 import learned as Lm
    L = Lm.lib()
    rng = np.random.default_rng(int(frac * 10))
    n = 100003
    a = rng.normal(0, 1, n).astype(np.float32)
    b = rng.normal(0, 1, n).astype(np.float32)
    imove = rng.choice(np.array([1, 1, 1, -3, 0], np.int32), n)
    seed = 0x9e3779b9
    below = min(int(frac * 2.0 ** 32), 0xffffffff)
    idx = np.arange(n, dtype=np.uint64)
    take = (imove == 1) & (lowbias32(idx ^ lowbias32(seed)) < below)
    ref = float((np.abs(a - b) * np.float32(0.25))[take].max()) if take.any() else 0.0
    dev = lambda x: torch.from_numpy(x).cuda()
    out = torch.empty(1, dtype=torch.float32, device="cuda")
    assert L.aqua_gnn_sample_max_diff(n, Lm._p(dev(a)), Lm._p(dev(b)),
                                      Lm._p(dev(imove)), seed, frac, 0.25,
                                      Lm._p(out), None) == 0
    assert float(out.item()) == ref
    if take.any():
        a2 = a.copy()
        a2[np.nonzero(take)[0][0]] = np.nan
        assert L.aqua_gnn_sample_max_diff(n, Lm._p(dev(a2)), Lm._p(dev(b)),
                                          Lm._p(dev(imove)), seed, frac, 0.25,
                                          Lm._p(out), None) == 0
        assert float(out.item()) == np.inf


def trained_model(torch, c, iters):
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    tb = cases.pack([c])
    radius = 0.9 * c.params.h
    pairs, dts = Lm.collect_pairs(tb, 8, n_pairs=6, gap=20, warm=20)
    model = Lm.Model(3, seed=0)
    Lm.fit_scales(model, pairs, dts, 8, c.params, Lm.case_ids(tb))
    sv = Solver(c.params, capacity=c.N)
    tr = Lm.Trainer(model, sv, tb, 8, lr=1e-3, cases_per_step=1, radius=radius)
    first = [float(tr.batch_loss(pairs[i], dts[i], 0, 1, train=False)[1].item())
             for i in range(len(pairs))]
    for _ in range(iters):
        tr.step(pairs, dts)
    last = [float(tr.batch_loss(pairs[i], dts[i], 0, 1, train=False)[1].item())
            for i in range(len(pairs))]
    sv.close()
    return model, float(np.mean(first)), float(np.mean(last))


def test_3d_training_and_fused_forward(torch):
    """A 3-D network trains on plain 3-D trajectories (the loss falls) and
    its inference forward with the receiver sums on chip equals the
    layer-by-layer one bit for bit."""
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    c = small_3d()
    model, first, last = trained_model(torch, c, 60)
    assert np.isfinite(last) and last < first
    sv = Solver(c.params, capacity=c.N)
    sv.set_case(c)
    s0 = Lm.Snapshot.capture(sv, 3)
    cid = torch.zeros(c.N, dtype=torch.int32, device="cuda")
    g = Lm.Graph(sv, 3, s0["r"], s0["imove"], cid, s0.n, 0.9 * c.params.h)
    # interior fluid nodes have the 26 lattice neighbours at 0.9 h
    assert 8 * g.n_nodes < g.n_edges < 40 * g.n_nodes
    x = Lm.Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                  s0["imove"], s0["normal"])
    outs = [Lm.Network(model, g, x, tcgen05=True, fused=f, fused_sum=fs)
            .forward(train=False).clone()
            for f, fs in ((False, False), (True, True))]
    assert torch.equal(outs[0], outs[1])
    sv.close()


def test_field_runner_accepts_and_rolls_back(torch):
    """With an infinite tolerance every proposal stands (the resident state
    is the network's proposal and t advances by k dt); with a zero one every
    proposal is rolled back: the resident state is then that of k plain
    steps from the start state, bit for bit."""
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    c = small_3d()
    model, _, _ = trained_model(torch, c, 20)
    for tol, expect_bad in ((np.inf, False), (0.0, True)):
        sv = Solver(c.params, capacity=c.N)
        sv.set_case(c)
        sv.step(5, graph=True)
        run = Lm.FieldProposalRunner(sv, c, model, k=8, tol=tol, seed=1)
        for _ in range(2):
            t0 = sv.scalars()
            s0 = Lm.Snapshot.capture(sv, 3)
            p_err, rho_err, bad = run.advance()
            assert bad is expect_bad
            assert np.all(np.isfinite(p_err)) and len(p_err) == 2
            assert np.isfinite(rho_err)
            t1 = sv.scalars()
            assert t1["iter"] == t0["iter"] + 8
            if expect_bad:
                ref = Solver(c.params, capacity=c.N)
                ref.set_state_raw(c.N, s0.ptrs(), False, t0["t"], t0["dt"],
                                  t0["iter"])
                ref.step(8, graph=True)
                ref.check()
                assert t1["t"] == ref.scalars()["t"]
                mine = Lm.Snapshot.capture(sv, 3)
                plain = Lm.Snapshot.capture(ref, 3)
                for f in ("r", "u", "rho"):
                    assert torch.equal(mine[f], plain[f]), f
                ref.close()
            else:
                assert abs(t1["t"] - (t0["t"] + 8 * t0["dt"])) <= 1e-6 * max(t1["t"], 1e-3)
        st = run.stats
        assert st["proposals"] == 2
        assert st["rolled_back"] == (2 if expect_bad else 0)
        assert st["n_edges"] > 0
        assert "judge" in st["phase_s"]
        run.close()
        sv.close()


def test_rate_sample_sweeps_only_its_cells(torch):
    """aqua_set_rate_sample: a step from a state with dt = 0 leaves the
    positions as they were, and with the sample on its rates equal the
    full step's on the sampled cells and around the probes; the judge's
    trapezoidal density of a state against itself (k dt = 0) is exact."""
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    c = small_3d()
    c.dt = c.params.dt_fixed
    out = {}
    for frac in (1.0, 0.3):
        sv = Solver(c.params, capacity=c.N)
        sv.set_precision(True)
        sv.set_rate_sample(frac, 7)
        sv.set_case(c)
        sv.step(1, graph=False)
        sv.check()
        g = sv.get_case()
        ex = sv.get_extra()
        out[frac] = (g, ex["icell"])
        sv.close()
    full, _ = out[1.0]
    samp, icell = out[0.3]
    assert np.array_equal(full.id, samp.id)
    h = np.array([_hash(int(k), 7) for k in icell], np.uint64)
    sampled = h < int(0.3 * 2 ** 32)
    fl = full.imove == 1
    assert 0.1 < sampled[fl].mean() < 0.5
    for f in ("dudt", "drhodt", "u", "rho", "r"):
        a, b = getattr(full, f), getattr(samp, f)
        assert np.array_equal(a[sampled & fl], b[sampled & fl]), f
    # unsampled cells away from the probes keep the gather's values: some
    # fluid rates differ from the full step's
    assert not np.array_equal(full.drhodt[~sampled & fl], samp.drhodt[~sampled & fl])


def _hash(key, seed):
    """sample_hash of the library (aqua_internal.cuh), in Python."""
    M = 0xFFFFFFFF
    h = ((key * 0x9E3779B1) & M) ^ ((seed * 0x85EBCA77 + 0x165667B1) & M)
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & M
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & M
    h ^= h >> 16
    return h


@pytest.mark.parametrize("dims", [2, 3])
def test_edge_features_from_records_equal_the_field_form(torch, dims):
    """aqua_gnn_edge_features_rec on the packed node records writes the same
    bits as aqua_gnn_edge_features on the separate node arrays."""
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    if dims == 3:
        c = small_3d()
        b = cases.pack([c])
    else:
        b = cases.sloshing_batch_2d(n_cases=3, seed=5, dx=0.02)
        c = b.case
    sv = Solver(c.params, capacity=c.N,
                ihoc_capacity=(len(b.offsets) - 1) * c.params.max_cells())
    sv.set_batch(b)
    sv.step(3, graph=True)
    s0 = Lm.Snapshot.capture(sv, dims)
    cid = Lm.case_ids(b)
    g = Lm.Graph(sv, dims, s0["r"], s0["imove"], cid, s0.n,
                 float(c.params.support * c.params.h))
    x = Lm.Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                  s0["imove"], s0["normal"])
    L = Lm.lib()
    sc = torch.tensor((float(c.params.h), 0.05, 0.5, 0.5, 5.0, 998.0),
                      dtype=torch.float32, device="cuda")
    E, n = g.n_edges, g.n_nodes
    ref = torch.empty((E, 16), dtype=torch.bfloat16, device="cuda")
    assert L.aqua_gnn_edge_features(E, dims, Lm._p(g.receivers),
                                    Lm._p(g.senders), Lm._p(x.r), Lm._p(x.u),
                                    Lm._p(x.rho), Lm._p(x.imove),
                                    Lm._p(x.normal), Lm._p(sc), Lm._p(ref),
                                    None) == 0
    rec = torch.empty((n, 12 if dims == 3 else 8), dtype=torch.float32,
                      device="cuda")
    assert L.aqua_gnn_node_records(n, dims, Lm._p(x.r), Lm._p(x.u),
                                   Lm._p(x.rho), Lm._p(x.imove),
                                   Lm._p(x.normal), Lm._p(rec), None) == 0
    got = torch.empty_like(ref)
    assert L.aqua_gnn_edge_features_rec(E, dims, Lm._p(g.receivers),
                                        Lm._p(g.senders), Lm._p(rec),
                                        Lm._p(sc), Lm._p(got), None) == 0
    torch.cuda.synchronize()
    assert E > 0 and torch.equal(got.view(torch.int16), ref.view(torch.int16))
    sv.close()
