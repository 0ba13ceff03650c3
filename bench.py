"""Benchmark: particle-steps/s of the canonical WCSPH step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c1|c0] [--no-cpu-baseline]

Workload (default c1): the 3-D dam break, SPHERIC test-2 tank 3.22 x 1.0 x
1.0 m, water block 1.228 x 1.0 x 0.55 m on a dx = 0.005 m lattice (5,412,000
fluid particles), boundary-integral elements at dx on the five walls
(466,400), 4 pressure probes: N = 5,878,404.  h = 2 dx, Wendland, c0 = 40,
linear EOS, delta-SPH 0.1, Morris viscosity nu = 1e-6, midpoint scheme, CFL
0.1.  Synthetic inputs built by aquagpusph_gb300.case.dam_break_3d().

A step is one full canonical step (link-list + sort + gather + fused sweep
+ integrator + dt), replayed from a CUDA graph.  The resident state (~2.5 GB)
is far larger than the 129 MB L2, so no flush is needed between steps.

One JSON line is printed by rank 0.  Multi-GPU runs (torchrun) are
independent replicas of the workload, one per GPU (the step has no exchange
between GPUs); value aggregates all ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (canonical WCSPH step, 1 GB300)"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle (3-D, V = 16 B):
#   whole step  B = 19 V + 96 + 20 P (P = 3 radix passes)     = 460 B
#   fused sweep = sweep + integrator: read r,u,rho,m,imove,normal (3V+12),
#                 write dudt,drhodt (V+4); read r,u,rho,dudt,drhodt (3V+8),
#                 write r,u,rho (2V+4)                          = 9V + 28
STEP_BYTES_3D = 19 * 16 + 96 + 20 * 3
SWEEP_BYTES_3D = 9 * 16 + 28
STEP_BYTES_2D = 19 * 8 + 96 + 20 * 2
SWEEP_BYTES_2D = 9 * 8 + 28


BATCH = {}


def workload(name):
    from aquagpusph_gb300 import case as cases
    if name == "c2":
        b = cases.sloshing_batch_2d()
        BATCH["c2"] = b
        c = b.case
    elif name == "c4":
        c = cases.dam_break_3d(dx=0.003)
    elif name == "c1s":
        c, _ = cpu_sample("c1")
    elif name == "c1m":
        # profiling size: same lattice, state (~0.8 GB) well above the L2
        c = cases.dam_break_3d(tank=(1.6, 0.5, 0.6), block=(0.8, 0.5, 0.55),
                               probes_z=(0.02, 0.06))
    elif name == "c0":
        c = cases.dam_break_2d()
    else:
        name = "c1"
        c = cases.dam_break_3d()
    if name != "c2":
        c.dt = c.params.dt_fixed
    assert c.N == WORKLOADS[name][1], (name, c.N)
    return c, workload_desc(name)


def cpu_sample(name):
    """A bounded sample of the workload for the CPU runs: the same lattice,
    smoothing length, constants and wall treatment on a smaller tank."""
    from aquagpusph_gb300 import case as cases
    if name == "c5":
        name = "c4"
    if name in ("c2", "c3"):
        b = cases.sloshing_batch_2d()
        return b, (f"the whole batch (64 tanks, N={b.case.N}), each tank "
                   "stepped by the oracle in turn")
    if name == "c4":
        c = cases.dam_break_3d(dx=0.003, tank=(0.48, 0.12, 0.36),
                               block=(0.24, 0.12, 0.33), probes_z=(0.02,))
        c.dt = c.params.dt_fixed
        return c, ("3-D dam break slab at the workload's dx=0.003 m / h=0.006 m: "
                   f"tank 0.48x0.12x0.36 m, block 0.24x0.12x0.33 m, N={c.N}")
    if name in ("c1s", "c1m"):
        name = "c1"
    if name == "c0":
        c = cases.dam_break_2d()
        desc = f"the full 2-D dam break (N={c.N})"
    else:
        c = cases.dam_break_3d(tank=(0.8, 0.2, 0.6), block=(0.4, 0.2, 0.55),
                               probes_z=(0.02, 0.06))
        desc = ("3-D dam break slab at the workload's dx=0.005 m / h=0.01 m: "
                f"tank 0.8x0.2x0.6 m, block 0.4x0.2x0.55 m, N={c.N}")
    c.dt = c.params.dt_fixed
    return c, desc


def time_oracle(c, steps, warmup, min_seconds=0.0, max_steps=100000):
    """CPU oracle throughput (all host threads) on a case or a batch (its
    tanks stepped in turn): ``steps`` steps, repeated until ``min_seconds``
    of CPU work have passed.  Returns (particle-steps/s, threads, seconds,
    steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    orc = O.load_oracle()
    nt = os.cpu_count() or 1
    if hasattr(c, "cases"):
        runs = [(O.OracleState(k), m) for k, m in zip(c.cases, c.motions)]
        n = c.case.N
    else:
        runs = [(O.OracleState(c), None)]
        n = c.N
    for st, m in runs:
        orc.step(st, nthreads=nt, steps=max(warmup, 0), motion=m)
    done = 0
    t0 = time.perf_counter()
    while True:
        for st, m in runs:
            orc.step(st, nthreads=nt, steps=steps, motion=m)
        done += steps
        dt = time.perf_counter() - t0
        if dt >= min_seconds or done >= max_steps:
            break
    return n * done / dt, nt, dt, done


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int) -> float:
    """The largest value over the ranks: the job takes as long as its
    slowest replica."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, n_per_rank: int, steps: int, seconds: float) -> float:
    """Particle-steps/s of the whole job: every rank advances its own replica
    of the workload (weak scaling)."""
    return world * n_per_rank * steps / seconds


# DRAM bytes per particle of the fused sweep from one ncu capture of the
# 1.89M-particle profiling case (dram__bytes_read.sum + dram__bytes_write.sum
# over N: 273.3 + 90.3 MB for the clustered sweep, the particle records plus
# its cluster tables), scaled to a launch by N.
SWEEP_DRAM_BYTES_PER_PARTICLE = {"k_sweep_cl<3>": 192.1, "k_sweep<3>": 170.5}

# FP32 instructions of one fluid-fluid pair of the fast sweep, counted from
# the source of the clustered sweep's pair (separation 3, |r|^2 3, sqrt 1,
# (2-q)^+ 2 with q folded into a fused multiply-add, (2-q)^2 1, F factor 2,
# Shepard term 2, velocity difference 3, (u_ij . r_ij) 3, pressure factor
# 2, grad p 3, lap u 3, div u 1, lap p 2), a fused multiply-add counted once
PAIR_FP32_INSTR = 31
# FP32 lanes x SMs of one GB300 (the instruction rate of the FMA pipes at
# the SM clock)
FP32_LANES = 128 * 152


def support_pairs(c, sample=40000, seed=0):
    """Fluid-fluid pairs within the support (2H, j != i) per fluid particle,
    counted with a k-d tree on a random sample of the fluid particles."""
    from scipy.spatial import cKDTree
    fl = np.flatnonzero(np.asarray(c.imove) == 1)
    d = c.dims
    pts = np.asarray(c.r, np.float64)[fl, :d]
    tree = cKDTree(pts)
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(fl), size=min(sample, len(fl)), replace=False)
    radius = float(c.params.SUPPORT) * float(c.params.H) * (1.0 - 1e-9)
    cnt = tree.query_ball_point(pts[pick], radius, return_length=True)
    return float(np.mean(cnt) - 1.0), len(fl)


def load_traffic(kernel):
    """Per-particle DRAM bytes of `kernel` from the committed ncu capture."""
    return SWEEP_DRAM_BYTES_PER_PARTICLE.get(kernel)


def run_reference(args):
    """The reference arm: the oracle (the reference's kernels restated in
    C++, OpenMP over particles on every host thread) steps the workload
    itself for --warmup untimed and --steps timed steps.  The 26M-particle
    workloads are sampled (a slab of the same lattice): a full step takes
    about half a minute on the host."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    name = args.workload
    if name in ("c4", "c5"):
        c, desc = cpu_sample(name)
        same = False
    else:
        c, desc = workload("c2" if name == "c3" else name)
        c = BATCH.get("c2", c) if name in ("c2", "c3") else c
        desc = "the workload itself" + (
            "; the 64 tanks stepped in turn" if name in ("c2", "c3") else "")
        same = name != "c3"
    value, nt, secs, done = time_oracle(c, args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_desc(name), "sample": desc,
                   "same_config": same},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt,
                         "kind": "port",
                         "sample": desc + "; the CPU oracle (C++ restatement of "
                         "the reference kernels, OpenMP over particles)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if name == "c1" and not args.no_cpu_baseline:
        # the slab sample earlier runs quoted, for continuity
        cs, sdesc = cpu_sample("c1")
        v2, _, _, _ = time_oracle(cs, 8, 1, min_seconds=args.cpu_seconds)
        line["slab_sample"] = {"value": v2, "unit": UNIT, "sample": sdesc}
    print(json.dumps(line), flush=True)
    return 0


# every workload's description and particle count: both arms of the bench
# report the same config
WORKLOADS = {
    "c1": ("3-D dam break, SPHERIC test-2 tank 3.22x1.0x1.0 m, block "
           "1.228x1.0x0.55 m, dx=0.005 m, h=0.01 m, c0=40, BIe walls on 5 "
           "faces, 4 probes", 5878404),
    "c2": ("batched 2-D sloshing: 64 closed tanks 0.9x0.5 m, fill U[0.1,0.4] m "
           "(numpy default_rng(2026)), dx=0.004 m, h=0.008 m, c0=25, BIe walls, "
           "roll about the bottom centre with amplitude U[2,8] deg and period "
           "U[1.2,2] s, one probe per tank", 935414),
    "c4": ("3-D dam break at dx=0.003 m, h=0.006 m (SPHERIC test-2 tank "
           "3.22x1.0x1.0 m, block 1.228x1.0x0.55 m), BIe walls on 5 faces, "
           "4 probes", 26217760),
    "c1m": ("3-D dam break at dx=0.005 m, h=0.01 m (tank 1.6x0.5x0.6 m, block "
            "0.8x0.5x0.55 m)", 1892802),
    "c1s": ("3-D dam break slab at dx=0.005 m, h=0.01 m (tank 0.8x0.2x0.6 m, "
            "block 0.4x0.2x0.55 m)", 406402),
    "c0": ("2-D dam break, tank 3.22x1.8 m, column 1.2x0.6 m, dx=0.01 m, "
           "h=0.02 m, c0=45, BIe walls, 1 probe", 8205),
}


def workload_desc(name):
    if name == "c3":
        return workload_desc("c2") + "; one step = one proposal of k=8 plain steps"
    if name == "c5":
        return (workload_desc("c4") + "; one step = one learned proposal of k=8 "
                "plain steps (graph radius 0.9h: 26 lattice neighbours), "
                "judged every proposal by the plain rates on a 10% cell "
                "sample (density residual, 4 probes)")
    d, n = WORKLOADS.get(name, WORKLOADS["c1"])
    return f"{d}: N={n}"


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from aquagpusph_gb300 import _lib
    from aquagpusph_gb300.solver import Solver

    c, desc = workload(args.workload)
    batch = BATCH.get(args.workload)
    three_d = c.dims == 3
    ncap = (batch.n_cases if batch else 1) * c.params.max_cells()
    sv = Solver(c.params, capacity=c.N, ihoc_capacity=ncap)
    sv.set_precision(args.precision == "fast")
    if batch:
        sv.set_batch(batch)
    else:
        sv.set_case(c)
    stream = torch.cuda.Stream()
    sid = stream.cuda_stream

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    with torch.cuda.stream(stream):
        sv.step(max(args.warmup, 3), graph=True, stream=sid)
    stream.synchronize()
    sv.check(stream=sid)
    # launch shape of the sweep: timed on this case (cached per GPU/case)
    tuning = None
    if not args.no_tune:
        from aquagpusph_gb300 import autotune
        tuning = autotune.autotune(sv, args.precision == "fast", stream=sid)

    # ---- timed region: K steps replayed from the CUDA graphs
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    sv.step(args.steps, graph=True, stream=sid)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms_total = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    sv.check(stream=sid)
    sc = sv.scalars(stream=sid)
    ms_total = max_over_ranks(ms_total, world)
    ms_step = ms_total / args.steps
    value = job_throughput(world, c.N, args.steps, ms_total * 1e-3)

    # ---- the other arithmetic build of the same step, same workload
    other = "exact" if args.precision == "fast" else "fast"
    sv.set_precision(other == "fast")
    other_tuning = None
    if not args.no_tune:
        # each build with its own launch shape
        other_tuning = autotune.autotune(sv, other == "fast", stream=sid)
    sv.step(3, graph=True, stream=sid)
    stream.synchronize()
    barrier()
    ev0.record(stream)
    sv.step(args.steps, graph=True, stream=sid)
    ev1.record(stream)
    ev1.synchronize()
    barrier()
    ms_other = ev0.elapsed_time(ev1) / args.steps
    sv.check(stream=sid)
    sv.set_precision(args.precision == "fast")
    if tuning is not None:
        sv.set_tuning(tuning["variant"], tuning["blocks_per_sm"])
    other_line = {"precision": other, "ms_per_step": ms_other,
                  "value": world * c.N / (ms_other * 1e-3)}
    if other_tuning is not None:
        other_line["tuning"] = {k: other_tuning[k] for k in
                                ("variant", "blocks_per_sm", "ms_per_step")}

    # ---- per-stage CUDA events (same graphs with event nodes), K steps
    sv.set_profiling(True)
    stage = {"linklist": [], "gather": [], "sweep": [], "finalize": []}
    for _ in range(args.steps):
        sv.step(1, graph=True, stream=sid)
        for k, v in sv.stage_times().items():
            stage[k].append(v)
    sv.set_profiling(False)
    sv.check(stream=sid)
    stage_ms = {k: float(np.mean(v)) for k, v in stage.items()}
    top = max(stage_ms, key=stage_ms.get)

    # ---- end to end through the C ABI with pinned host buffers.  Two
    # contexts take the steps in turn, each on its own stream, so the copies
    # of one step overlap the other's compute; every step still uploads its
    # whole input state and downloads its whole result.
    sv2 = Solver(c.params, capacity=c.N, ihoc_capacity=ncap)
    sv2.set_precision(args.precision == "fast")
    if batch:
        sv2.set_batch(batch)
    else:
        sv2.set_case(c)
    if tuning is not None:
        sv2.set_tuning(tuning["variant"], tuning["blocks_per_sm"])
    stream2 = torch.cuda.Stream()
    sid2 = stream2.cuda_stream
    with torch.cuda.stream(stream2):
        sv2.step(3, graph=True, stream=sid2)  # captures its graphs
    stream2.synchronize()
    host = {}
    for name, a in c.state_arrays().items():
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = np.ascontiguousarray(a).view(np.uint8).ravel()
        host[name] = t
    outs = [{name: torch.empty_like(t, pin_memory=True)
             for name, t in host.items()} for _ in range(2)]
    addr_in = {k: t.data_ptr() for k, t in host.items()}
    addr_out = [{k: t.data_ptr() for k, t in o.items()} for o in outs]
    h2d = sum(t.numel() for t in host.values())
    d2h = sum(t.numel() for t in outs[0].values())
    # about 0.5 s of device work (at least K steps, at most 400), so that
    # host jitter and the loop's first upload and last download (which
    # nothing hides) weigh little
    e2e_steps = max(args.steps, int(math.ceil(500.0 / max(ms_step, 1e-3))))
    e2e_steps = 2 * max(1, min(e2e_steps, 400) // 2)
    ctxs = ((sv, sid, stream), (sv2, sid2, stream2))
    # the steps of the two contexts run one after the other (each waits for
    # the other's previous step), so that they do not share the SMs and the
    # L2; each context's copies overlap the other's step
    step_done = (torch.cuda.Event(), torch.cuda.Event())

    def e2e_round_trip(k):
        s_, sid_, st_ = ctxs[k % 2]
        s_.set_state_raw(c.N, addr_in, True, c.t, c.dt, c.iter, stream=sid_)
        if batch:
            s_.set_cases(batch, stream=sid_)
        if k > 0:
            st_.wait_event(step_done[(k - 1) % 2])
        s_.step(1, graph=True, stream=sid_)
        step_done[k % 2].record(st_)
        s_.get_state_raw(addr_out[k % 2], True, stream=sid_)

    # one untimed round trip per context (the stage profiling above dropped
    # the main context's graphs: they are captured here, not in the timing)
    for k in range(2):
        e2e_round_trip(k)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_round_trip(k)
    stream.synchronize()
    stream2.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_s = max_over_ranks(e2e_s, world)
    sv.check(stream=sid)
    sv2.check(stream=sid2)
    sv2.close()
    e2e_value = job_throughput(world, c.N, e2e_steps, e2e_s)

    # ---- roofline of the dominant kernel (the fused sweep)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    sweep_b = SWEEP_BYTES_3D if three_d else SWEEP_BYTES_2D
    step_b = STEP_BYTES_3D if three_d else STEP_BYTES_2D
    achieved = sweep_b * c.N / (stage_ms["sweep"] * 1e-3) / 1e9
    clustered = (three_d and args.precision == "fast" and
                 (tuning is None or tuning["variant"] >= 15))
    kname = ("k_sweep_cl" if clustered else "k_sweep") + ("<3>" if three_d else "<2>")
    traffic_pp = load_traffic(kname)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_src,
                "traffic": traffic_pp * c.N if traffic_pp else None,
                "algorithmic_bytes_per_launch": sweep_b * c.N}
    step_achieved = step_b * c.N / (ms_step * 1e-3) / 1e9
    # the sweep is bound by instruction issue, not HBM: its useful FP32 work
    # (in-support fluid pairs x the pair's FP32 instructions) against the
    # FP32 lanes at the SM clock sampled during the timed steps
    fp32_roofline = None
    if rank == 0:
        per, n_fl = support_pairs(c)
        pairs = per * n_fl
        mhz = (clk or {}).get("sm_mhz") or 2070.0
        peak_ops = FP32_LANES * mhz * 1e6
        ach = pairs * PAIR_FP32_INSTR / (stage_ms["sweep"] * 1e-3)
        fp32_roofline = {"bound": "fp32 issue", "kernel": kname,
                         "achieved": ach / 1e12, "peak": peak_ops / 1e12,
                         "unit": "T instr/s", "frac": ach / peak_ops,
                         "pairs_per_fluid_particle": per,
                         "pair_fp32_instr": PAIR_FP32_INSTR,
                         "note": "useful pair arithmetic only: the filter, "
                                 "out-of-support lanes, staging and the "
                                 "epilogue are the rest"}

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cs, sdesc = cpu_sample(args.workload)
            v, nt, secs, done = time_oracle(cs, args.cpu_steps, 1,
                                            min_seconds=args.cpu_seconds)
            cpu = {"value": v, "unit": UNIT, "cores": nt, "kind": "port",
                   "sample": f"{sdesc}, {done} steps in {secs:.1f} s "
                             "(CPU oracle: C++ restatement of the reference "
                             "kernels, OpenMP over particles)"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (resident state ~"
                             f"{sv.capacity * 430 / 1e9:.1f} GB)",
                       "cuda_graph": True,
                       "precision": args.precision + (
                           " (-use_fast_math build; per-step rates within 1e-5 "
                           "of the reference arithmetic)" if args.precision ==
                           "fast" else " (IEEE f32, no FMA contraction; "
                           "bit-exact with the reference kernels)")},
            "other_build": other_line,
            "tuning": tuning,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps, "contexts": 2},
            "gpu_launches": sv.launches_per_step() * args.steps,
            "roofline": roofline,
            "fp32_roofline": fp32_roofline,
            "step_roofline": {"bound": "hbm", "achieved": step_achieved,
                              "peak": peak, "unit": "GB/s",
                              "frac": step_achieved / peak,
                              "algorithmic_bytes_per_particle_step": step_b},
            "stage_ms": stage_ms, "dominant_stage": top,
            "cpu_baseline": cpu, "clocks": clk,
            "sim": {"t": sc["t"], "dt": sc["dt"], "iter": sc["iter"],
                    "n_cells": [int(x) for x in sc["n_cells"]]},
        }
        if batch:
            ks = sv.case_scalars(stream=sid)
            line["sim"]["cases"] = {
                "n": len(ks), "t_min": min(k["t"] for k in ks),
                "t_max": max(k["t"] for k in ks),
                "dt_min": min(k["dt"] for k in ks),
                "dt_max": max(k["dt"] for k in ks)}
    sv.close()
    if line is not None:
        if args.workload == "c1" and world == 1 and not args.no_learned:
            line["learned"] = learned_summary(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def learned_summary(args):
    """The learned k = 8 proposal on the 64-tank sloshing batch with a
    bounded training budget, for the default bench line: proposal
    throughput against the plain step on the same batch, judge statistics
    and the held-out gain of the trained network over extrapolation."""
    la = argparse.Namespace(**vars(args))
    la.train_pairs, la.train_iters = args.learned_pairs, args.learned_iters
    la.train_runs = args.learned_runs
    # trained on and evaluated in the same regime: after learned_warm plain
    # steps the sloshing has reached the left-wall probes
    la.steps, la.warmup, la.eval_warm = 5, 3, args.learned_warm
    la.train_warm = args.learned_warm
    t0 = time.perf_counter()
    try:
        r = learned_c3(la)
    except Exception as e:  # reported, not hidden: the line says what failed
        return {"error": f"{type(e).__name__}: {e}"}
    keys = ("metric", "value", "unit", "ms_per_step", "plain_value",
            "learned_over_plain", "heldout_mse", "judge_stats", "e2e",
            "roofline", "gpu_launches")
    out = {k: r[k] for k in keys if k in r}
    out["config"] = {"workload": r["config"]["workload"],
                     "training": r["config"]["training"],
                     "proposals_timed": la.steps,
                     "plain_steps_before": la.eval_warm,
                     "judge": r["config"]["judge"]}
    out["wall_s"] = time.perf_counter() - t0
    return out


def learned_c3(args):
    """Learned k = 8 proposals with a plain judge on a quarter of the cases,
    on the 64-tank sloshing batch; the network is first trained on plain
    trajectories of other tanks drawn from the same distribution: online
    over ``train_runs`` runs (generations of 64 tanks through a ring of
    snapshot pairs), or, with train_runs = 0, on one 32-tank trajectory.
    Returns the bench line."""
    import torch
    from aquagpusph_gb300 import case as cases
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    torch.cuda.set_device(0)
    K = 8
    t0 = time.perf_counter()
    train_warm = getattr(args, "train_warm", 500)
    runs = getattr(args, "train_runs", 0)
    model = Lm.Model(2, seed=0)
    if runs:
        # online: generations of 64 tanks (seeds 1234, 1235, ...) through a
        # ring of snapshot pairs; held out: 16 tanks of seed 999
        per_pair = max(1, -(-args.train_iters // (max(1, runs // 64) * 8)))
        online = Lm.online_train(
            model, K, lambda n, g: cases.sloshing_batch_2d(n_cases=n, seed=1234 + g),
            n_runs=runs, runs_per_gen=64, capacity=16, warm=train_warm, gap=300,
            pairs_per_gen=8, iters_per_pair=per_pair, cases_per_step=16,
            lr=1e-3, seed=0)
        tb = cases.sloshing_batch_2d(n_cases=16, seed=999)
        pairs, dts = Lm.collect_pairs(tb, K, n_pairs=4, gap=300, warm=train_warm)
        held = list(range(len(pairs)))
        train_desc = {"tanks": f"{online['runs']} sloshing runs of the config-2 "
                               "distribution in generations of 64 (seeds 1234 + "
                               "generation), online through a ring of snapshot "
                               "pairs; held out: 16 tanks, seed 999",
                      **online}
        train_s = online["train_s"]
    else:
        tb = cases.sloshing_batch_2d(n_cases=32, seed=1234)
        pairs, dts = Lm.collect_pairs(tb, K, n_pairs=args.train_pairs, gap=300,
                                      warm=train_warm)
        Lm.fit_scales(model, pairs, dts, K, tb.case.params, Lm.case_ids(tb))
        held = list(range(len(pairs) - 4, len(pairs)))
    sv_t = Solver(tb.case.params, capacity=tb.case.N)
    tr = Lm.Trainer(model, sv_t, tb, K, lr=1e-3, cases_per_step=16)

    def held_loss(m):
        tr.model = m
        v = [float(tr.batch_loss(pairs[i], dts[i], 0, 16, train=False)[1].item())
             for i in held]
        tr.model = model
        return float(np.mean(v))
    zero = Lm.Model(2, seed=0)
    zero.flat.zero_()
    zero._refresh()
    zero.scales.copy_(model.scales)
    zero.out_scale = model.out_scale
    loss_zero = held_loss(zero)
    if not runs:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(args.train_iters):
            tr.step(pairs[:-4], dts[:-4])
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t1
        train_desc = {"tanks": "32 sloshing tanks, seed 1234 (config-2 distribution)",
                      "pairs": args.train_pairs, "iterations": args.train_iters,
                      "first_pair_after_steps": train_warm, "cases_per_step": 16}
    loss_trained = held_loss(model)
    sv_t.close()
    prep_s = time.perf_counter() - t0

    eb = cases.sloshing_batch_2d()
    c = eb.case
    sv = Solver(c.params, capacity=c.N,
                ihoc_capacity=eb.n_cases * c.params.max_cells())
    sv.set_precision(args.precision == "fast")
    sv.set_batch(eb)
    sv.step(args.eval_warm, graph=True)
    sv.check()
    run = Lm.ProposalRunner(sv, eb, model, k=K, judge_fraction=0.25, tol=0.02,
                            fast=args.precision == "fast")
    for _ in range(args.warmup):
        run.advance()
    for key in ("p_err", "rho_err"):
        run.stats[key] = []
    run.stats.update(proposals=0, judged=0, rolled_back=0)
    # forward pass alone (the network's dense layers), CUDA events
    s0 = Lm.Snapshot.capture(sv, 2)
    g = Lm.Graph(sv, 2, s0["r"], s0["imove"], run.cid, s0.n, run.radius)
    x = Lm.Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                  s0["imove"], s0["normal"])
    net = Lm.Network(model, g, x)
    net.forward()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    net.forward()
    e1.record()
    e1.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    flops = 0
    for name, n, kk, act in Lm.LAYERS:
        rows = g.n_edges if name[0] == "e" else g.n_nodes
        flops += 2 * rows * n * kk
    del net, x, g, s0

    clocks = ClockSampler(0)
    clocks.start()
    calls0 = Lm.CALLS[0]
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for _ in range(args.steps):
        run.advance()
    torch.cuda.synchronize()
    dt_s = time.perf_counter() - t2
    clk = clocks.stop()
    calls = Lm.CALLS[0] - calls0
    judge_launches = args.steps * K * run.judge.launches_per_step()
    value = c.N * K * args.steps / dt_s
    # the plain step on the same batch, same number of particle-steps
    e0.record()
    sv.step(K * args.steps, graph=True)
    e1.record()
    e1.synchronize()
    sv.check()
    plain_ms = e0.elapsed_time(e1)
    plain_value = c.N * K * args.steps / (plain_ms * 1e-3)
    # end to end: state from pinned host memory in, proposal, state out
    host = Lm.Snapshot.capture(sv, 2)
    pin = {f: torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
           for f, v in host.a.items()}
    for f in pin:
        pin[f].copy_(host[f])
    out = {f: torch.empty_like(v, pin_memory=True) for f, v in pin.items()}
    scal = sv.case_scalars()
    n_e2e = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    for _ in range(n_e2e):
        sv.set_state_raw(c.N, {f: v.data_ptr() for f, v in pin.items()}, True,
                         scal[0]["t"], scal[0]["dt"], scal[0]["iter"])
        Lm.ProposalRunner._set_cases(sv, eb, scal)
        run.advance()
        sv.get_state_raw({f: v.data_ptr() for f, v in out.items()
                          if f != "id"}, True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t3
    nbytes = sum(v.numel() * v.element_size() for v in pin.values())
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    peak = peaks.get("bf16_tflops") or 1900.0
    st = run.stats
    line = {
        "metric": "particle-steps/s (learned k=8 proposal + plain judge on 25% "
                  "of the cases, 1 GB300)",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (f32 accumulate), f32 state", "data": "synthetic",
        "config": {"workload": workload_desc("c3") if K == 8 else
                   workload_desc("c2") + f"; one step = one proposal of k={K} "
                   "plain steps", "training": {
                       **train_desc, "train_s": train_s, "prep_s": prep_s},
                   "judge": "plain step re-run of 25% of the cases; rollback at "
                            "> 2% probe-pressure error (of max(|p|, rho g 4h)) "
                            "or > 2% density error (of refd)"},
        "plain_value": plain_value, "learned_over_plain": value / plain_value,
        "heldout_mse": {"trained": loss_trained,
                        "extrapolation_only": loss_zero},
        "judge_stats": {"judged": st["judged"], "rolled_back": st["rolled_back"],
                        "p_err_median": float(np.median(st["p_err"])),
                        "p_err_max": float(np.max(st["p_err"])),
                        "rho_err_median": float(np.median(st["rho_err"])),
                        "rho_err_max": float(np.max(st["rho_err"]))},
        "e2e": {"value": c.N * K * n_e2e / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": n_e2e},
        "gpu_launches": calls + judge_launches,
        "gpu_launches_note": "library entry points called (each launches at "
                             "least one kernel) plus the judge's plain-step "
                             "kernels",
        "roofline": {"bound": "tensor", "kernel": "network forward (dense "
                     "layers and graph gathers)", "achieved": flops / (fwd_ms * 1e-3) / 1e12,
                     "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / (fwd_ms * 1e-3) / 1e12 / peak,
                     "peak_source": "measured" if peaks.get("bf16_tflops") else "fallback",
                     "flops_per_forward": flops, "forward_ms": fwd_ms,
                     "traffic": None},
        "clocks": clk, "cpu_baseline": None,
    }
    run.close()
    sv.close()
    return line


def run_learned(args):
    print(json.dumps(learned_c3(args)), flush=True)
    return 0


def run_learned_3d(args):
    """Learned k = 8 proposals on the 26M-particle 3-D dam break, each judged
    by the plain rates at both ends on a 10% cell sample (and the cells
    around the probes); a failed proposal is replaced by k plain steps.  The
    network is first trained on plain trajectories of a small dam break with
    the same dx, h and walls."""
    import torch
    from aquagpusph_gb300 import case as cases
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    torch.cuda.set_device(0)
    K = 8
    t0 = time.perf_counter()
    small = cases.dam_break_3d(dx=0.003, tank=(0.48, 0.12, 0.36),
                               block=(0.24, 0.12, 0.33), probes_z=(0.02,))
    small.dt = small.params.dt_fixed
    tb = cases.pack([small])
    radius = 0.9 * small.params.h
    pairs, dts = Lm.collect_pairs(tb, K, n_pairs=args.train_pairs, gap=100,
                                  warm=200)
    model = Lm.Model(3, seed=0)
    Lm.fit_scales(model, pairs, dts, K, small.params, Lm.case_ids(tb))
    sv_t = Solver(small.params, capacity=small.N)
    tr = Lm.Trainer(model, sv_t, tb, K, lr=1e-3, cases_per_step=1,
                    radius=radius)
    # held-out pairs spread over the trajectory (one in six)
    held = list(range(3, len(pairs), 6))
    train_pairs = [q for i, q in enumerate(pairs) if i not in held]
    train_dts = [q for i, q in enumerate(dts) if i not in held]

    def held_loss(m):
        tr.model = m
        v = [float(tr.batch_loss(pairs[i], dts[i], 0, 1, train=False)[1].item())
             for i in held]
        tr.model = model
        return float(np.mean(v))
    zero = Lm.Model(3, seed=0)
    zero.flat.zero_()
    zero._refresh()
    zero.scales.copy_(model.scales)
    zero.out_scale = model.out_scale
    loss_zero = held_loss(zero)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.train_iters):
        tr.step(train_pairs, train_dts)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    loss_trained = held_loss(model)
    sv_t.close()
    del pairs, dts, tr, train_pairs, train_dts
    prep_s = time.perf_counter() - t0

    c, _ = workload("c4")
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(args.precision == "fast")
    sv.set_case(c)
    sv.step(args.eval_warm, graph=True)
    sv.check()
    run = Lm.FieldProposalRunner(sv, c, model, k=K, radius=radius,
                                 rho_sample=0.1, tol=0.02,
                                 fast=args.precision == "fast")
    for _ in range(args.warmup):
        run.advance()
    st = run.stats
    st.update(proposals=0, rolled_back=0, p_err=[], rho_err=[], phase_s={})
    clocks = ClockSampler(0)
    clocks.start()
    calls0 = Lm.CALLS[0]
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for _ in range(args.steps):
        run.advance()
    torch.cuda.synchronize()
    dt_s = time.perf_counter() - t2
    clk = clocks.stop()
    calls = Lm.CALLS[0] - calls0
    # two rate-sampled plain steps per proposal, k plain steps per rollback
    judge_launches = (2 * args.steps * run.judge.launches_per_step() +
                      st["rolled_back"] * K * sv.launches_per_step())
    value = c.N * K * args.steps / dt_s
    # the plain step on the same case, same number of particle-steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    sv.step(K * args.steps, graph=True)
    e1.record()
    e1.synchronize()
    sv.check()
    plain_ms = e0.elapsed_time(e1)
    plain_value = c.N * K * args.steps / (plain_ms * 1e-3)
    # the network forward alone on the current state, CUDA events
    s0 = Lm.Snapshot.capture(sv, 3)
    g = Lm.Graph(sv, 3, s0["r"], s0["imove"], run.cid, s0.n, radius)
    x = Lm.Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                  s0["imove"], s0["normal"])
    net = Lm.Network(model, g, x)
    net.forward()
    e0.record()
    net.forward()
    e1.record()
    e1.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    flops = 0
    for name, n, kk, act in Lm.LAYERS:
        rows = g.n_edges if name[0] == "e" else g.n_nodes
        flops += 2 * rows * n * kk
    n_edges = g.n_edges
    del net, x, g, s0
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    peak = peaks.get("bf16_tflops") or 1900.0
    steps = args.steps
    line = {
        "metric": "particle-steps/s (learned k=8 proposal judged by the plain "
                  "rates on a 10% cell sample, 1 GB300)",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt_s / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (f32 accumulate), f32 state", "data": "synthetic",
        "config": {"workload": workload_desc("c5"), "training": {
                       "case": "3-D dam break slab at dx=0.003 m, h=0.006 m: "
                               "tank 0.48x0.12x0.36 m, block 0.24x0.12x0.33 m, "
                               f"N={small.N}",
                       "pairs": args.train_pairs, "held_out": len(held),
                       "iterations": args.train_iters,
                       "train_s": train_s, "prep_s": prep_s},
                   "judge": "every proposal: the plain rates (one plain "
                            "step) at the start and the proposed state on a "
                            "hashed 10% of the cells plus the cells around the "
                            "4 probes; rollback (k plain steps from the start "
                            "state) at > 2% density error (of refd) against "
                            "the trapezoidal plain continuity equation on the "
                            "sampled fluid, or > 2% probe-pressure error (of "
                            "max(|p|, rho g 4h)) against the interpolation of "
                            "those plain densities"},
        "plain_value": plain_value, "learned_over_plain": value / plain_value,
        "heldout_mse": {"trained": loss_trained,
                        "extrapolation_only": loss_zero},
        "judge_stats": {"proposals": st["proposals"],
                        "rolled_back": st["rolled_back"],
                        "p_err_median": float(np.median(st["p_err"])),
                        "p_err_max": float(np.max(st["p_err"])),
                        "rho_err_median": float(np.median(st["rho_err"])),
                        "rho_err_max": float(np.max(st["rho_err"]))},
        "phase_ms_per_proposal": {k: 1e3 * v / steps
                                  for k, v in st["phase_s"].items()},
        "graph_edges": n_edges,
        "gpu_launches": calls + judge_launches,
        "gpu_launches_note": "library entry points called (each launches at "
                             "least one kernel) plus the judge's plain-step "
                             "kernels",
        "roofline": {"bound": "tensor", "kernel": "network forward (fused "
                     "tcgen05 edge MLPs with on-chip receiver sums, node "
                     "layers, graph gathers)",
                     "achieved": flops / (fwd_ms * 1e-3) / 1e12,
                     "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / (fwd_ms * 1e-3) / 1e12 / peak,
                     "peak_source": "measured" if peaks.get("bf16_tflops") else "fallback",
                     "flops_per_forward": flops, "forward_ms": fwd_ms,
                     "traffic": None},
        "clocks": clk, "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)
    run.close()
    sv.close()
    return 0


def run_forward_only(args):
    """The network forward alone on the 64-tank batch (c3) or the 26M-particle
    dam break (c5), untrained weights, after a few plain steps: one warm-up
    forward, then one timed with CUDA events (for kernel launch lists)."""
    import torch
    from aquagpusph_gb300 import case as cases
    from aquagpusph_gb300 import learned as Lm
    from aquagpusph_gb300.solver import Solver
    torch.cuda.set_device(0)
    if args.workload == "c5":
        c, _ = workload("c4")
        dims, radius, cid = 3, 0.9 * c.params.h, None
        sv = Solver(c.params, capacity=c.N)
        sv.set_case(c)
    else:
        eb = cases.sloshing_batch_2d()
        c = eb.case
        dims, radius = 2, float(c.params.support * c.params.h)
        sv = Solver(c.params, capacity=c.N,
                    ihoc_capacity=eb.n_cases * c.params.max_cells())
        sv.set_batch(eb)
        cid = Lm.case_ids(eb)
    if cid is None:
        cid = torch.zeros(c.N, dtype=torch.int32, device="cuda")
    sv.step(20, graph=True)
    sv.check()
    model = Lm.Model(dims, seed=0)
    s0 = Lm.Snapshot.capture(sv, dims)
    g = Lm.Graph(sv, dims, s0["r"], s0["imove"], cid, s0.n, radius)
    x = Lm.Inputs(g, s0["r"], s0["u"], s0["rho"], s0["dudt"], s0["drhodt"],
                  s0["imove"], s0["normal"])
    net = Lm.Network(model, g, x)
    net.forward()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    net.forward()
    e1.record()
    e1.synchronize()
    flops = sum(2 * (g.n_edges if name[0] == "e" else g.n_nodes) * n * kk
                for name, n, kk, act in Lm.LAYERS)
    ms = e0.elapsed_time(e1)
    print(json.dumps({"workload": workload_desc(args.workload),
                      "forward_ms": ms, "edges": g.n_edges, "nodes": g.n_nodes,
                      "flops": flops, "tflops": flops / (ms * 1e-3) / 1e12}),
          flush=True)
    sv.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c1",
                    choices=["c1", "c0", "c1s", "c1m", "c2", "c3", "c4",
                             "c5"])
    ap.add_argument("--train-pairs", type=int, default=24)
    ap.add_argument("--train-iters", type=int, default=300)
    ap.add_argument("--eval-warm", type=int, default=None,
                    help="plain steps before the proposals (3000 for c3, 200 for c5)")
    ap.add_argument("--cpu-steps", type=int, default=8)
    ap.add_argument("--precision", default="fast", choices=["exact", "fast"])
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="minimum CPU work of the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forward-only", action="store_true",
                    help="c3 / c5: time the network forward alone")
    ap.add_argument("--no-learned", action="store_true",
                    help="c1: leave out the learned-proposal sub-object")
    ap.add_argument("--learned-pairs", type=int, default=24)
    ap.add_argument("--learned-runs", type=int, default=256,
                    help="runs of the online trainer of the learned sub-object "
                         "(0: one 32-tank trajectory of --learned-pairs pairs)")
    ap.add_argument("--train-runs", type=int, default=256,
                    help="runs of the online trainer of --workload c3 (0: one "
                         "32-tank trajectory of --train-pairs pairs)")
    ap.add_argument("--learned-iters", type=int, default=300)
    ap.add_argument("--learned-warm", type=int, default=20000)
    ap.add_argument("--train-warm", type=int, default=500,
                    help="c3: plain steps before the first training pair")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.eval_warm is None:
        args.eval_warm = 200 if args.workload == "c5" else 3000
    if args.forward_only and args.workload in ("c3", "c5"):
        return run_forward_only(args)
    if args.workload == "c3":
        return run_learned(args)
    if args.workload == "c5":
        return run_learned_3d(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
