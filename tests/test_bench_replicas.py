"""The multi-GPU path of bench.py on the CPU: two ranks over gloo
(127.0.0.1), the job time taken as the slowest rank's, weak-scaling
throughput, and the reference arm running on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, loc = bench.dist_setup()
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, w)
    value = bench.job_throughput(w, 1000, 20, slowest)
    # the reference arm: rank 1 exits without work and without output
    args = type("A", (), {"steps": 1, "warmup": 0, "workload": "c0",
                          "gpus": world})()
    ret = bench.run_reference(args) if r == 1 else 0
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, loc, slowest, value, ret))


def test_two_ranks_over_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, slowest, value, ret) in enumerate(out):
        assert (rank, world, local) == (r, 2, r)
        assert slowest == 15.0               # the slower rank's time
        assert value == 2 * 1000 * 20 / 15.0   # both replicas' work
        assert ret == 0


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(1, 10, 4, 2.0) == 20.0


def test_workload_table_is_shared_by_both_arms():
    """Every workload the bench accepts has one description and particle
    count, which the CPU sample of the reference arm names too; the learned
    workloads extend their plain workload's description."""
    import bench
    for name in ("c0", "c1", "c1s", "c1m", "c2", "c4"):
        desc = bench.workload_desc(name)
        d, n = bench.WORKLOADS[name]
        assert desc == f"{d}: N={n}"
    assert bench.workload_desc("c3").startswith(bench.workload_desc("c2"))
    assert bench.workload_desc("c5").startswith(bench.workload_desc("c4"))
    assert "10% cell sample" in bench.workload_desc("c5")
