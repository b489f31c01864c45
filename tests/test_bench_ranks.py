"""bench.py with one replica per rank (torchrun, N > 1): the step time is the maximum over ranks, so the
reported whole-job rate is N / (slowest rank's time).  Two gloo ranks on the CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.max_over_ranks(0.25 + rank, world, "cpu")))
    finally:
        dist.destroy_process_group()


def test_step_time_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert got == [(0, 1.25), (1, 1.25)]
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(0.5, 1, "cpu") == 0.5


def test_traffic_table_and_profiles_are_consistent():
    """Every measured-traffic entry of the bench names a workload it can run and a committed profile
    summary, and every profile summary gives the command that made it."""
    import bench
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for (workload, precision), traffic in bench.SWEEP_DRAM_BYTES.items():
        assert workload in bench.WORKLOADS, workload
        assert precision in ("fp32", "fp64"), precision
        assert traffic > 0
        src = bench.SWEEP_DRAM_SOURCE[(workload, precision)].split(" ")[0]
        assert os.path.exists(os.path.join(root, src)), src
    for name in os.listdir(os.path.join(root, "profiles")):
        text = open(os.path.join(root, "profiles", name)).read()
        assert "Command" in text and "ncu " in text, name
