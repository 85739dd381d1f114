"""The replica path of bench.py on CPU: two gloo ranks, each timing its own volume,
reduce to the slowest rank's time and report the whole job's throughput (what the
bench does over NCCL with one rank per GPU)."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _rank_main(rank, world, port, results):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" (r + 1) seconds for its replica of 1000 units
        t = bench.max_over_ranks(dist, float(rank + 1), "cpu")
        results[rank] = (t, bench.replica_throughput(1000, world, t))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_slowest_time_and_job_throughput():
    torch = pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    world = 2
    manager = mp.Manager()
    results = manager.dict()
    mp.start_processes(_rank_main, args=(world, port, results), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        t, thr = results[r]
        assert t == 2.0                      # the slowest replica
        assert thr == world * 1000 / 2.0     # all units over that time


def test_single_process_needs_no_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(None, 3.5, "cpu") == 3.5
    assert bench.replica_throughput(10, 1, 2.0) == 5.0
