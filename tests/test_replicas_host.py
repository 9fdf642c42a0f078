"""The multi-GPU form of the benchmark (independent replicas, one per rank, no data-path
collective): the slowest rank's time is the whole job's, and the throughput counts every
replica's quartets.  Two gloo ranks on the CPU exercise the reduction."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total_ms, e2e_s = bench.max_over_ranks([100.0 * (rank + 1), 1.0 + rank], dist)
        q.put((rank, total_ms, e2e_s, bench.replica_throughput(world, 45_230_223, 5, total_ms * 1e-3)))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total_ms, e2e_s, value in out:
        assert total_ms == 200.0 and e2e_s == 2.0
        assert abs(value - 2 * 45_230_223 * 5 / 0.2 / 1e9) < 1e-12


def test_single_process_values_pass_through():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([3.0, 4.5]) == [3.0, 4.5]
    assert abs(bench.replica_throughput(1, 1e9, 1, 1.0) - 1.0) < 1e-15
