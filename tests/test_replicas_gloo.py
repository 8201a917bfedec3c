"""The N>1 bench path on CPU: two gloo ranks, each a full replica of the
workload; the job time is the slowest rank's and the throughput counts the
work of every replica.  (The path has no data exchange: no collective runs
in the timed work itself.)"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 25.0 * rank, "cpu")
        value = bench.replica_value(1_000_000, world, ms)
        dist.barrier()
    finally:
        dist.destroy_process_group()
    Path(out_dir, "rank%d" % rank).write_text("%r %r" % (ms, value))


def test_two_replicas_gloo(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    mp.spawn(_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        ms, value = map(float, (tmp_path / ("rank%d" % r)).read_text().split())
        assert ms == 125.0
        assert value == pytest.approx(2 * 1_000_000 / 0.125)


def test_single_process_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.replica_value(10, 1, 1000.0) == 10.0
