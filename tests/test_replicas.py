"""bench.py's multi-GPU path is independent replicas: every rank times its own steps, the job's
time is the slowest rank's (all-reduce MAX) and the job's rate counts every rank's units.  Two
gloo ranks on the CPU stand in for two GPUs; no data-path collective is involved."""
import os
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        total, rate = bench.replica_rate(times[rank], units=1e9, steps=4, world=world, dist=dist)
        out[rank] = (total, rate)
    finally:
        dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    world, times = 2, [800.0, 1000.0]  # ms for 4 steps on each rank
    manager = mp.get_context("spawn").Manager()  # no fork of a multi-threaded process
    out = manager.dict()
    mp.start_processes(_rank, args=(world, port, times, out), nprocs=world, join=True, start_method="spawn")
    results = dict(out)
    manager.shutdown()
    assert len(results) == world
    for rank in range(world):
        total, rate = results[rank]
        assert total == 1000.0
        assert rate == pytest.approx(world * 1e9 * 4 / 1.0 / 1e9)


def test_replica_rate_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    total, rate = bench.replica_rate(500.0, units=2e9, steps=5, world=1)
    assert total == 500.0 and rate == pytest.approx(2e9 * 5 / 0.5 / 1e9)
