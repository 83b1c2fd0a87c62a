"""Multi-GPU runs are independent replicas (one batch of rebuilds per rank,
no data-path exchange); only the timings meet, in the max-over-ranks
reduction of bench.py.  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    # Rank r processed 16 (r + 1) rebuilds in 2 (r + 1) seconds.
    rate, slowest = bench.replica_rate(2.0 * (rank + 1), 16.0 * (rank + 1), world)
    out[rank] = (rate, slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_is_total_units_over_slowest_rank():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True,
                       start_method="spawn")
    # 16 + 32 rebuilds over the slowest rank's 4 s, on every rank.
    for r in range(world):
        assert out[r] == (pytest.approx(12.0), pytest.approx(4.0))


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.replica_rate(2.0, 10.0, 1) == (5.0, 2.0)
