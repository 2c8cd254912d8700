"""The multi-GPU form is replicas only: every rank runs its own grid on its own
points, and the bench's only cross-rank step is the max of the timed region.
Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, rank, world)
    ms = bench.slowest_rank_ms(1.5 + rank, world, "cpu")  # rank 1 is the slow one
    out[rank] = (ms, bench.replica_throughput(1000, ms, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.5
    assert res[0][1] == res[1][1] == pytest.approx(2 * 1000 / 2.5e-3)


def test_single_rank_needs_no_process_group():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    assert bench.slowest_rank_ms(3.0, 1, "cpu") == 3.0
    assert bench.replica_throughput(4_194_304, 2.0, 1) == pytest.approx(4_194_304 / 2e-3)
