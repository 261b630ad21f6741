"""The N-GPU form of the benchmark (independent replicas, "replicas only": one gprMax model is
one grid and the reference has no multi-GPU solve) on CPU with the gloo backend, two ranks: the
timed region ends at the slowest rank (max over ranks) and the whole-job rate counts every
rank's cells."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    seconds = [0.8, 1.25][rank]
    slowest = bench.barrier_max(dist, seconds)
    rate = bench.replica_rate(world, 32_000_000, 1000, slowest)
    out[rank] = (slowest, rate)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_count_all_cells():
    world = 2
    port = _free_port()
    with mp.get_context('spawn').Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        slowest, rate = res[rank]
        assert slowest == 1.25
        assert rate == pytest.approx(2 * 32_000_000 * 1000 / 1.25 / 1e6)
