"""The multi-GPU path is replicas: each rank renders its own ISAAC streams
(distinct seeds) and the job's time is the slowest rank's.  Its host logic,
the reduction over ranks in bench.py, runs here on CPU as two gloo ranks."""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    kern_ms = [40.0, 55.0][rank]
    binned = [1_000_000_000, 900_000_000][rank]
    wall = [0.5, 0.7][rank]
    q.put((rank, bench.rank_totals(kern_ms, binned, wall, dist), bench.rank_seed(7, rank)))
    dist.destroy_process_group()


def test_rank_totals_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (ms, binned, wall), seed in got:
        assert ms == 55.0 and binned == 1.9e9 and wall == 0.7
    assert got[0][2] != got[1][2]


def test_rank_totals_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_totals(3.0, 10, 1.5) == (3.0, 10.0, 1.5)
