"""The N-GPU bench path runs independent replicas (one deck per rank, seed +
rank) and combines them with one reduction: checked here with two gloo
ranks on the CPU."""
import os
import sys

import pytest

from conftest import REPO


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, REPO)
    import bench
    out = bench.combine_ranks(dist, 100.0 + 50.0 * rank, 1e9 * (rank + 1), 1e6 * (rank + 1))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_replicas_combine_max_time_and_summed_work():
    import socket
    import torch.multiprocessing as mp
    torch = pytest.importorskip("torch")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        t, segs, hist = res[r]
        assert t == 150.0 and segs == 3e9 and hist == 3e6


def test_single_rank_passes_through():
    sys.path.insert(0, REPO)
    import bench
    assert bench.combine_ranks(None, 5.0, 7.0, 9.0) == (5.0, 7.0, 9.0)
