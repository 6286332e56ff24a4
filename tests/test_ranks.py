"""Multi-rank host logic on CPU (gloo, world size 2): the bench's reduction of
per-rank timings and step counts (max time, summed work)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    secs, units = bench.reduce_over_ranks(1.5 + rank, 1000 * (rank + 1), world)
    q.put((rank, secs, units))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, secs, units in out:
        assert secs == 2.5 and units == 3000.0


def test_reduce_single_rank_is_identity():
    import bench
    assert bench.reduce_over_ranks(3.0, 7, 1) == (3.0, 7.0)
