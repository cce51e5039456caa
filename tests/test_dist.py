"""bench.py's rank helper on two gloo ranks (CPU): barrier and max-over-ranks."""

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    d = bench.Dist(world)
    d.barrier()
    out[rank] = d.max(float(rank + 1) * 10.0)
    d.close()


def test_two_rank_max_and_barrier():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 20.0, 1: 20.0}
