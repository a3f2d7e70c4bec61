"""CPU, world_size 2 over gloo: the replica bookkeeping bench.py uses for N>1
(barrier, max over ranks of the step time, rank-0-only output).  The path
itself has no collective: each rank solves its own system."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(10.0 + rank)
    s = d.sum(1.0)
    d.barrier()
    q.put((rank, m, s, d.world))
    d.close()


def test_replica_bookkeeping_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    out = sorted(q.get(timeout=5) for _ in range(2))
    assert out == [(0, 11.0, 2.0, 2), (1, 11.0, 2.0, 2)]
