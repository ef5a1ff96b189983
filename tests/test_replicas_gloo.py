"""The N > 1 path of bench.py is replicas only: each rank runs its own
simulation and the job reports sum-over-ranks work / max-over-ranks time.
Its host logic (rendezvous from the torchrun environment, barrier, max over
ranks) runs here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench
    w, r, local = bench.dist_init()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    # each replica reports its own time; the job time is the slowest replica's
    t = bench.allmax(w, 1.0 + rank)
    out.put((rank, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2.0), (1, 2.0)]
