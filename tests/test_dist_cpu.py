"""Multi-process host logic of bench.py on CPU (gloo, world_size 2): the
barrier and the max-over-ranks timing used for replicas-only scaling."""
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
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(dist)
    m = bench.allmax(dist, 10.0 + rank)  # rank 1 is the slowest
    value = world * 100.0 / m            # replicas: total work / slowest rank
    q.put((rank, m, value))
    dist.destroy_process_group()


def test_replicas_timing_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [11.0, 11.0]
    assert all(abs(r[2] - 200.0 / 11.0) < 1e-12 for r in res)
