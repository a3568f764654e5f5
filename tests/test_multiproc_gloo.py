"""N > 1 host logic of bench.py on CPU: two gloo ranks (replicas only).

Each rank times its own replica; the job's time is the max over ranks and its
value all ranks' units over that time. No GPU, no collective on the data path.
"""
import os
import socket

import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    ms = 100.0 + 50.0 * rank            # rank 1 is the slower replica
    m = bench.reduce_max(dist, ms)
    q.put((rank, m, bench.replica_rate(world, 1000, 10, m)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == 150.0
        assert abs(v - 2 * 1000 * 10 / 0.150) < 1e-6
