"""bench.py's multi-rank aggregation (replicas: summed zones over the max
time of all ranks), run as two gloo ranks on the CPU."""
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
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.aggregate(dist, local_ms=10.0 + rank, local_units=1000.0 * (rank + 1))
    q.put((rank, ms, units))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, units in out:
        assert ms == 11.0            # max over ranks
        assert units == 3000.0       # sum over ranks
