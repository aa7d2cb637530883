"""Replica aggregation of bench.py across ranks (gloo, world size 2, CPU):
every rank gets the max of the per-rank step times and the whole-job rate
counts one step per rank."""
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
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [120.0, 180.0][rank]
    m = bench.max_over_ranks(local_ms)
    q.put((rank, m, bench.replica_rate(m, world), bench.dist_env()))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_ranks():
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
    for rank, m, rate, env in out:
        assert m == 180.0
        assert rate == pytest.approx(2 * 1000.0 / 180.0)
        assert env[0] == rank and env[1] == 2
