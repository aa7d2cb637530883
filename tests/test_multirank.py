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


def _replica_worker(rank, world, port, q):
    """One replica per rank, as bench.py --gpus N runs them, here through the
    CPU oracle: the rank's own fiber (seed 1 + rank) and noise stream, two
    steps, no collective in the step; the ranks meet only to take the max of
    their step times."""
    import sys
    import tempfile
    import time
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    from oracle.pyoracle import Oracle, OracleNoise
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    fib = make_fiber(FiberSpec(2, [20, 20], seed=1 + rank, n_sites=60), tempfile.mkdtemp())
    orc, g = Oracle(fib), OracleNoise(100 + rank)
    t0 = time.perf_counter()
    energies = [orc.step(*g.step(s, fib.arrays["r_var"], fib.m)) for s in range(2)]
    ms = (time.perf_counter() - t0) * 1000.0 / 2
    m = bench.max_over_ranks(ms)
    q.put((rank, ms, m, bench.replica_rate(m, world), energies, orc.get("r").tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_run_independently():
    import tempfile
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = max(o[1] for o in out)
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    from oracle.pyoracle import Oracle, OracleNoise
    for rank, ms, m, rate, energies, r in out:
        assert m == slowest and rate == pytest.approx(2 * 1000.0 / slowest)
        # the same replica alone in this process: bit for bit the rank's result
        fib = make_fiber(FiberSpec(2, [20, 20], seed=1 + rank, n_sites=60), tempfile.mkdtemp())
        orc, g = Oracle(fib), OracleNoise(100 + rank)
        e1 = [orc.step(*g.step(s, fib.arrays["r_var"], fib.m)) for s in range(2)]
        assert e1 == energies
        assert np.array_equal(orc.get("r"), np.array(r))
    assert out[0][5] != out[1][5]  # two different fibers
