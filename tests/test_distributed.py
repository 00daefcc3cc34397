"""Multi-rank host logic of bench.py on CPU with the gloo backend
(world size 2): every rank runs an independent replica of the workload; the
step time is the maximum over ranks and the throughput counts all replicas."""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import numpy as np

    import oracle
    # each rank evaluates its own small replica on the CPU oracle and times it
    rng = np.random.default_rng(rank)
    P = rng.random((3, 1500))
    x = rng.standard_normal(1500)
    O = oracle.OraclePlan(P, None, 2, 0.8, 0)
    y, _ = O.action(0, 1.0, x, nthreads=1)
    ms_local = 10.0 * (rank + 1)
    ms = bench.max_over_ranks(ms_local, dist, None)
    value = bench.replica_throughput(1500, ms, world)
    q.put((rank, ms, value, float(np.linalg.norm(y))))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_max_over_ranks_gloo():
    import torch.multiprocessing as mp

    from oracle import build as oracle_build
    oracle_build.build()  # once, before the workers load it
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [20.0, 20.0]          # the slowest rank's time
    assert all(abs(o[2] - 2 * 1500 / 0.02) < 1e-6 for o in out)
    assert all(o[3] > 0 for o in out)


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_throughput(100, 1.0, 1) == pytest.approx(1e5)
