"""Replica aggregation of bench.py (--gpus N runs N independent instances,
no data-path collective): world_size 2 over gloo on the CPU, each rank
running its own small oracle instance."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    import time
    import importlib.util
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    sys.path.insert(0, os.path.join(REPO, "wormlike-chain-triblock_gb300"))
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench", os.path.join(REPO, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    o = oracle.Oracle((8, 8, 8), 2, 6, (2, 2, 2), (0.15,) * 3, 1.0, (0.5,) * 3, (15,) * 3, nthreads=1)
    o.set_fields(np.random.default_rng(rank).normal(0, 0.5, (3, 512)))
    t0 = time.perf_counter()
    o.propagate(1)
    o.propagate(-1)
    dt = time.perf_counter() - t0 + 0.05 * rank
    v, units, tmax = bench.replica_throughput(12, dt)
    out[rank] = (v, units, tmax, dt)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_throughput():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    v0, u0, t0, d0 = out[0]
    v1, u1, t1, d1 = out[1]
    assert u0 == u1 == 24  # units summed over ranks
    assert t0 == t1 == max(d0, d1)  # slowest rank's time
    assert abs(v0 - 24 / max(d0, d1)) < 1e-9 * v0
