"""The replica reductions of bench.py on two CPU ranks (gloo): barrier,
slowest-rank time, total work, whole-job rate."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    from mdcraft_gb300.replicas import Replicas
    r = Replicas(world, rank, "gloo")
    r.barrier()
    atoms, seconds = 1000.0 * (rank + 1), 0.5 + rank  # rank 1 is slower and did more
    q.put((rank, r.max(seconds), r.sum(atoms), r.throughput(atoms, seconds)))
    r.barrier()
    r.close()


def test_two_rank_reductions():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, rate in res:
        assert mx == 1.5
        assert sm == 3000.0
        assert rate == pytest.approx(3000.0 / 1.5)


def test_single_process_needs_no_group():
    from mdcraft_gb300.replicas import Replicas
    r = Replicas(1)
    assert r.max(2.0) == 2.0 and r.sum(3.0) == 3.0 and r.throughput(10.0, 2.0) == 5.0
    r.close()
