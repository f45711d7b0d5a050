"""Replica sharding and the max-over-ranks timing reduction, with two gloo
ranks on the CPU (the engine's multi-GPU mode is replicas only)."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from uastar_gb300 import replicas  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items = list(range(11))
    mine = replicas.shard(items, rank, world)
    replicas.barrier()
    t = replicas.max_over_ranks(1.5 + rank)
    total = replicas.sum_over_ranks(len(mine))
    q.put((rank, mine, t, total))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
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
    (r0, s0, t0, n0), (r1, s1, t1, n1) = out
    assert sorted(s0 + s1) == list(range(11)) and not set(s0) & set(s1)
    assert t0 == t1 == 2.5
    assert n0 == n1 == 11


def test_shard_single_rank_and_errors():
    assert replicas.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    with pytest.raises(ValueError):
        replicas.shard([1], 2, 2)
