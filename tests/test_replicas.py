"""Replica sharding on CPU with a world-size-2 gloo process group."""

from __future__ import annotations

import os
import socket

import pytest

from vsr_gb300 import replicas


def test_assign_covers_every_unit_once_and_balances():
    sizes = [4096 * 4096, 256 * 300, 1000 * 2000, 4000 * 3000, 512 * 512, 2048 * 2048, 777 * 999]
    for ws in (1, 2, 3, 4):
        parts = [replicas.assign(sizes, ws, r) for r in range(ws)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)
    with pytest.raises(ValueError):
        replicas.assign(sizes, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.assign(sizes, world, rank)
    t = replicas.max_over_ranks([float(sum(sizes[i] for i in mine)), float(rank)])
    q.put((rank, mine, t))
    dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    sizes = [10, 7, 5, 5, 3, 1]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, t0), (r1, m1, t1) = res
    assert sorted(m0 + m1) == list(range(len(sizes)))
    assert not set(m0) & set(m1)
    # both ranks see the same maxima: the larger load and the larger rank
    assert t0 == t1
    assert t0[0] == max(sum(sizes[i] for i in m0), sum(sizes[i] for i in m1))
    assert t0[1] == 1.0
