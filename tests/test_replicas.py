"""The multi-GPU (replicas) host logic with two gloo ranks on CPU: request sharding, and the
sum / max / gather aggregation bench.py reports over ranks."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

from micrographia_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mine = replicas.shard(range(11), rank, world)
        units, secs = replicas.aggregate(dist, units=100 * (rank + 1), seconds=0.25 + rank)
        lat = replicas.gather(dist, [rank + 0.5] * (rank + 1))
        allreq = replicas.gather(dist, mine)
        out.put((rank, mine, units, secs, lat, sorted(allreq)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_aggregate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, m0, u0, s0, l0, a0), (_, m1, u1, s1, l1, a1) = res
    assert m0 == [0, 2, 4, 6, 8, 10] and m1 == [1, 3, 5, 7, 9]
    assert u0 == u1 == 300.0 and s0 == s1 == 1.25
    assert l0 == l1 == [0.5, 1.5, 1.5]
    assert a0 == a1 == list(range(11))


def test_single_process_is_identity():
    assert replicas.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert replicas.aggregate(None, 5, 2.0) == (5.0, 2.0)
    assert replicas.gather(None, (1, 2)) == [1, 2]
