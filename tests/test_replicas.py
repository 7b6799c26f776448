"""Replicas on several GPUs, host side: sharding of independent units and
the benchmark's slowest-rank timing, run as two gloo ranks on the CPU."""
import os
import socket

import pytest

from opesci import replicas


def test_shard_covers_every_unit_once():
    items = list(range(23))
    parts = [replicas.shard(items, r, 4) for r in range(4)]
    assert sorted(sum(parts, [])) == items
    assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        replicas.shard(items, 4, 4)


def test_single_rank_aggregate():
    rate, t = replicas.aggregate_rate(1e9, 2.0)
    assert rate == 5e8 and t == 2.0


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        # rank r "took" 1 + r seconds for the same work
        rate, t = replicas.aggregate_rate(100.0, 1.0 + rank, dist, device='cpu')
        mine = replicas.shard(range(10), rank, world)
        out.put((rank, rate, t, mine))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    pytest.importorskip('torch')
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, t, mine in res:
        assert t == 2.0                      # the slower rank's time
        assert rate == 100.0 * 2 / 2.0       # all ranks' units over it
    assert res[0][3] == [0, 2, 4, 6, 8] and res[1][3] == [1, 3, 5, 7, 9]
