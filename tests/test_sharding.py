"""PD sharding across ranks (host logic, CPU, gloo world_size 2)."""
import os
import socket

import numpy as np
import pytest

from manifoldem_python_gb300.sharding import lpt_partition, pd_cost, shard


def test_lpt_covers_each_pd_once_and_balances():
    rng = np.random.default_rng(0)
    counts = np.clip(np.round(rng.lognormal(np.log(400), 0.6, 800)), 100, 3000).astype(int)
    for world in (1, 2, 3, 8):
        bins = lpt_partition([pd_cost(n, 128) for n in counts], world)
        allp = sorted(p for b in bins for p in b)
        assert allp == list(range(len(counts)))
        loads = [sum(pd_cost(counts[p], 128) for p in b) for b in bins]
        assert max(loads) <= min(loads) + max(pd_cost(n, 128) for n in counts)
        assert all(b == sorted(b) for b in bins)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, counts, q):
    import torch.distributed as dist
    from manifoldem_python_gb300.sharding import max_over_ranks, shard
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    mine = shard(counts, 128, rank, world)
    t = max_over_ranks(float(10 + rank))
    q.put((rank, mine, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_disjoint_shards():
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    counts = [100, 3000, 450, 460, 700, 120, 2500, 333]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, counts, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = [r[1] for r in res]
    assert sorted(shards[0] + shards[1]) == list(range(len(counts)))
    assert not set(shards[0]) & set(shards[1])
    assert all(r[2] == 11.0 for r in res)        # max over ranks
