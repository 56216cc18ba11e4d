"""Host logic of the multi-rank path: LPT sharding of batch items and the
result gather / max-time reduction, on two gloo ranks (CPU, no GPU)."""
import os
import socket

import numpy as np
import pytest


def test_lpt_partition_balance_and_cover():
    from wot_gb300.ot.shard import lpt_partition
    rng = np.random.default_rng(0)
    w = rng.lognormal(0, 1.5, 1000)
    for n in (1, 2, 3, 8):
        parts = lpt_partition(w, n)
        assert sorted(k for p in parts for k in p) == list(range(1000))
        loads = [w[p].sum() for p in parts]
        # LPT bound: max load <= total / n + max item
        assert max(loads) <= w.sum() / n + w.max() + 1e-9


def test_item_work_uses_pair_shapes():
    from wot_gb300.ot.shard import item_work, my_items
    shapes = [(10, 20), (30, 40)]
    items = [(0, {}), (1, {}), (1, {}), (0, {})]
    assert item_work(shapes, items) == [200.0, 1200.0, 1200.0, 200.0]
    assert sorted(my_items(shapes, items, 0, 2) + my_items(shapes, items, 1, 2)) == [0, 1, 2, 3]


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from wot_gb300.ot.shard import gather, max_over_ranks, my_items
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        shapes = [(100 * (p + 1), 50 * (p + 2)) for p in range(7)]
        items = [(p, {'epsilon': e}) for p in range(7) for e in (0.01, 0.05, 0.1)]
        mine = my_items(shapes, items, rank, world)
        local = [(k, ('solved', items[k][0], rank)) for k in mine]
        allres = gather(local)
        t = max_over_ranks(1.0 + rank)
        q.put((rank, mine, [k for k, _ in allres], t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_gather():
    import multiprocessing as mp
    pytest.importorskip('torch')
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    mine0, mine1 = out[0][1], out[1][1]
    assert not set(mine0) & set(mine1)
    assert sorted(mine0 + mine1) == list(range(21))
    assert out[0][2] == out[1][2] == list(range(21))   # every rank holds every result, in order
    assert out[0][3] == out[1][3] == 2.0               # the slowest rank's time
