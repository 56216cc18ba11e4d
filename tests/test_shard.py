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


class _StubMap:
    """What a solve returns per item, as far as the sharded path reads it."""

    def __init__(self, pair_shape, cfg):
        self.status = 1 if cfg['epsilon'] < 0.02 else 0
        self.stats = {'iterations': int(1000 * cfg['epsilon']) + pair_shape[0]}
        self.pair_shape = pair_shape
        self.cfg = cfg


def _sharded_worker(rank, world, port, q):
    import torch.distributed as dist
    from wot_gb300.ot.shard import solve_sharded
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        shapes = [(100 * (p + 1), 50 * (p + 2)) for p in range(6)]
        items = [(p, {'epsilon': e, 'lambda1': l}) for p in range(6) for e in (0.01, 0.05) for l in (1, 3)]
        built, calls = [], []

        def build_pair(p):
            built.append(p)
            return ('pair', p, shapes[p])

        def solve(pairs, its):
            calls.append(len(its))
            return [_StubMap(pairs[lp][2], cfg) for lp, cfg in its]

        maps, summary = solve_sharded(shapes, items, build_pair, rank, world, solve=solve)
        mine = sorted(maps)
        ok = all(maps[k].pair_shape == shapes[items[k][0]] and maps[k].cfg == items[k][1] for k in mine)
        q.put((rank, mine, built, calls, summary, ok))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_run_a_sharded_batch():
    """shard.solve_sharded (the path OTModel.compute_transport_maps_batched
    takes with world > 1) on two gloo ranks around a stub solver: the ranks
    solve disjoint item sets that cover the batch, in one batched call each,
    build only the pairs their items use, get every item's result for its own
    pair and parameters, and all hold the same gathered summary of every item
    (status, iteration count, owning rank) in item order."""
    import multiprocessing as mp
    pytest.importorskip('torch')
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort(key=lambda t: t[0])
    (_, mine0, built0, calls0, sum0, ok0), (_, mine1, built1, calls1, sum1, ok1) = out
    n_items = 24
    assert ok0 and ok1
    assert not set(mine0) & set(mine1) and sorted(mine0 + mine1) == list(range(n_items))
    assert calls0 == [len(mine0)] and calls1 == [len(mine1)]
    items_pair = [k // 4 for k in range(n_items)]
    assert built0 == sorted({items_pair[k] for k in mine0})
    assert built1 == sorted({items_pair[k] for k in mine1})
    assert sum0 == sum1 and [k for k, _ in sum0] == list(range(n_items))
    for k, rec in sum0:
        assert rec['rank'] == (0 if k in mine0 else 1)
        assert rec['status'] == (1 if (k // 2) % 2 == 0 else 0)


def test_sharded_batch_on_one_rank_is_the_whole_batch():
    from wot_gb300.ot.shard import solve_sharded
    shapes = [(10, 20), (30, 40)]
    items = [(0, {'epsilon': 0.05}), (1, {'epsilon': 0.01}), (1, {'epsilon': 0.05})]
    maps, summary = solve_sharded(shapes, items, lambda p: ('pair', p, shapes[p]), 0, 1,
                                  solve=lambda pairs, its: [_StubMap(pairs[lp][2], c) for lp, c in its])
    assert sorted(maps) == [0, 1, 2] and [r['rank'] for _, r in summary] == [0, 0, 0]
    assert [r['status'] for _, r in summary] == [0, 1, 0]
