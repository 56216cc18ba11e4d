"""Sharding a batch of transport problems over ranks (one GPU per rank).

Items (day pair x parameter set) are independent, so N ranks split them with
no data-path collective: each rank solves the items of its longest-processing-
time share (greedy by estimated work, largest first, onto the least-loaded rank)
and the ranks only meet to gather results and to take the slowest rank's time.
The reference computes maps one by one in one process (wot/ot/ot_model.py:124-201).

``solve_sharded`` is the sharded batch: the partition is made from the pairs'
shapes alone (cell counts), so a rank builds the costs of only the pairs its
items use; its maps stay on its GPU, and one gather of per-item summaries
(statuses, iteration counts, which rank holds the map) is the only collective.
"""
from __future__ import annotations

import heapq


def lpt_partition(weights, n_parts):
    """Indices of `weights` split into n_parts lists by LPT (largest first onto
    the least-loaded part); each list is returned in ascending index order."""
    if n_parts < 1:
        raise ValueError('n_parts must be >= 1')
    heap = [(0.0, p) for p in range(n_parts)]
    parts = [[] for _ in range(n_parts)]
    for k in sorted(range(len(weights)), key=lambda k: (-float(weights[k]), k)):
        load, p = heapq.heappop(heap)
        parts[p].append(k)
        heapq.heappush(heap, (load + float(weights[k]), p))
    return [sorted(x) for x in parts]


def item_work(shapes, items, iterations=None):
    """Estimated work of each item: I * J of its pair, times its iteration count
    when known (from an earlier solve)."""
    w = []
    for k, (p, _cfg) in enumerate(items):
        I, J = shapes[p]
        w.append(float(I) * float(J) * (float(iterations[k]) if iterations is not None else 1.0))
    return w


def my_items(shapes, items, rank, world, iterations=None):
    """The item indices rank `rank` of `world` solves."""
    return lpt_partition(item_work(shapes, items, iterations), world)[rank]


def gather(local, group=None):
    """All ranks' (index, result) lists merged and ordered by index (on every
    rank); one all_gather_object, the only collective of a sharded batch."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return sorted(local, key=lambda t: t[0])
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, local, group=group)
    return sorted((t for part in out for t in part), key=lambda t: t[0])


def max_over_ranks(seconds, group=None):
    """The slowest rank's time (the job's time)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    if dist.get_backend(group) == 'nccl':
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def solve_sharded(shapes, items, build_pair, rank=0, world=1, group=None, solve=None, iterations=None):
    """This rank's share of a batch: the items ``my_items`` assigns it, solved
    in one batched call on its own GPU.

    ``shapes`` holds each pair's (I, J); ``items`` is a list of (pair index,
    config); ``build_pair(p)`` builds pair p on this rank's device (called only
    for the pairs this rank's items use, in ascending order); ``solve(pairs,
    items)`` solves a batch and returns one result per item (default:
    ``batch.solve_batched``). Returns ``(maps, summary)``: ``maps`` maps each
    item index this rank solved to its result (an ImplicitMap, held on this
    rank's device); ``summary`` lists, for every item of the whole batch in
    index order and on every rank, ``(index, {'rank', 'status', 'stats'})``,
    from one gather of these small records."""
    if solve is None:
        from .batch import solve_batched as solve
    mine = my_items(shapes, items, rank, world, iterations)
    used = sorted({items[k][0] for k in mine})
    local = {p: i for i, p in enumerate(used)}
    pairs = [build_pair(p) for p in used]
    results = solve(pairs, [(local[items[k][0]], items[k][1]) for k in mine]) if mine else []
    maps = dict(zip(mine, results))
    records = [(k, {'rank': rank, 'status': int(getattr(m, 'status', 0)), 'stats': dict(getattr(m, 'stats', {}))})
               for k, m in maps.items()]
    summary = gather(records, group)
    if [k for k, _ in summary] != list(range(len(items))):
        raise RuntimeError('sharded batch: the gathered summaries do not cover the %d items' % len(items))
    return maps, summary
