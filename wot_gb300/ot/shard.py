"""Sharding a batch of transport problems over ranks (one GPU per rank).

Items (day pair x parameter set) are independent, so N ranks split them with
no data-path collective: each rank solves the items of its longest-processing-
time share (greedy by estimated work, largest first, onto the least-loaded rank)
and the ranks only meet to gather results and to take the slowest rank's time.
The reference computes maps one by one in one process (wot/ot/ot_model.py:124-201).
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
