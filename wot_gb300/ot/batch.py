"""Batched transport maps: many (day pair x parameter set) problems solved together.

The reference computes maps one after another (``OTModel.compute_all_transport_maps``,
wot/ot/ot_model.py:124-201) and a parameter sweep repeats that per parameter set.
``solve_batched`` hands every item to ``wotg_solve_batched``: one persistent
launch per Sinkhorn half-step over all items, each pair's cost read once for all
of its items, the reference's control flow per item on the device, replayed from
a CUDA graph. Each result is the reference's map for that item, held as
potentials (an ``ImplicitMap``) instead of a dense I x J matrix.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from .. import _native as N
from . import device as D
from .implicit import ImplicitCoupling


@dataclass
class BatchPair:
    """One day pair on the device: FP32 cost, its transpose, growth G."""
    cost: D.DeviceCost
    CT: object
    G: object

    @property
    def shape(self):
        return self.cost.shape


def prepare_pair(cost: D.DeviceCost, G) -> BatchPair:
    torch = N.require_cuda()
    Gd = D._dev_f64(G, torch).reshape(-1)
    if Gd.numel() != cost.I:
        raise ValueError('G has %d entries for %d source cells' % (Gd.numel(), cost.I))
    return BatchPair(cost, D.transpose_cost(cost), Gd)


class ImplicitMap(ImplicitCoupling):
    """One batch item's map as potentials: tmap_ij = exp((u_bar_i + v_bar_j - scale C_ij) / eps) * s,
    s = 1/J (or 1 when max_iter was hit), exactly the coupling the reference returns."""

    def __init__(self, pair, params, u_bar, v_bar, row_sums, learned_growth, stats, status):
        c = pair.cost
        log_scale = 0.0 if stats['hit_max_iter'] else -math.log(c.J)
        super().__init__(u_bar, v_bar, stats['final_epsilon'], c.scale, log_scale, X=c.X, Y=c.Y, cost=c,
                         CT=pair.CT, row_sums=row_sums, stats=stats)
        self.pair = pair
        self.params = params
        self.learned_growth = learned_growth
        self.status = status


def report_statuses(statuses, raise_nonfinite=True):
    """The reference's per-map outcomes for a batch's item statuses: the
    max_iter warning (optimal_transport.py:143-145) for each item that hit
    max_iter, and the RuntimeError of a NaN duality gap (optimal_transport.py:
    162-163) when any item ended non-finite (unless raise_nonfinite is False)."""
    bad = []
    for k, s in enumerate(statuses):
        s = int(s)
        if s == N.WOTG_MAX_ITER:
            N.check(s, 'wotg_solve_batched item %d' % k)
        elif s == N.WOTG_NONFINITE:
            bad.append(k)
        elif s != N.WOTG_OK:
            raise RuntimeError('wotg_solve_batched item %d: status %d' % (k, s))
    if bad and raise_nonfinite:
        raise RuntimeError('Overflow encountered in duality gap computation, please report this incident '
                           '(batch items %s)' % ', '.join(str(k) for k in bad))
    return bad


def solve_batched(pairs, items, raise_nonfinite=True):
    """Solve every item; ``items`` is a list of (pair index, config dict) with the
    reference's ot_config keys (duality-gap solver). Returns one ImplicitMap per item
    (its ``status`` the item's wotg status). Items that hit max_iter log the
    reference's warning; an item whose duality gap became NaN raises the
    reference's RuntimeError unless raise_nonfinite is False."""
    torch = N.require_cuda()
    lib = N.load()
    np_, ni = len(pairs), len(items)
    if ni == 0:
        return []
    hp = (N.Pair * np_)()
    for p, bp in enumerate(pairs):
        c = bp.cost
        hp[p] = N.Pair(I=c.I, J=c.J, C=c.C.data_ptr(), ldc=c.ldc, CT=bp.CT.data_ptr(), ldct=bp.CT.stride(0),
                       cost_scale=float(c.scale), G=bp.G.data_ptr())
    hi = (N.Item * ni)()
    row_off = col_off = g_off = 0
    offs = []
    for k, (p, cfg) in enumerate(items):
        if not 0 <= p < np_:
            raise ValueError('item %d names pair %d of %d' % (k, p, np_))
        params = D.make_params(cfg, N.SOLVER_DUALITY_GAP)
        c = pairs[p].cost
        hi[k] = N.Item(pair=p, params=params, row_offset=row_off, col_offset=col_off, growth_offset=g_off)
        offs.append((row_off, col_off, g_off, max(1, params.growth_iters)))
        row_off += c.I
        col_off += c.J
        g_off += c.I * max(1, params.growth_iters)
    u_bar = torch.empty(row_off, dtype=torch.float64, device='cuda')
    row_sums = torch.empty(row_off, dtype=torch.float64, device='cuda')
    v_bar = torch.empty(col_off, dtype=torch.float64, device='cuda')
    learned = torch.empty(g_off, dtype=torch.float64, device='cuda')
    nbytes = lib.wotg_batch_workspace_bytes(hp, np_, hi, ni)
    if nbytes == 0:
        raise ValueError('invalid batch (duality-gap solver only; positive epsilon, lambdas)')
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    stats = (N.Stats * ni)()
    statuses = (ctypes.c_int32 * ni)()
    N.check(lib.wotg_solve_batched(hp, np_, hi, ni, u_bar.data_ptr(), v_bar.data_ptr(), row_sums.data_ptr(),
                                   learned.data_ptr(), stats, statuses, ws.data_ptr(), nbytes, D._stream()),
            'wotg_solve_batched')
    report_statuses(statuses, raise_nonfinite)
    out = []
    for k, (p, cfg) in enumerate(items):
        ro, co, go, gi = offs[k]
        c = pairs[p].cost
        lg = [learned[go + g * c.I: go + (g + 1) * c.I] for g in range(gi)]
        out.append(ImplicitMap(pairs[p], dict(cfg), u_bar[ro:ro + c.I], v_bar[co:co + c.J], row_sums[ro:ro + c.I],
                               lg, stats[k].as_dict(), int(statuses[k])))
    return out
