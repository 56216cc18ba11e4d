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
from dataclasses import dataclass, field

import numpy as np

from .. import _native as N
from . import device as D


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


@dataclass
class ImplicitMap:
    """A transport map as potentials: tmap_ij = exp((u_bar_i + v_bar_j - scale C_ij) / eps) * s,
    s = 1/J (or 1 when max_iter was hit), exactly the coupling the reference returns."""
    pair: BatchPair
    params: dict
    u_bar: object
    v_bar: object
    row_sums: object
    learned_growth: list
    stats: dict
    status: int
    eps: float = field(init=False)
    log_scale: float = field(init=False)

    def __post_init__(self):
        self.eps = float(self.stats['final_epsilon'])
        self.log_scale = 0.0 if self.stats['hit_max_iter'] else -math.log(self.pair.cost.J)

    @property
    def shape(self):
        return self.pair.shape

    def dense(self):
        """I x J FP64 device tensor of the coupling."""
        return D.coupling_from_potentials(self.pair.cost, self.u_bar, self.v_bar, self.eps, self.log_scale)

    def _lse(self, src, tgt_pot, P, C, ldc, rows, cols):
        torch = N.require_cuda()
        P = D._dev_f64(P, torch)
        if P.dim() == 1:
            P = P.reshape(1, -1)
        if P.shape[1] != cols:
            raise ValueError('population length %d does not match %d cells' % (P.shape[1], cols))
        k = P.shape[0]
        ldw = N.round_up(cols, 4)
        W = torch.zeros((k, ldw), dtype=torch.float32, device='cuda')
        with np.errstate(divide='ignore'):
            W[:, :cols] = ((tgt_pot / self.eps).reshape(1, -1) + torch.log(P)) * (1.0 / math.log(2.0))
        kappa2 = self.pair.cost.scale / self.eps / math.log(2.0)
        L = D.lse_multi(C, rows, cols, ldc, W, [kappa2] * k)
        return torch.exp(L + (src / self.eps).reshape(1, -1) + self.log_scale)

    def pull_back(self, p, normalize=True):
        """(tmap @ p.T).T for populations p (k x J): transport_map_model.py:356-358."""
        c = self.pair.cost
        out = self._lse(self.u_bar, self.v_bar, p, c.C, c.ldc, c.I, c.J)
        return out / out.sum(dim=1, keepdim=True) if normalize else out

    def push_forward(self, p, normalize=True):
        """p @ tmap for populations p (k x I): transport_map_model.py:290-292."""
        c = self.pair.cost
        out = self._lse(self.v_bar, self.u_bar, p, self.pair.CT, self.pair.CT.stride(0), c.J, c.I)
        return out / out.sum(dim=1, keepdim=True) if normalize else out


def solve_batched(pairs, items):
    """Solve every item; ``items`` is a list of (pair index, config dict) with the
    reference's ot_config keys (duality-gap solver). Returns one ImplicitMap per item."""
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
    out = []
    for k, (p, cfg) in enumerate(items):
        ro, co, go, gi = offs[k]
        c = pairs[p].cost
        lg = [learned[go + g * c.I: go + (g + 1) * c.I] for g in range(gi)]
        out.append(ImplicitMap(pairs[p], dict(cfg), u_bar[ro:ro + c.I], v_bar[co:co + c.J], row_sums[ro:ro + c.I],
                               lg, stats[k].as_dict(), int(statuses[k])))
    return out
