"""Transport maps held as potentials instead of dense matrices.

A solve returns the absorbed potentials (u_bar, v_bar) and the final epsilon;
the map the reference returns is then
    tmap_ij = exp((u_bar_i + v_bar_j - s |x_i - y_j|^2) / eps) * scale,
scale = 1/J (or 1 when max_iter was hit), s the cost scale. An
``ImplicitCoupling`` keeps the points (and, when it was built, the FP32 cost)
and applies the map to populations without forming it:
    pull back  (tmap @ p.T).T   (transport_map_model.py:356)
        out_i = exp(u_bar_i/eps + log scale) sum_j exp(v_bar_j/eps + log p_j - s c_ij/eps)
    push forward  p @ tmap      (transport_map_model.py:290)
        out_j = exp(v_bar_j/eps + log scale) sum_i exp(u_bar_i/eps + log p_i - s c_ij/eps)
on the tensor cores from the points (``wotg_apply_points``: the cost recomputed
tile by tile, one exp per entry shared by every population, the populations'
weights applied in the epilogue) when the points are held (at most 62
dimensions), else as one log-sum-exp half-step per population on the
materialised cost or its transpose (``wotg_lse_matvec_multi``, every
population in one pass; built from the points for the call when they have more
dimensions). A 60000 x 60000 map costs 1 MB of potentials instead of 28.8 GB
of FP64.
"""
from __future__ import annotations

import math

from .. import _native as N
from . import device as D

LOG2E = 1.0 / math.log(2.0)


class ImplicitCoupling:
    def __init__(self, u_bar, v_bar, eps, cost_scale, log_scale, X=None, Y=None, cost=None, CT=None,
                 row_sums=None, stats=None):
        self.u_bar, self.v_bar = u_bar, v_bar
        self.eps = float(eps)
        self.cost_scale = float(cost_scale)
        self.log_scale = float(log_scale)
        self.X, self.Y = X, Y
        self.cost, self.CT = cost, CT
        self.row_sums = row_sums
        self.stats = stats or {}

    @classmethod
    def from_solve(cls, cost: D.DeviceCost, res: D.SolveResult, keep_cost=False):
        """From a ``device.solve(..., want_potentials=True)`` result on a cost
        built from points (the FP32 cost is dropped unless keep_cost)."""
        st = res.stats
        log_scale = 0.0 if st.get('hit_max_iter') else -math.log(cost.J)
        return cls(res.u_bar, res.v_bar, st['final_epsilon'], cost.scale, log_scale, X=cost.X, Y=cost.Y,
                   cost=cost if keep_cost else None, row_sums=res.row_sums, stats=st)

    @property
    def shape(self):
        return (self.u_bar.shape[0], self.v_bar.shape[0])

    def dense(self):
        """I x J FP64 device tensor of the coupling (builds the FP32 cost if needed)."""
        cost = self.cost
        if cost is None:
            cost = D.cost_from_points(self.X, self.Y)
            cost.scale = self.cost_scale
        return D.coupling_from_potentials(cost, self.u_bar, self.v_bar, self.eps, self.log_scale)

    def _apply(self, P, src_pot, tgt_pot, src_pts, tgt_pts, C=None, ldc=0):
        torch = N.require_cuda()
        P = D._dev_f64(P, torch)
        if P.dim() == 1:
            P = P.reshape(1, -1)
        rows, cols = src_pot.shape[0], tgt_pot.shape[0]
        if P.shape[1] != cols:
            raise ValueError('population length %d does not match %d cells' % (P.shape[1], cols))
        if src_pts is None and C is None:
            raise ValueError('this implicit coupling holds neither points nor the cost for this direction')
        inv_eps = 1.0 / self.eps
        if C is None and src_pts.shape[1] > D.TC_MAX_DIM:
            # too many dimensions for the tensor-core packing: this direction's cost from the points
            c = D.cost_from_points(src_pts, tgt_pts)
            C, ldc = c.C, c.ldc
        if src_pts is not None and C is None:
            return D.apply_points(src_pts, tgt_pts, tgt_pot * inv_eps, src_pot * inv_eps + self.log_scale, P,
                                  self.cost_scale * inv_eps)
        W = tgt_pot.reshape(1, -1) * inv_eps + torch.log(P)            # natural log weights, k x cols
        ldw = N.round_up(cols, 4)
        W2 = torch.zeros((W.shape[0], ldw), dtype=torch.float32, device='cuda')
        W2[:, :cols] = W * LOG2E
        k2 = self.cost_scale * inv_eps * LOG2E
        L = D.lse_multi(C, rows, cols, ldc, W2, [k2] * W.shape[0])
        return torch.exp(L + src_pot.reshape(1, -1) * inv_eps + self.log_scale)

    def pull_back(self, P, normalize=True):
        """(tmap @ P.T).T for populations P (k x J) -> k x I (transport_map_model.py:356-358)."""
        c = self.cost
        out = self._apply(P, self.u_bar, self.v_bar, self.X, self.Y,
                          C=None if c is None else c.C, ldc=0 if c is None else c.ldc)
        return out / out.sum(dim=1, keepdim=True) if normalize else out

    def push_forward(self, P, normalize=True):
        """P @ tmap for populations P (k x I) -> k x J (transport_map_model.py:290-292)."""
        CT = self.CT
        out = self._apply(P, self.v_bar, self.u_bar, self.Y, self.X,
                          C=CT, ldc=0 if CT is None else CT.stride(0))
        return out / out.sum(dim=1, keepdim=True) if normalize else out
