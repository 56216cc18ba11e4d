"""Differentiable unbalanced OT objective (no counterpart in the reference).

``ot_objective(x, y, log_g)`` returns the converged regularised unbalanced OT
objective of the reference's solver (its dual at the optimum,
wot/ot/optimal_transport.py:56-62) for the cost C_ij = s |x_i - y_j|^2 and the
source growth p = exp(dt * log_g), as a torch scalar whose backward gives
d/dx, d/dy and d/dlog_g. Forward: the duality-gap solve
(``wotg_compute_transport_matrix``), a few hundred warm-started iterations at the
final epsilon (``wotg_refine_potentials``) so that the potentials sit at the
optimum, then ``wotg_ot_adjoint``, which evaluates the envelope-theorem gradient
in one pass over the implicit coupling per side with the cost recomputed from the
points. The cost scale s is a constant of the objective (1/median of the first
cost when not given, not differentiated).
"""
from __future__ import annotations

import math

import numpy as np

from .. import _native as N
from . import device as D

DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


def _function():
    torch = N.require_cuda()

    class UnbalancedOT(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, y, log_g, cfg, cost_scale, dt, refine_iters, form):
            X = x.detach().to(device='cuda', dtype=torch.float32).contiguous()
            Y = y.detach().to(device='cuda', dtype=torch.float32).contiguous()
            lg = log_g.detach().to(device='cuda', dtype=torch.float64).reshape(-1)
            p = torch.exp(dt * lg)
            cost = D.cost_from_points(X, Y)
            cost.scale = float(cost_scale)
            res = D.solve(cost, p, cfg, N.SOLVER_DUALITY_GAP, want_tmap=False, want_potentials=True, form=form)
            eps = res.stats['final_epsilon']
            u, v = res.u_bar, res.v_bar
            if refine_iters > 0:
                D.refine(cost, p, cfg, u, v, eps, refine_iters, form=form)  # in place
            obj, gx, gy, gp = D.ot_adjoint(X, Y, cost.scale, eps, cfg['lambda1'], cfg['lambda2'], u, v, p)
            ctx.save_for_backward(gx, gy, gp * p * dt)
            ctx.dtypes = (x.dtype, y.dtype, log_g.dtype, x.device, y.device, log_g.device, log_g.shape)
            ctx.stats = res.stats
            return torch.tensor(obj, dtype=torch.float64, device=x.device)

        @staticmethod
        def backward(ctx, g):
            gx, gy, glg = ctx.saved_tensors
            tx, ty, tl, dx, dy, dl, shl = ctx.dtypes
            g = g.to(device='cuda', dtype=torch.float64)
            return ((g * gx).to(device=dx, dtype=tx), (g * gy).to(device=dy, dtype=ty),
                    (g * glg).reshape(shl).to(device=dl, dtype=tl), None, None, None, None, None)

    return UnbalancedOT


_FN = None


def ot_objective(x, y, log_g, epsilon=0.05, lambda1=1.0, lambda2=50.0, cost_scale=None, dt=1.0,
                 refine_iters=400, form='auto', **cfg):
    """Converged unbalanced OT objective (differentiable in x, y, log_g).

    x: I x d, y: J x d points (d <= 64); log_g: I log-growth rates; cost
    C = cost_scale |x - y|^2 with cost_scale = 1/median when None (a constant).
    Other keyword arguments are the reference's solver keys (epsilon0, tau,
    tolerance, batch_size, max_iter)."""
    global _FN
    torch = N.require_cuda()
    if _FN is None:
        _FN = _function()
    conf = dict(DEFAULTS, epsilon=epsilon, lambda1=lambda1, lambda2=lambda2, growth_iters=1, **cfg)
    if cost_scale is None:
        c = D.cost_from_points(x.detach().to(device='cuda', dtype=torch.float32),
                               y.detach().to(device='cuda', dtype=torch.float32))
        cost_scale = 1.0 / D.median(c)
        del c
    return _FN.apply(x, y, log_g, conf, float(cost_scale), float(dt), int(refine_iters), form)
