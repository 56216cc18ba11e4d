"""Drop-in solver functions of wot.ot (wot/ot/optimal_transport.py), run on the GPU.

Same names, signatures, return values and error behaviour as the reference:

* ``compute_transport_matrix(solver, **params) -> (tmap, learned_growth)``
  (optimal_transport.py:10-33). When ``solver`` is one of the two solvers of
  this module, all ``growth_iters`` solves run on the device in one
  ``wotg_compute_transport_matrix`` call; any other callable is driven by the
  reference's Python loop.
* ``optimal_transport_duality_gap(C, G, lambda1, lambda2, epsilon, batch_size,
  tolerance, tau, epsilon0, max_iter, **ignored)`` (:67-164), the default.
* ``transport_stablev2(C, lambda1, lambda2, epsilon, scaling_iter, G, tau,
  epsilon0, extra_iter, inner_iter_max, **ignored)`` (:167-236).

``C`` is the reference's dense cost (ndarray, or a CUDA tensor), or a
``DeviceCost`` already on the device (the coordinates path of ``OTModel``).
Results are FP64 ndarrays like the reference's.
"""
from __future__ import annotations

import logging

import numpy as np

from .. import _native as N
from . import device as D

logger = logging.getLogger('wot')


def _as_cost(C):
    if isinstance(C, D.DeviceCost):
        return C
    return D.cost_from_dense(C)


def _host(t):
    return None if t is None else t.cpu().numpy()


def _run(C, G, cfg, solver_id):
    cost = _as_cost(C)
    res = D.solve(cost, G, cfg, solver_id, want_tmap=True)
    return _host(res.tmap), [_host(g) for g in res.learned_growth], res


def optimal_transport_duality_gap(C, G, lambda1, lambda2, epsilon, batch_size, tolerance, tau, epsilon0,
                                  max_iter, **ignored):
    """Entropic unbalanced OT with epsilon scaling, stopped on the relative
    duality gap (optimal_transport.py:67-164). Returns the I x J coupling."""
    cfg = dict(lambda1=lambda1, lambda2=lambda2, epsilon=epsilon, batch_size=batch_size, tolerance=tolerance,
               tau=tau, epsilon0=epsilon0, max_iter=max_iter, growth_iters=1)
    return _run(C, G, cfg, N.SOLVER_DUALITY_GAP)[0]


def transport_stablev2(C, lambda1, lambda2, epsilon, scaling_iter, G, tau, epsilon0, extra_iter,
                       inner_iter_max, **ignored):
    """Fixed-iteration stabilised unbalanced Sinkhorn (optimal_transport.py:167-236)."""
    cfg = dict(lambda1=lambda1, lambda2=lambda2, epsilon=epsilon, scaling_iter=scaling_iter, tau=tau,
               epsilon0=epsilon0, extra_iter=extra_iter, inner_iter_max=inner_iter_max, growth_iters=1)
    return _run(C, G, cfg, N.SOLVER_FIXED_ITERS)[0]


_NATIVE = {optimal_transport_duality_gap: N.SOLVER_DUALITY_GAP, transport_stablev2: N.SOLVER_FIXED_ITERS}


def native_solver_id(solver):
    """The libwotg solver id of a solver callable of this module, else None."""
    return _NATIVE.get(solver)


def compute_transport_matrix(solver, **params):
    """Growth-iteration driver (optimal_transport.py:10-33)."""
    sid = native_solver_id(solver)
    if sid is None:
        G = params['G']
        growth_iters = params['growth_iters']
        learned_growth = []
        tmap = None
        for i in range(growth_iters):
            row_sums = G if i == 0 else tmap.sum(axis=1)
            params['G'] = row_sums
            learned_growth.append(row_sums)
            tmap = solver(**params)
        return tmap, learned_growth
    if params['growth_iters'] < 1:
        raise UnboundLocalError("local variable 'tmap' referenced before assignment")
    tmap, learned, _ = _run(params['C'], params['G'], params, sid)
    # the first entry is the caller's G itself in the reference
    learned[0] = params['G']
    return tmap, learned


# --- the objectives of the duality-gap test (optimal_transport.py:37-62) -------
# The solvers evaluate these in O(I+J) on the device from their own state; these
# functions give the reference's dense forms for arrays a caller holds. Inputs go
# to the device in FP64; each returns a Python float.

def _dev(x, torch):
    if isinstance(x, torch.Tensor):
        return x.to(dtype=torch.float64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device='cuda')


def _fdiv(l, x, p, dx):
    import torch
    return l * torch.sum(dx * (x * torch.log(x / p) - x + p))


def _fdivstar(l, u, p, dx):
    import torch
    return l * torch.sum((p * dx) * (torch.exp(u / l) - 1))


def _primal(C, K, R, dx, dy, p, q, epsilon, lambda1, lambda2):
    import torch
    I, J = p.shape[0], q.shape[0]
    return (_fdiv(lambda1, R @ dy, p, dx) + _fdiv(lambda2, R.T @ dx, q, dy)
            + (epsilon * torch.sum(R * torch.nan_to_num(torch.log(R)) - R + K) + torch.sum(R * C)) / (I * J))


def _dual(K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    import torch
    I, J = p.shape[0], q.shape[0]
    return (-_fdivstar(lambda1, -epsilon * torch.log(a), p, dx) - _fdivstar(lambda2, -epsilon * torch.log(b), q, dy)
            - epsilon * torch.sum(R - K) / (I * J))


def fdiv(l, x, p, dx):
    """KL-type divergence term (optimal_transport.py:37-38)."""
    torch = N.require_cuda()
    return float(_fdiv(l, _dev(x, torch), _dev(p, torch), _dev(dx, torch)))


def fdivstar(l, u, p, dx):
    """Its convex conjugate (optimal_transport.py:41-42)."""
    torch = N.require_cuda()
    return float(_fdivstar(l, _dev(u, torch), _dev(p, torch), _dev(dx, torch)))


def primal(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """Primal objective of the unbalanced problem (optimal_transport.py:45-53)."""
    torch = N.require_cuda()
    C, K, R, dx, dy, p, q = (_dev(v, torch) for v in (C, K, R, dx, dy, p, q))
    return float(_primal(C, K, R, dx, dy, p, q, epsilon, lambda1, lambda2))


def dual(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """Dual objective (optimal_transport.py:56-62)."""
    torch = N.require_cuda()
    K, R, dx, dy, p, q, a, b = (_dev(v, torch) for v in (K, R, dx, dy, p, q, a, b))
    return float(_dual(K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2))
