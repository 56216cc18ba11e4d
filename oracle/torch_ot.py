"""FP64 restatement of the reference's default solver on torch tensors (test
infrastructure only: the checker for problems too large for the NumPy oracle).

Follows ``wot/ot/optimal_transport.py`` of wot 1.0.8 (optimal_transport.py:
10-33, 37-62, 67-164) in the same operation order as ``oracle.optimal_transport``
(the NumPy restatement, which is pinned to the reference's golden outputs), with
NumPy's dense arrays replaced by FP64 torch tensors so that the same arithmetic
runs on a GPU for 20,000 x 25,000 and 30,000 x 30,000 cost matrices: the dense
``K`` rebuilds, the two matrix-vector products per iteration and the dense
primal and dual objectives of every duality-gap check, exactly as the reference
evaluates them. ``tests/test_oracle.py`` checks it against the NumPy oracle.
"""
from __future__ import annotations

import logging
import math

logger = logging.getLogger('wot')


def _torch():
    import torch
    return torch


def compute_transport_matrix(solver, **params):
    """Growth-iteration driver (optimal_transport.py:10-33)."""
    learned = []
    tmap = None
    for it in range(params['growth_iters']):
        row_sums = params['G'] if it == 0 else tmap.sum(dim=1)
        params['G'] = row_sums
        learned.append(row_sums)
        tmap = solver(**params)
    return tmap, learned


def fdiv(lam, x, p, dx):
    """optimal_transport.py:37-38."""
    torch = _torch()
    return lam * torch.sum(dx * (x * (torch.log(x / p)) - x + p))


def fdivstar(lam, u, p, dx):
    """optimal_transport.py:41-42."""
    torch = _torch()
    return lam * torch.sum((p * dx) * (torch.exp(u / lam) - 1))


def primal(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """optimal_transport.py:45-53 (np.nan_to_num of log 0 -> the most negative double)."""
    torch = _torch()
    n_rows, n_cols = p.shape[0], q.shape[0]
    marg = fdiv(lambda1, R @ dy, p, dx) + fdiv(lambda2, R.T @ dx, q, dy)
    ent = epsilon * torch.sum(R * torch.nan_to_num(torch.log(R)) - R + K)
    return marg + (ent + torch.sum(R * C)) / (n_rows * n_cols)


def dual(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """optimal_transport.py:56-62."""
    torch = _torch()
    n_rows, n_cols = p.shape[0], q.shape[0]
    return (- fdivstar(lambda1, - epsilon * torch.log(a), p, dx)
            - fdivstar(lambda2, - epsilon * torch.log(b), q, dy)
            - epsilon * torch.sum(R - K) / (n_rows * n_cols))


def _stabilised_kernel(u, C, v, eps):
    torch = _torch()
    return torch.exp((u[:, None] - C + v[None, :]) / eps)


def optimal_transport_duality_gap(C, G, lambda1, lambda2, epsilon, batch_size, tolerance, tau,
                                  epsilon0, max_iter, stats=None, **ignored):
    """optimal_transport.py:67-164 on FP64 tensors (C, G on any one device)."""
    torch = _torch()
    C = C.to(torch.float64)
    dev = C.device
    n_scalings = 5
    scale_factor = math.exp(- math.log(epsilon) / n_scalings)
    n_rows, n_cols = C.shape
    dx = torch.full((n_rows,), 1.0 / n_rows, dtype=torch.float64, device=dev)
    dy = torch.full((n_cols,), 1.0 / n_cols, dtype=torch.float64, device=dev)
    p = G.to(device=dev, dtype=torch.float64)
    q = torch.ones(n_cols, dtype=torch.float64, device=dev) * p.mean()
    u = torch.zeros(n_rows, dtype=torch.float64, device=dev)
    v = torch.zeros(n_cols, dtype=torch.float64, device=dev)
    a = torch.ones(n_rows, dtype=torch.float64, device=dev)
    b = torch.ones(n_cols, dtype=torch.float64, device=dev)
    eps_i = epsilon0 * scale_factor
    n_iter = 0
    n_absorb = 0
    gap = math.inf
    R = None
    for stage in range(n_scalings + 1):
        gap = math.inf
        u = u + eps_i * torch.log(a)
        v = v + eps_i * torch.log(b)
        eps_i = eps_i / scale_factor
        K0 = torch.exp(-C / eps_i)
        alpha1 = lambda1 / (lambda1 + eps_i)
        alpha2 = lambda2 / (lambda2 + eps_i)
        K = _stabilised_kernel(u, C, v, eps_i)
        a = torch.ones(n_rows, dtype=torch.float64, device=dev)
        b = torch.ones(n_cols, dtype=torch.float64, device=dev)
        old_a, old_b = a, b
        final = stage == n_scalings
        threshold = tolerance if final else 1e-6
        while gap > threshold:
            for _ in range(batch_size if final else 5):
                n_iter += 1
                old_a, old_b = a, b
                a = (p / (K @ (b * dy))) ** alpha1 * torch.exp(-u / (lambda1 + eps_i))
                b = (q / (K.T @ (a * dx))) ** alpha2 * torch.exp(-v / (lambda2 + eps_i))
                if max(float(a.abs().max()), float(b.abs().max())) > tau:
                    u = u + eps_i * torch.log(a)
                    v = v + eps_i * torch.log(b)
                    K = _stabilised_kernel(u, C, v, eps_i)
                    a = torch.ones(n_rows, dtype=torch.float64, device=dev)
                    b = torch.ones(n_cols, dtype=torch.float64, device=dev)
                    n_absorb += 1
                if n_iter >= max_iter:
                    logger.warning("Reached max_iter with duality gap still above threshold. Returning")
                    if stats is not None:
                        stats.update(iterations=n_iter, absorptions=n_absorb, gap=gap, max_iter=True)
                    return (K.T * a).T * b
            true_a = a * torch.exp(u / eps_i)
            true_b = b * torch.exp(v / eps_i)
            if final:
                R = (K.T * a).T * b
                pri = primal(C, K0, R, dx, dy, p, q, true_a, true_b, eps_i, lambda1, lambda2)
                dua = dual(C, K0, R, dx, dy, p, q, true_a, true_b, eps_i, lambda1, lambda2)
                gap = float((pri - dua) / abs(pri))
                del R
            else:
                gap = max(
                    float(torch.linalg.norm(true_a - old_a * torch.exp(u / eps_i)) / (1 + torch.linalg.norm(true_a))),
                    float(torch.linalg.norm(true_b - old_b * torch.exp(v / eps_i)) / (1 + torch.linalg.norm(true_b))))
    if stats is not None:
        stats.update(iterations=n_iter, absorptions=n_absorb, gap=gap, max_iter=False)
    if math.isnan(gap):
        raise RuntimeError("Overflow encountered in duality gap computation, please report this incident")
    return (K.T * a).T * b / C.shape[1]


def default_cost(a, b):
    """Median-normalised squared-Euclidean cost (ot_model.py:242-253) in FP64
    from FP64 coordinates (already scaled by the singular values), as the
    NumPy oracle's ``compute_default_cost_matrix``: |a|^2 + |b|^2 - 2 a.b
    clipped at 0, divided by its median (the mean of the two middle values)."""
    torch = _torch()
    a = a.to(torch.float64)
    b = b.to(torch.float64)
    C = -2.0 * (a @ b.T)
    C += (a * a).sum(1)[:, None]
    C += (b * b).sum(1)[None, :]
    C.clamp_(min=0.0)
    flat = C.reshape(-1)
    n = flat.numel()
    k = n // 2
    if n % 2:
        med = torch.kthvalue(flat, k + 1).values
    else:
        med = 0.5 * (torch.kthvalue(flat, k).values + torch.kthvalue(flat, k + 1).values)
    return C / med
