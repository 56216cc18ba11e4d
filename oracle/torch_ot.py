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


# Rows per block of the dense sums below: large problems are summed block by
# block (the same terms in a different order), so that the temporaries of a
# 60,000 x 60,000 problem stay a few GB.
BLOCK_ROWS = 4096


def _blocked_sum(fn, n_rows):
    total = 0.0
    for r0 in range(0, n_rows, BLOCK_ROWS):
        total = total + fn(slice(r0, min(n_rows, r0 + BLOCK_ROWS)))
    return total


def primal(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """optimal_transport.py:45-53 (np.nan_to_num of log 0 -> the most negative double)."""
    torch = _torch()
    n_rows, n_cols = p.shape[0], q.shape[0]
    marg = fdiv(lambda1, R @ dy, p, dx) + fdiv(lambda2, R.T @ dx, q, dy)
    ent = epsilon * _blocked_sum(lambda s: torch.sum(R[s] * torch.nan_to_num(torch.log(R[s])) - R[s] + K[s]),
                                 n_rows)
    return marg + (ent + _blocked_sum(lambda s: torch.sum(R[s] * C[s]), n_rows)) / (n_rows * n_cols)


def dual(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """optimal_transport.py:56-62."""
    torch = _torch()
    n_rows, n_cols = p.shape[0], q.shape[0]
    return (- fdivstar(lambda1, - epsilon * torch.log(a), p, dx)
            - fdivstar(lambda2, - epsilon * torch.log(b), q, dy)
            - epsilon * _blocked_sum(lambda s: torch.sum(R[s] - K[s]), n_rows) / (n_rows * n_cols))


def _stabilised_kernel(u, C, v, eps, out=None):
    """exp((u_i - C_ij + v_j) / eps), built block by block (into ``out`` when given)."""
    torch = _torch()
    K = torch.empty_like(C) if out is None else out
    for r0 in range(0, C.shape[0], BLOCK_ROWS):
        s = slice(r0, min(C.shape[0], r0 + BLOCK_ROWS))
        torch.exp((u[s, None] - C[s] + v[None, :]) / eps, out=K[s])
    return K


def _scaled(K, a, b):
    """(K.T * a).T * b, block by block."""
    torch = _torch()
    R = torch.empty_like(K)
    for r0 in range(0, K.shape[0], BLOCK_ROWS):
        s = slice(r0, min(K.shape[0], r0 + BLOCK_ROWS))
        torch.mul(K[s] * a[s, None], b[None, :], out=R[s])
    return R


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
    R = K = K0 = None
    for stage in range(n_scalings + 1):
        gap = math.inf
        u = u + eps_i * torch.log(a)
        v = v + eps_i * torch.log(b)
        eps_i = eps_i / scale_factor
        K0 = _stabilised_kernel(torch.zeros_like(u), C, torch.zeros_like(v), eps_i, out=K0 if stage else None)
        alpha1 = lambda1 / (lambda1 + eps_i)
        alpha2 = lambda2 / (lambda2 + eps_i)
        K = _stabilised_kernel(u, C, v, eps_i, out=K if stage else None)
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
                    K = _stabilised_kernel(u, C, v, eps_i, out=K)
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
                R = _scaled(K, a, b)
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
    R = _scaled(K, a, b)
    del K, K0
    return R.div_(C.shape[1])


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
        med = kth_smallest(flat, k + 1)
    else:
        med = 0.5 * (kth_smallest(flat, k) + kth_smallest(flat, k + 1))
    return C.div_(med)


def kth_smallest(flat, k, block=1 << 26):
    """The k-th smallest (1-based) entry of a 1-D tensor, exactly (np.median's
    middle values): bounds from a sorted sample, a blockwise count below and
    between them, and a sort of only the entries between them."""
    torch = _torch()
    n = flat.numel()
    if n <= block:
        return float(torch.kthvalue(flat, k).values)
    g = torch.Generator(device=flat.device).manual_seed(0)
    sample = torch.sort(flat[torch.randint(0, n, (1 << 20,), device=flat.device, generator=g)]).values
    q = k / n
    for width in (0.002, 0.02, 0.2, 1.0):
        lo = float(sample[max(0, int((q - width) * sample.numel()))]) if q - width > 0 else -math.inf
        hi = float(sample[min(sample.numel() - 1, int((q + width) * sample.numel()))]) if q + width < 1 else math.inf
        below = 0
        mid = []
        for b0 in range(0, n, block):
            x = flat[b0:b0 + block]
            below += int((x < lo).sum())
            mid.append(x[(x >= lo) & (x <= hi)])
        mid = torch.cat(mid)
        if below < k <= below + mid.numel():
            return float(torch.sort(mid).values[k - below - 1])
    raise RuntimeError('kth_smallest: no bracket found')
