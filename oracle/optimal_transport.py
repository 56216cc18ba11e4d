"""FP64 NumPy restatement of the reference solvers (test infrastructure only).

Follows ``wot/ot/optimal_transport.py`` of wot 1.0.8 line by line in its
arithmetic (same operation order, same quirks) so that it reproduces the
reference's couplings to FP64 round-off:

* ``compute_transport_matrix``        — optimal_transport.py:10-33
* ``fdiv`` / ``fdivstar``             — :37-42 (Chizat's KL entropy and conjugate)
* ``primal`` / ``dual``               — :45-62
* ``optimal_transport_duality_gap``   — :67-164 (default solver)
* ``transport_stablev2``              — :167-236 (``solver='fixed_iters'``)

Quirks kept on purpose (they change iteration counts or outputs):

* 5 epsilon scalings => 6 stages; the final epsilon is ``epsilon0 * epsilon``
  (:101-120);
* the stage-exit test compares against ``old_a`` taken at the start of the
  last iteration of the batch, even when that iteration absorbed (:132,
  :148-160);
* on ``max_iter`` the coupling is returned WITHOUT the final ``/ J``
  (:143-145);
* a NaN duality gap after the final stage raises ``RuntimeError`` (:162-163).

Each solver accepts an optional ``stats`` dict that it fills with the
iteration count, number of tau-absorptions and the last duality gap; the
reference has no such output, it is only used to compare iteration counts.
"""
from __future__ import annotations

import logging

import numpy as np

logger = logging.getLogger('wot')


def compute_transport_matrix(solver, **params):
    """Growth-iteration driver (optimal_transport.py:10-33).

    Runs ``growth_iters`` full solves; the first uses ``G``, each later one
    uses the row sums of the previous coupling as its source growth.
    Returns ``(tmap, learned_growth)``.
    """
    growth_iters = params['growth_iters']
    learned = []
    tmap = None
    for it in range(growth_iters):
        row_sums = params['G'] if it == 0 else tmap.sum(axis=1)
        params['G'] = row_sums
        learned.append(row_sums)
        tmap = solver(**params)
    return tmap, learned


def fdiv(lam, x, p, dx):
    """lam * KL-type divergence sum (optimal_transport.py:37-38)."""
    return lam * np.sum(dx * (x * (np.log(x / p)) - x + p))


def fdivstar(lam, u, p, dx):
    """Its convex conjugate (optimal_transport.py:41-42)."""
    return lam * np.sum((p * dx) * (np.exp(u / lam) - 1))


def primal(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """Primal objective of the KL-relaxed problem (optimal_transport.py:45-53)."""
    n_rows, n_cols = len(p), len(q)
    with np.errstate(divide='ignore'):
        marg = fdiv(lambda1, np.dot(R, dy), p, dx) + fdiv(lambda2, np.dot(R.T, dx), q, dy)
        ent = epsilon * np.sum(R * np.nan_to_num(np.log(R)) - R + K)
        return marg + (ent + np.sum(R * C)) / (n_rows * n_cols)


def dual(C, K, R, dx, dy, p, q, a, b, epsilon, lambda1, lambda2):
    """Dual objective (optimal_transport.py:56-62)."""
    n_rows, n_cols = len(p), len(q)
    return (- fdivstar(lambda1, - epsilon * np.log(a), p, dx)
            - fdivstar(lambda2, - epsilon * np.log(b), q, dy)
            - epsilon * np.sum(R - K) / (n_rows * n_cols))


def _stabilised_kernel(u, C, v, eps):
    return np.exp((u[:, None] - C + v[None, :]) / eps)


def optimal_transport_duality_gap(C, G, lambda1, lambda2, epsilon, batch_size, tolerance, tau,
                                  epsilon0, max_iter, stats=None, **ignored):
    """Default solver: epsilon-scaled stabilised unbalanced Sinkhorn stopped on
    the relative duality gap (optimal_transport.py:67-164)."""
    C = np.asarray(C, dtype=np.float64)
    n_scalings = 5
    scale_factor = np.exp(- np.log(epsilon) / n_scalings)
    n_rows, n_cols = C.shape
    dx = np.ones(n_rows) / n_rows
    dy = np.ones(n_cols) / n_cols
    p = G
    q = np.ones(n_cols) * np.average(G)
    u = np.zeros(n_rows)
    v = np.zeros(n_cols)
    a = np.ones(n_rows)
    b = np.ones(n_cols)
    eps_i = epsilon0 * scale_factor
    n_iter = 0
    n_absorb = 0
    gap = np.inf
    R = None
    for stage in range(n_scalings + 1):
        gap = np.inf
        u = u + eps_i * np.log(a)
        v = v + eps_i * np.log(b)
        eps_i = eps_i / scale_factor
        K0 = np.exp(-C / eps_i)
        alpha1 = lambda1 / (lambda1 + eps_i)
        alpha2 = lambda2 / (lambda2 + eps_i)
        K = _stabilised_kernel(u, C, v, eps_i)
        a = np.ones(n_rows)
        b = np.ones(n_cols)
        old_a, old_b = a, b
        final = stage == n_scalings
        threshold = tolerance if final else 1e-6
        while gap > threshold:
            for _ in range(batch_size if final else 5):
                n_iter += 1
                old_a, old_b = a, b
                a = (p / (K.dot(np.multiply(b, dy)))) ** alpha1 * np.exp(-u / (lambda1 + eps_i))
                b = (q / (K.T.dot(np.multiply(a, dx)))) ** alpha2 * np.exp(-v / (lambda2 + eps_i))
                if max(max(abs(a)), max(abs(b))) > tau:
                    u = u + eps_i * np.log(a)
                    v = v + eps_i * np.log(b)
                    K = _stabilised_kernel(u, C, v, eps_i)
                    a = np.ones(n_rows)
                    b = np.ones(n_cols)
                    n_absorb += 1
                if n_iter >= max_iter:
                    logger.warning("Reached max_iter with duality gap still above threshold. Returning")
                    if stats is not None:
                        stats.update(iterations=n_iter, absorptions=n_absorb, gap=gap, max_iter=True)
                    return (K.T * a).T * b
            true_a = a * np.exp(u / eps_i)
            true_b = b * np.exp(v / eps_i)
            if final:
                R = (K.T * a).T * b
                pri = primal(C, K0, R, dx, dy, p, q, true_a, true_b, eps_i, lambda1, lambda2)
                dua = dual(C, K0, R, dx, dy, p, q, true_a, true_b, eps_i, lambda1, lambda2)
                gap = (pri - dua) / abs(pri)
            else:
                gap = max(
                    np.linalg.norm(true_a - old_a * np.exp(u / eps_i)) / (1 + np.linalg.norm(true_a)),
                    np.linalg.norm(true_b - old_b * np.exp(v / eps_i)) / (1 + np.linalg.norm(true_b)))
    if stats is not None:
        stats.update(iterations=n_iter, absorptions=n_absorb, gap=gap, max_iter=False)
    if np.isnan(gap):
        raise RuntimeError("Overflow encountered in duality gap computation, please report this incident")
    return R / C.shape[1]


def transport_stablev2(C, lambda1, lambda2, epsilon, scaling_iter, G, tau, epsilon0, extra_iter,
                       inner_iter_max, stats=None, **ignored):
    """Fixed-iteration solver (optimal_transport.py:167-236)."""
    warm_start = tau is not None
    eps_final = epsilon

    def schedule(n):
        return (epsilon0 - eps_final) * np.exp(-n) + eps_final

    eps_i = epsilon0 if warm_start else epsilon
    dx = np.ones(C.shape[0]) / C.shape[0]
    dy = np.ones(C.shape[1]) / C.shape[1]
    p = G
    q = np.ones(C.shape[1]) * np.average(G)
    u = np.zeros(len(p))
    v = np.zeros(len(q))
    b = np.ones(len(q))
    K = np.exp(-C / eps_i)
    alpha1 = lambda1 / (lambda1 + eps_i)
    alpha2 = lambda2 / (lambda2 + eps_i)
    eps_index = 0
    since_change = 0
    n_absorb = 0
    for _ in range(scaling_iter):
        a = (p / (K.dot(np.multiply(b, dy)))) ** alpha1 * np.exp(-u / (lambda1 + eps_i))
        b = (q / (K.T.dot(np.multiply(a, dx)))) ** alpha2 * np.exp(-v / (lambda2 + eps_i))
        since_change += 1
        if max(max(abs(a)), max(abs(b))) > tau:
            u = u + eps_i * np.log(a)
            v = v + eps_i * np.log(b)
            K = _stabilised_kernel(u, C, v, eps_i)
            a = np.ones(len(p))
            b = np.ones(len(q))
            n_absorb += 1
        if warm_start and since_change == inner_iter_max:
            eps_index += 1
            since_change = 0
            u = u + eps_i * np.log(a)
            v = v + eps_i * np.log(b)
            eps_i = schedule(eps_index)
            alpha1 = lambda1 / (lambda1 + eps_i)
            alpha2 = lambda2 / (lambda2 + eps_i)
            K = _stabilised_kernel(u, C, v, eps_i)
            a = np.ones(len(p))
            b = np.ones(len(q))
    for _ in range(extra_iter):
        a = (p / (K.dot(np.multiply(b, dy)))) ** alpha1 * np.exp(-u / (lambda1 + eps_i))
        b = (q / (K.T.dot(np.multiply(a, dx)))) ** alpha2 * np.exp(-v / (lambda2 + eps_i))
    if stats is not None:
        stats.update(iterations=scaling_iter + extra_iter, absorptions=n_absorb, final_epsilon=eps_i)
    R = (K.T * a).T * b
    return R / C.shape[1]
