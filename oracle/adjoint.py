"""FP64 references for the gradient of the converged unbalanced OT objective.

TEST INFRASTRUCTURE (the oracle): only tests/ and bench.py's checks use this
module; the product path (wot_gb300.ot.adjoint, wotg_ot_adjoint) never does.

The objective is the reference's dual at the optimum
(wot/ot/optimal_transport.py:56-62):
    D = -lambda1 dx sum_i p_i (exp(-ubar_i/lambda1) - 1)
        -lambda2 dy sum_j q_j (exp(-vbar_j/lambda2) - 1) - eps dx dy sum_ij (R_ij - K0_ij),
    R_ij = exp((ubar_i + vbar_j - C_ij)/eps), K0_ij = exp(-C_ij/eps),
    q_j = mean(p) (optimal_transport.py:108), dx = 1/I, dy = 1/J,
with ubar = u + eps log a, vbar = v + eps log b. The reference's updates
(optimal_transport.py:131-135) written for these absorbed potentials are
    ubar_i = eps alpha1 (log p_i - log sum_j dy exp((vbar_j - C_ij)/eps))
    vbar_j = eps alpha2 (log q_j - log sum_i dx exp((ubar_i - C_ij)/eps))
(the stabilising u, v cancel exactly: alpha1 + eps/(lambda1 + eps) = 1), so a
fixed-epsilon iteration of these two lines has the same fixed point as the
reference's final stage. Everything here is FP64 torch on any device: the
unrolled iterations are differentiated by autograd, and the converged objective
by central finite differences.
"""
from __future__ import annotations

import math

import torch


def cost(x, y, scale):
    """C_ij = scale |x_i - y_j|^2 in FP64 (difference form)."""
    return scale * ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)


def iterate(C, logp, logq, ubar, vbar, eps, lambda1, lambda2, n):
    I, J = C.shape
    a1 = lambda1 / (lambda1 + eps)
    a2 = lambda2 / (lambda2 + eps)
    ldx, ldy = -math.log(I), -math.log(J)
    for _ in range(n):
        ubar = eps * a1 * (logp - torch.logsumexp(ldy + (vbar[None, :] - C) / eps, dim=1))
        vbar = eps * a2 * (logq - torch.logsumexp(ldx + (ubar[:, None] - C) / eps, dim=0))
    return ubar, vbar


def dual(C, p, q, ubar, vbar, eps, lambda1, lambda2):
    I, J = C.shape
    dx, dy = 1.0 / I, 1.0 / J
    R = torch.exp((ubar[:, None] + vbar[None, :] - C) / eps)
    K0 = torch.exp(-C / eps)
    return (-lambda1 * dx * (p * (torch.exp(-ubar / lambda1) - 1)).sum()
            - lambda2 * dy * (q * (torch.exp(-vbar / lambda2) - 1)).sum()
            - eps * dx * dy * (R - K0).sum())


def _marginals(logg, dt, J):
    p = torch.exp(dt * logg)
    q = p.mean() * torch.ones(J, dtype=p.dtype, device=p.device)
    return p, q


def converge(x, y, logg, eps, lambda1, lambda2, scale, ubar=None, vbar=None, dt=1.0, tol=1e-13,
             max_iter=200000, check_every=20):
    """Fixed-epsilon iterations to max |change| < tol (warm start optional)."""
    with torch.no_grad():
        C = cost(x, y, scale)
        p, q = _marginals(logg, dt, C.shape[1])
        if ubar is None:
            ubar = torch.zeros(C.shape[0], dtype=C.dtype, device=C.device)
            vbar = torch.zeros(C.shape[1], dtype=C.dtype, device=C.device)
        n = 0
        while n < max_iter:
            u0, v0 = ubar, vbar
            ubar, vbar = iterate(C, torch.log(p), torch.log(q), ubar, vbar, eps, lambda1, lambda2, check_every)
            n += check_every
            ch = max(float((ubar - u0).abs().max()), float((vbar - v0).abs().max()))
            if ch < tol:
                break
        return ubar, vbar, n


def objective(x, y, logg, eps, lambda1, lambda2, scale, ubar0=None, vbar0=None, dt=1.0, tol=1e-13):
    """Converged objective D and its potentials."""
    ubar, vbar, _ = converge(x, y, logg, eps, lambda1, lambda2, scale, ubar0, vbar0, dt=dt, tol=tol)
    with torch.no_grad():
        C = cost(x, y, scale)
        p, q = _marginals(logg, dt, C.shape[1])
        return float(dual(C, p, q, ubar, vbar, eps, lambda1, lambda2)), ubar, vbar


def unrolled_gradient(x, y, logg, eps, lambda1, lambda2, scale, ubar0, vbar0, n_unroll=30, dt=1.0):
    """Autograd through n_unroll iterations started at converged potentials
    (detached), then the dual: (D, dD/dx, dD/dy, dD/dlogg)."""
    x = x.detach().clone().requires_grad_(True)
    y = y.detach().clone().requires_grad_(True)
    logg = logg.detach().clone().requires_grad_(True)
    C = cost(x, y, scale)
    p, q = _marginals(logg, dt, C.shape[1])
    ubar, vbar = iterate(C, torch.log(p), torch.log(q), ubar0.detach(), vbar0.detach(), eps, lambda1, lambda2,
                         n_unroll)
    D = dual(C, p, q, ubar, vbar, eps, lambda1, lambda2)
    D.backward()
    return float(D.detach()), x.grad, y.grad, logg.grad


def fd_gradient(x, y, logg, eps, lambda1, lambda2, scale, coords, ubar0, vbar0, h=1e-4, dt=1.0, tol=1e-13):
    """Central differences of the converged objective at coords = [(name, index), ...]
    with name in {'x', 'y', 'logg'} and index a tuple into that tensor."""
    out = []
    for name, idx in coords:
        vals = []
        for sgn in (1.0, -1.0):
            xs, ys, ls = x.clone(), y.clone(), logg.clone()
            t = {'x': xs, 'y': ys, 'logg': ls}[name]
            t[idx] += sgn * h
            D, _, _ = objective(xs, ys, ls, eps, lambda1, lambda2, scale, ubar0, vbar0, dt=dt, tol=tol)
            vals.append(D)
        out.append((vals[0] - vals[1]) / (2 * h))
    return out
