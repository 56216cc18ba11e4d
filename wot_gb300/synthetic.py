"""Seeded synthetic single-cell time courses.

The reference ships no benchmark data and its tutorial dataset is not
redistributable here, so every measurement and parity case runs on
synthetic cells with the shapes and value distributions of the workloads
it is quoted on:

* counts are negative-binomial with dispersion 0.5 (mean ``mu``, size
  ``r = 1/0.5 = 2``, so ``var = mu + 0.5 mu^2``);
* each cell's mean profile is drawn around one of ``n_clusters`` cluster
  profiles whose per-gene means are lognormal(sigma=1); the cell jitters
  its log-means by a Gaussian (a Gaussian mixture in log-mean space) and
  clusters drift slowly with the day so that consecutive days differ;
* a global scale is solved for so that about ``zero_frac`` (90 %) of the
  counts are zero;
* expression is ``log1p(CP10k)``;
* per-cell growth rates are lognormal(0, 0.3).

Everything is a pure function of the seed (``numpy.random.default_rng``).
"""
from __future__ import annotations

import numpy as np

NB_SIZE = 2.0  # negative-binomial size r = 1 / dispersion(0.5)


def _scale_for_zero_fraction(mu: np.ndarray, zero_frac: float) -> float:
    """Bisect a global scale s so that mean((r/(r+s*mu))^r) == zero_frac."""
    lo, hi = 1e-6, 1e6
    for _ in range(200):
        mid = np.sqrt(lo * hi)
        z = np.mean((NB_SIZE / (NB_SIZE + mid * mu)) ** NB_SIZE)
        if z > zero_frac:
            lo = mid
        else:
            hi = mid
    return float(np.sqrt(lo * hi))


def time_course(cells_per_day, n_genes=1000, n_clusters=6, seed=0, zero_frac=0.9,
                jitter=0.25, drift=0.1, days=None):
    """Generate a synthetic time course.

    Parameters
    ----------
    cells_per_day : sequence of int
        Number of cells sampled at each day.
    n_genes, n_clusters, seed, zero_frac : see module docstring.
    days : sequence of float, optional
        Day labels (default 0, 1, 2, ...).

    Returns
    -------
    X : ndarray (sum(cells_per_day), n_genes) float64, log1p(CP10k)
    day : ndarray float64, the day of each cell
    growth : ndarray float64, lognormal(0, 0.3) growth rate of each cell
    """
    rng = np.random.default_rng(seed)
    cells_per_day = [int(n) for n in cells_per_day]
    if days is None:
        days = np.arange(len(cells_per_day), dtype=np.float64)
    days = np.asarray(days, dtype=np.float64)
    log_mu = rng.normal(0.0, 1.0, size=(n_clusters, n_genes))          # lognormal(sigma=1) means
    log_drift = rng.normal(0.0, drift, size=(n_clusters, n_genes))       # per-day drift
    weights = rng.dirichlet(np.ones(n_clusters) * 2.0, size=len(cells_per_day))
    n_total = int(sum(cells_per_day))
    cell_log_mu = np.empty((n_total, n_genes))
    day = np.empty(n_total)
    row = 0
    for t, n in enumerate(cells_per_day):
        k = rng.choice(n_clusters, size=n, p=weights[t])
        cell_log_mu[row:row + n] = (log_mu[k] + t * log_drift[k]
                                    + rng.normal(0.0, jitter, size=(n, n_genes)))
        day[row:row + n] = days[t]
        row += n
    mu = np.exp(cell_log_mu)
    s = _scale_for_zero_fraction(mu[: min(n_total, 2000)], zero_frac)
    mu *= s
    counts = rng.negative_binomial(NB_SIZE, NB_SIZE / (NB_SIZE + mu)).astype(np.float64)
    totals = np.maximum(counts.sum(axis=1, keepdims=True), 1.0)
    X = np.log1p(counts / totals * 1e4)
    growth = rng.lognormal(0.0, 0.3, size=n_total)
    return X, day, growth


def gaussian_mixture_points(n, d=30, n_components=10, seed=0, spread=1.0):
    """FP32 points from a Gaussian mixture (the differentiation workload's input)."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, spread, size=(n_components, d))
    k = rng.integers(0, n_components, size=n)
    return (centers[k] + rng.normal(0.0, 0.3, size=(n, d))).astype(np.float32)


def log_uniform_day_sizes(n_days, lo=1000, hi=30000, seed=2):
    """Per-day cell counts log-uniform in [lo, hi] (the batched time-course workload)."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_days)).astype(np.int64)


def course_profiles(n_days, n_genes=1000, n_clusters=20, seed=0, drift=0.1):
    """Cluster profiles of a long time course: lognormal(sigma=1) cluster means,
    per-day drift and per-day cluster weights, from one seeded stream."""
    rng = np.random.default_rng(seed)
    log_mu = rng.normal(0.0, 1.0, size=(n_clusters, n_genes))
    log_drift = rng.normal(0.0, drift, size=(n_clusters, n_genes))
    weights = rng.dirichlet(np.ones(n_clusters) * 2.0, size=n_days)
    mu0 = np.exp(log_mu[rng.integers(0, n_clusters, size=2000)])
    scale = _scale_for_zero_fraction(mu0, 0.9)
    return {'log_mu': log_mu, 'log_drift': log_drift, 'weights': weights, 'scale': scale, 'seed': seed}


def course_day(profiles, t, n, jitter=0.25):
    """Cells of day t of a long time course (same generator as time_course, one
    seeded stream per day so that days can be produced independently):
    returns X (n x genes, log1p(CP10k)) and growth rates (lognormal(0, 0.3))."""
    rng = np.random.default_rng([profiles['seed'], int(t) + 1])
    log_mu, log_drift = profiles['log_mu'], profiles['log_drift']
    k = rng.choice(log_mu.shape[0], size=int(n), p=profiles['weights'][t])
    mu = np.exp(log_mu[k] + t * log_drift[k] + rng.normal(0.0, jitter, size=(int(n), log_mu.shape[1])))
    mu *= profiles['scale']
    counts = rng.negative_binomial(NB_SIZE, NB_SIZE / (NB_SIZE + mu)).astype(np.float32)
    totals = np.maximum(counts.sum(axis=1, keepdims=True), 1.0)
    X = np.log1p(counts / totals * 1e4).astype(np.float32)
    growth = rng.lognormal(0.0, 0.3, size=int(n))
    return X, growth
