"""FP64 NumPy restatement of the per-pair orchestration (test infrastructure only).

* ``compute_pca``                 — wot/ot/util.py:240-255. The reference fits
  scikit-learn ``PCA(n_components, random_state=58951)`` on ``x.T`` (cells are
  the PCA *features*), which picks the randomized SVD solver at these shapes.
  This restatement uses an exact SVD of the same double-centred matrix, so
  coordinates agree with the reference up to sign/rotation within the top
  subspace and to randomized-SVD error; parity of the solver is therefore
  pinned on shared coordinates (both sides fed the same ``p0_x``, ``p1_x``).
* ``compute_pca_reference``       — the same PCA as the reference computes it:
  scikit-learn's solver choice and, for its randomized solver, the randomized
  range finder (Halko, Martinsson, Tropp 2011, Alg. 4.4) with LU-normalised
  power iterations, seeded by ``numpy.random.RandomState(58951)``, restated
  with NumPy / SciPy calls; pinned to the reference's own output in
  ``tests/golden/pair_120x150.npz`` and to scikit-learn where it is installed.
* ``compute_default_cost_matrix`` — wot/ot/ot_model.py:242-253 (coordinates
  scaled by the singular values, squared Euclidean as
  ``|x|^2 - 2 x.y + |y|^2`` clipped at 0 like scikit-learn's
  ``pairwise_distances(metric='sqeuclidean')``, divided by ``np.median``).
* ``compute_single_transport_map`` — wot/ot/ot_model.py:255-326 (day
  selection, PCA, cost unless given, ``G = growth ** (t1 - t0)``, growth
  iterations, ``g0..gk`` learned-growth columns).
"""
from __future__ import annotations

import numpy as np

from . import optimal_transport as ot

DEFAULT_CONFIG = {'local_pca': 30, 'growth_iters': 1, 'epsilon': 0.05, 'lambda1': 1, 'lambda2': 50,
                  'epsilon0': 1, 'tau': 10000, 'scaling_iter': 3000, 'inner_iter_max': 50,
                  'tolerance': 1e-8, 'max_iter': 1e7, 'batch_size': 5, 'extra_iter': 1000}


def compute_pca(m1, m2, n_components):
    """Double-centred PCA of the stacked cells (wot/ot/util.py:240-255), exact SVD.

    Returns ``(pca_1, pca_2, singular_values, mean_shift)`` where ``pca_k`` are
    the rows of ``components_.T`` for each day.
    """
    x = np.vstack([np.asarray(m1, dtype=np.float64), np.asarray(m2, dtype=np.float64)])
    mean_shift = x.mean(axis=0)
    x = x - mean_shift
    n_components = min(n_components, x.shape[0])
    xt = x.T                                  # genes are the samples, cells the features
    xt = xt - xt.mean(axis=0)                 # PCA centring of each feature (cell)
    _, s, vt = np.linalg.svd(xt, full_matrices=False)
    comp = vt[:n_components].T
    n1 = m1.shape[0]
    return comp[:n1], comp[n1:], s[:n_components], mean_shift


def sqeuclidean(a, b):
    """|a|^2 - 2 a.b + |b|^2, clipped at 0 (scikit-learn's sqeuclidean formula)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = -2.0 * a @ b.T
    d += (a * a).sum(axis=1)[:, None]
    d += (b * b).sum(axis=1)[None, :]
    np.maximum(d, 0.0, out=d)
    return d


def compute_pca_reference(m1, m2, n_components, seed=58951, n_oversamples=10):
    """The reference's PCA (wot/ot/util.py:240-255: scikit-learn
    ``PCA(n_components, random_state=58951).fit(x.T)``) restated: returns
    ``(pca_1, pca_2, singular_values, mean_shift, solver)``."""
    import scipy.linalg as sl
    x = np.vstack([np.asarray(m1, dtype=np.float64), np.asarray(m2, dtype=np.float64)])
    mean_shift = x.mean(axis=0)
    x = x - mean_shift
    k = min(n_components, x.shape[0])
    data = x.T                                   # genes x cells: genes are the samples
    data = data - data.mean(axis=0)              # PCA centring of each feature (cell)
    n_s, n_f = data.shape
    if n_f <= 1000 and n_s >= 10 * n_f:
        solver = 'covariance_eigh'
    elif max(n_s, n_f) <= 500:
        solver = 'full'
    elif 1 <= k < 0.8 * min(n_s, n_f):
        solver = 'randomized'
    else:
        solver = 'full'
    if solver == 'randomized':
        n_iter = 7 if k < 0.1 * min(n_s, n_f) else 4
        transpose = n_s < n_f
        M = data.T if transpose else data
        Q = np.random.RandomState(seed).normal(size=(M.shape[1], k + n_oversamples))
        for _ in range(n_iter):
            Q, _ = sl.lu(M @ Q, permute_l=True)
            Q, _ = sl.lu(M.T @ Q, permute_l=True)
        Q, _ = sl.qr(M @ Q, mode='economic')
        Uh, s, Vt = sl.svd(Q.T @ M, full_matrices=False)
        comp = (Q @ Uh)[:, :k].T if transpose else Vt[:k]       # k x cells
        s = s[:k]
    else:
        _, s, vt = np.linalg.svd(data, full_matrices=False)
        comp, s = vt[:k], s[:k]
    i = np.argmax(np.abs(comp), axis=1)
    comp = comp * np.sign(comp[np.arange(comp.shape[0]), i])[:, None]
    comp = comp.T
    n1 = np.asarray(m1).shape[0]
    return comp[:n1], comp[n1:], s, mean_shift, solver


def compute_default_cost_matrix(a, b, eigenvals=None):
    """Median-normalised squared-Euclidean cost (wot/ot/ot_model.py:242-253)."""
    if eigenvals is not None:
        a = a.dot(eigenvals)
        b = b.dot(eigenvals)
    c = sqeuclidean(a, b)
    return c / np.median(c)


def compute_single_transport_map(X, day, t0, t1, growth=None, C=None, solver='duality_gap', pca='exact',
                                 **params):
    """One transport map from day ``t0`` to ``t1`` (wot/ot/ot_model.py:255-326).

    Returns ``(tmap, obs_growth)`` with ``obs_growth = {'g0': ..., ...}``, or
    ``None`` when a day has no cells. ``pca`` 'exact' uses ``compute_pca``,
    'reference' the reference's own PCA (``compute_pca_reference``).
    """
    config = dict(DEFAULT_CONFIG)
    config.update(params)
    sel0 = day == float(t0)
    sel1 = day == float(t1)
    if sel0.sum() == 0 or sel1.sum() == 0:
        return None
    local_pca = config.pop('local_pca', None)
    eigenvals = None
    if local_pca is not None and local_pca > 0:
        if pca == 'reference':
            x0, x1, s, _, _ = compute_pca_reference(X[sel0], X[sel1], local_pca)
        else:
            x0, x1, s, _ = compute_pca(X[sel0], X[sel1], local_pca)
        eigenvals = np.diag(s)
    else:
        x0, x1 = X[sel0], X[sel1]
    if C is None:
        C = compute_default_cost_matrix(x0, x1, eigenvals)
    delta = t1 - t0
    G = np.power(growth[sel0], delta) if growth is not None else np.ones(C.shape[0])
    fn = ot.transport_stablev2 if solver == 'fixed_iters' else ot.optimal_transport_duality_gap
    tmap, learned = ot.compute_transport_matrix(solver=fn, C=C, G=G, **config)
    learned.append(tmap.sum(axis=1))
    obs = {'g' + str(i): np.power(g, 1.0 / delta) for i, g in enumerate(learned)}
    return tmap, obs
