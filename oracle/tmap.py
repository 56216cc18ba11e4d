"""FP64 NumPy restatement of the map-analysis path (test infrastructure only).

Dense couplings are plain ``ndarray``s keyed by ``(t0, t1)``.

* ``push_forward`` / ``pull_back``   — wot/tmap/transport_map_model.py:235-299 / :301-365
  (``p @ X`` / ``(X @ p.T).T`` per day step, optional row normalisation)
* ``fates``                          — :40-69
* ``transition_table``               — :71-103
* ``trajectories``                   — :105-143
* ``glue`` / ``chain``               — wot/tmap/util.py:74-94, wot/tmap/chaining.py:4-40
* ``copy_populations``               — wot/population.py:39-67 (binary / normalised
  copies plus the "Other" population of cells no population covers)
"""
from __future__ import annotations

import numpy as np


def _step_maps(tmaps, timepoints, i, j):
    return [tmaps[(timepoints[k], timepoints[k + 1])] for k in range(i, j)]


def push_forward(tmaps, timepoints, P, t_from, t_to=None, normalize=True):
    """P: k x n(t_from) -> k x n(t_to)."""
    i = timepoints.index(t_from)
    j = i + 1 if t_to is None else timepoints.index(t_to)
    P = np.atleast_2d(np.asarray(P, dtype=np.float64))
    for X in _step_maps(tmaps, timepoints, i, j):
        P = P @ X
        if normalize:
            P = (P.T / np.sum(P, axis=1)).T
    return P


def pull_back(tmaps, timepoints, P, t_from, t_to=None, normalize=True):
    """P: k x n(t_from) -> k x n(t_to) with t_to < t_from."""
    i = timepoints.index(t_from)
    j = i - 1 if t_to is None else timepoints.index(t_to)
    P = np.atleast_2d(np.asarray(P, dtype=np.float64))
    for X in reversed(_step_maps(tmaps, timepoints, j, i)):
        P = (X @ P.T).T
        if normalize:
            P = (P.T / np.sum(P, axis=1)).T
    return P


def copy_populations(P, normalize=None, add_missing=False):
    """Population.copy restated on a k x n matrix of measures."""
    P = np.atleast_2d(np.array(P, dtype=np.float64))
    names_other = False
    if add_missing:
        missing = P.sum(axis=0) == 0
        if missing.any():
            P = np.vstack([P, missing.astype(np.float64)])
            names_other = True
    if normalize is True:
        P = P / P.sum(axis=1, keepdims=True)
    elif normalize is False:
        P = (P > 0.0).astype(np.float64)
    return P, names_other


def fates(tmaps, timepoints, P, t):
    """Rows: cells of every day <= t; columns: populations (+ 'Other')."""
    P, _ = copy_populations(P, normalize=False, add_missing=True)
    blocks = [P.T]
    i = timepoints.index(t)
    while i > 0:
        P = pull_back(tmaps, timepoints, P, timepoints[i], normalize=False)
        blocks.insert(0, P.T)
        i -= 1
    X = np.concatenate(blocks)
    return X / X.sum(axis=1, keepdims=1)


def trajectories(tmaps, timepoints, P, t):
    P, _ = copy_populations(P, normalize=True, add_missing=False)
    out = [P.T]
    i = timepoints.index(t)
    Q = P
    while i > 0:
        Q = pull_back(tmaps, timepoints, Q, timepoints[i])
        out.insert(0, Q.T)
        i -= 1
    i = timepoints.index(t)
    Q = P
    while i < len(timepoints) - 1:
        Q = push_forward(tmaps, timepoints, Q, timepoints[i])
        out.append(Q.T)
        i += 1
    return np.concatenate(out)


def transition_table(tmaps, timepoints, P_start, t_start, P_end, t_end):
    P_start, _ = copy_populations(P_start, normalize=False, add_missing=True)
    P_end, _ = copy_populations(P_end, normalize=False, add_missing=True)
    i = timepoints.index(t_end)
    Q = P_end
    while i > 0 and timepoints[i] > t_start:
        Q = pull_back(tmaps, timepoints, Q, timepoints[i], normalize=False)
        i -= 1
    T = P_start @ Q.T
    return T / T.sum()


def glue(X0, X1):
    """np.dot of two consecutive dense couplings (wot/tmap/util.py:93)."""
    return np.dot(X0, X1)


def chain(tmaps, path):
    X = tmaps[path[0]]
    for key in path[1:]:
        X = glue(X, tmaps[key])
    return X
