"""Minimal AnnData / DataFrame stand-ins.

The reference's API takes and returns ``anndata.AnnData`` with ``pandas``
obs/var frames. Neither package is required here: ``OTModel`` and
``TransportMapModel`` accept real AnnData objects when those packages are
installed and otherwise these small classes, which provide the subset the
transport-map path reads (``X``, ``obs[col]``, ``obs.columns``,
``obs.index``, row selection).
"""
from __future__ import annotations

import numpy as np


class Frame:
    """Column table: ``columns`` (list of names), ``index`` (ids), ``frame[name]`` -> ndarray."""

    def __init__(self, data=None, index=None):
        data = dict(data or {})
        n = None
        for v in data.values():
            n = len(v)
            break
        if index is None:
            index = np.arange(n if n is not None else 0).astype(str)
        self.index = np.asarray(index)
        self._cols = {k: np.asarray(v) for k, v in data.items()}
        for k, v in self._cols.items():
            if len(v) != len(self.index):
                raise ValueError('column %s has %d rows, index has %d' % (k, len(v), len(self.index)))

    @property
    def columns(self):
        return list(self._cols.keys())

    def __getitem__(self, key):
        if isinstance(key, str):
            return self._cols[key]
        rows = _rows(key, len(self.index))
        return Frame({k: v[rows] for k, v in self._cols.items()}, index=self.index[rows])

    def __setitem__(self, key, value):
        value = np.asarray(value)
        if value.ndim == 0:
            value = np.full(len(self.index), value)
        self._cols[key] = value

    def __contains__(self, key):
        return key in self._cols

    def __len__(self):
        return len(self.index)

    def copy(self):
        return Frame({k: v.copy() for k, v in self._cols.items()}, index=self.index.copy())

    def to_dict(self):
        return {k: v.tolist() for k, v in self._cols.items()}


class Dataset:
    """AnnData-like: ``X`` (n_obs x n_vars), ``obs`` and ``var`` Frames."""

    def __init__(self, X=None, obs=None, var=None):
        self.X = X
        n_obs = X.shape[0] if X is not None else (len(obs) if obs is not None else 0)
        n_var = X.shape[1] if X is not None and getattr(X, 'ndim', 2) == 2 else (len(var) if var is not None else 0)
        self.obs = obs if obs is not None else Frame(index=np.arange(n_obs).astype(str))
        self.var = var if var is not None else Frame(index=np.arange(n_var).astype(str))

    @property
    def shape(self):
        return (len(self.obs), len(self.var))

    def __getitem__(self, key):
        if isinstance(key, tuple):
            rows, cols = key
        else:
            rows, cols = key, slice(None)
        r = _rows(rows, self.shape[0])
        c = _rows(cols, self.shape[1])
        if self.X is None:
            X = None
        else:
            # slices index X as views (no copy of the expression matrix)
            X = self.X[rows if isinstance(rows, slice) else r]
            X = X[:, cols] if isinstance(cols, slice) else X[:, c]
        return Dataset(X, self.obs[r], self.var[c])

    def copy(self):
        return Dataset(None if self.X is None else self.X.copy(), self.obs.copy(), self.var.copy())


def _rows(key, n):
    if isinstance(key, slice):
        return np.arange(n)[key]
    key = np.asarray(key)
    if key.dtype == bool:
        return np.nonzero(key)[0]
    return key.astype(np.int64)


def column(frame, name):
    """``frame[name]`` as an ndarray for a Frame or a pandas DataFrame."""
    v = frame[name]
    return np.asarray(getattr(v, 'values', v))


def columns(frame):
    return list(frame.columns)


def index(frame):
    return np.asarray(frame.index)


def dense(X):
    """Sparse or dense matrix -> dense FP64 ndarray."""
    if hasattr(X, 'toarray'):
        X = X.toarray()
    return np.asarray(X, dtype=np.float64)


def make_result(X, obs_cols, obs_index, var_index, like=None):
    """Build the reference's return object: an AnnData when the input was one
    (and anndata is importable), else a Dataset."""
    if like is not None and type(like).__module__.startswith('anndata'):
        import anndata
        import pandas as pd
        return anndata.AnnData(X, pd.DataFrame(index=obs_index, data=obs_cols), pd.DataFrame(index=var_index))
    return Dataset(X, Frame(obs_cols, index=obs_index), Frame(index=var_index))
