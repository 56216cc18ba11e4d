"""Transport-map files (the subset of wot/io/io.py the transport-map path uses).

``h5ad`` / ``loom`` go through anndata when it is installed (the reference's
own writer, wot/io/io.py:439-452). Without anndata, maps are written as
``.npz`` archives (X, obs columns, obs/var ids) under the same naming scheme,
``{prefix}_{t0}_{t1}`` (ot_model.py:183-189), and read back by
``read_dataset`` and ``TransportMapModel.from_directory``.
"""
from __future__ import annotations

import logging
import os

import numpy as np

from .dataset import Dataset, Frame

logger = logging.getLogger('wot')


def _have_anndata():
    try:
        import anndata  # noqa: F401
        return True
    except ImportError:
        return False


def check_file_extension(name, output_format):
    """Append the format's extension unless present (wot/io/io.py:366-375)."""
    expected = {'txt': '.txt', 'txt.gz': '.txt.gz', 'loom': '.loom', 'h5ad': '.h5ad', 'npz': '.npz'}
    ext = expected.get(output_format, '.' + output_format)
    if output_format in ('h5ad', 'loom') and not _have_anndata():
        ext = '.npz'
    if not str(name).lower().endswith(ext):
        name = str(name) + ext
    return name


def write_dataset(ds, path, output_format='h5ad'):
    if output_format in ('h5ad', 'loom') and _have_anndata() and type(ds).__module__.startswith('anndata'):
        if output_format == 'h5ad':
            ds.write(path)
        else:
            ds.write_loom(path)
        return
    if output_format in ('h5ad', 'loom') and not _have_anndata():
        logger.warning('anndata is not installed: writing %s as .npz', path)
    obs = ds.obs
    cols = {('obs:' + c): np.asarray(obs[c]) for c in list(obs.columns)}
    np.savez(path if str(path).endswith('.npz') else str(path) + '.npz', X=np.asarray(ds.X),
             obs_index=np.asarray(obs.index).astype(str), var_index=np.asarray(ds.var.index).astype(str), **cols)


def read_dataset(path):
    """Read a map written by write_dataset (npz, or h5ad/loom through anndata)."""
    path = str(path)
    if path.endswith('.npz'):
        with np.load(path, allow_pickle=False) as z:
            cols = {k[4:]: z[k] for k in z.files if k.startswith('obs:')}
            return Dataset(z['X'], Frame(cols, index=z['obs_index']), Frame(index=z['var_index']))
    import anndata
    if path.endswith('.loom'):
        return anndata.read_loom(path)
    return anndata.read_h5ad(path)


def read_ids(path):
    """(obs ids, var ids) of a map file without loading X when possible."""
    path = str(path)
    if path.endswith('.npz'):
        with np.load(path, allow_pickle=False) as z:
            return z['obs_index'], z['var_index']
    ds = read_dataset(path)
    return np.asarray(ds.obs.index).astype(str), np.asarray(ds.var.index).astype(str)


def write_learned_growth(tables, path):
    """Concatenated g0..gk obs tables as tab-separated text with an 'id' column
    (ot_model.py:196-201)."""
    cols = list(tables[0].columns)
    with open(path, 'w') as f:
        f.write('\t'.join(['id'] + cols) + '\n')
        for t in tables:
            idx = np.asarray(t.index)
            data = [np.asarray(t[c]) for c in cols]
            for r in range(len(idx)):
                f.write('\t'.join([str(idx[r])] + [repr(float(d[r])) for d in data]) + '\n')
