"""Local PCA of a day pair on the device (wot/ot/util.py:240-255).

The reference stacks both days' cells, removes the per-gene mean, and fits
``sklearn.decomposition.PCA(n_components, random_state=58951)`` on ``x.T``, so
genes are the samples and cells the features; the cell coordinates are the
rows of ``components_.T`` and ``singular_values_`` scale them in the cost.
Here the same double-centred matrix is decomposed exactly: the (genes x genes)
Gram matrix of the centred ``x.T`` is formed on the device in FP64, its small
eigendecomposition runs in NumPy, and the top eigenpairs give the singular
values and (projected on the device) the cell coordinates. The reference's
randomized SVD approximates exactly these, so coordinates agree up to sign,
rotation inside degenerate subspaces and the randomized solver's error.
"""
from __future__ import annotations

import numpy as np

from .. import _native as N
from ..dataset import dense


def compute_pca(m1, m2, n_components):
    """Returns ``(pca_1, pca_2, singular_values, mean_shift)`` as device tensors
    (FP64): pca_k are the components_.T rows of each day."""
    torch = N.require_cuda()
    x = torch.cat([torch.as_tensor(dense(m1), device='cuda', dtype=torch.float64),
                   torch.as_tensor(dense(m2), device='cuda', dtype=torch.float64)])
    mean_shift = x.mean(dim=0)
    x = x - mean_shift
    n_components = min(int(n_components), x.shape[0])
    xt = x.T                                  # genes x cells
    xt = xt - xt.mean(dim=0, keepdim=True)    # PCA centring of each cell (feature)
    gram = xt @ xt.T                          # genes x genes, FP64 GEMM on the device
    # the eigendecomposition of this small (genes x genes) matrix runs in NumPy
    evals, evecs = np.linalg.eigh(gram.cpu().numpy())
    order = np.argsort(evals)[::-1][:n_components].copy()
    s = torch.as_tensor(np.sqrt(np.clip(evals[order], 0.0, None)), device='cuda')
    U = torch.as_tensor(evecs[:, order], device='cuda')
    comp = (xt.T @ U) / torch.where(s > 0, s, torch.ones_like(s))   # V = Xc^T U S^-1
    n1 = m1.shape[0]
    return comp[:n1], comp[n1:], s, mean_shift
