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

The Gram matrix is not formed from the centred (dense) matrix: with x the
n x p stacked expression, mu its gene means and H = I - 11^T/p the centring
over genes (the second, per-cell centring),
    Gram = H (x^T x - n mu mu^T) H,
so only x^T x touches the cells. Expression matrices are mostly zeros
(log1p of counts); below ``SPARSE_DENSITY`` nonzeros x^T x is a sparse-dense
product (cuSPARSE, FP64) over the nonzeros instead of a dense FP64 GEMM, about
1/density times fewer FMAs on a part whose FP64 rate is low.
"""
from __future__ import annotations

import warnings

import numpy as np

from .. import _native as N
from ..dataset import dense


SPARSE_DENSITY = 0.3


def centred_gram(x, mu, sparse=None):
    """Gram matrix of the double-centred ``x`` (n x p, FP64, not centred) given
    its column means ``mu``: H (x^T x - n mu mu^T) H, H the centring over the p
    columns. ``sparse`` None picks the sparse product below SPARSE_DENSITY
    nonzeros. Any device."""
    import torch
    n, p = x.shape
    if sparse is None:
        sparse = int(torch.count_nonzero(x)) < SPARSE_DENSITY * x.numel()
    if sparse:
        with warnings.catch_warnings():         # torch marks sparse CSR as beta
            warnings.simplefilter('ignore', UserWarning)
            xs = x.T.contiguous().to_sparse_csr()   # p x n, the nonzeros only
            A = torch.sparse.mm(xs, x)
        A = 0.5 * (A + A.T)                     # exact symmetry for eigh
    else:
        A = x.T @ x
    A = A - n * torch.outer(mu, mu)
    r = A.mean(dim=1)
    return A - r[:, None] - r[None, :] + r.mean()


def compute_pca(m1, m2, n_components):
    """Returns ``(pca_1, pca_2, singular_values, mean_shift)`` as device tensors
    (FP64): pca_k are the components_.T rows of each day."""
    torch = N.require_cuda()
    x = torch.cat([torch.as_tensor(dense(m1), device='cuda', dtype=torch.float64),
                   torch.as_tensor(dense(m2), device='cuda', dtype=torch.float64)])
    mean_shift = x.mean(dim=0)
    n_components = min(int(n_components), x.shape[0])
    gram = centred_gram(x, mean_shift)        # genes x genes, FP64 on the device
    # the eigendecomposition of this small (genes x genes) matrix runs in NumPy
    evals, evecs = np.linalg.eigh(gram.cpu().numpy())
    order = np.argsort(evals)[::-1][:n_components].copy()
    s = torch.as_tensor(np.sqrt(np.clip(evals[order], 0.0, None)), device='cuda')
    U = torch.as_tensor(evecs[:, order], device='cuda')
    # V = Xc^T U S^-1 with Xc^T = (x - mean_shift) H: H U = U (U spans the range of a
    # matrix whose rows and columns sum to zero), so V = (x U - mean_shift . U) S^-1
    comp = (x @ U - (mean_shift @ U)[None, :]) / torch.where(s > 0, s, torch.ones_like(s))
    n1 = m1.shape[0]
    return comp[:n1], comp[n1:], s, mean_shift
