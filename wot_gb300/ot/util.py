"""Local PCA of a day pair on the device (wot/ot/util.py:240-255).

The reference stacks both days' cells, removes the per-gene mean, and fits
``sklearn.decomposition.PCA(n_components, random_state=58951)`` on ``x.T``, so
genes are the samples and cells the features; the cell coordinates are the
rows of ``components_.T`` and ``singular_values_`` scale them in the cost.
``solver='exact'`` decomposes the same double-centred matrix exactly: the (genes x genes)
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

``solver='reference'`` (the default) reproduces the reference's decomposition itself:
scikit-learn's choice of solver for this shape and, where that is its
randomized solver, the randomized range finder of Halko, Martinsson and Tropp
(SIAM Review 53(2), 2011, Algorithm 4.4 with a re-orthonormalised power
iteration) with the reference's seed: the same Gaussian test matrix
(``numpy.random.RandomState(58951)``), 10 oversampling columns, 7 (or 4) power
iterations, then the SVD of the small projected matrix and the sign convention
of the largest entry of each component. The products with the double-centred
matrix run on the device from the sparse expression and rank-one centring
terms; only 40 x 40 and 40 x genes factorisations run on the host. The result
equals scikit-learn's to FP64 rounding (the subspace does not depend on how
the iterates are re-orthonormalised).
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


def sklearn_pca_solver(n_samples, n_features, n_components):
    """scikit-learn's PCA(svd_solver='auto') choice (releases 1.5 and later) for
    an n_samples x n_features data matrix; the reference fits genes x cells."""
    if n_features <= 1000 and n_samples >= 10 * n_features:
        return 'covariance_eigh'
    if max(n_samples, n_features) <= 500:
        return 'full'
    if 1 <= n_components < 0.8 * min(n_samples, n_features):
        return 'randomized'
    return 'full'


class _Centred:
    """The reference's double-centred matrix as an operator, never formed:
    T = x - 1 mu^T - c 1^T (cells x genes; mu the gene means, c each cell's mean
    over genes after removing mu), i.e. the transpose of the matrix the
    reference hands to scikit-learn. Products with T and T^T come from x (or
    its sparse form) and two rank-one terms."""

    def __init__(self, x, mu, sparse=None):
        import torch
        self.x, self.mu = x, mu
        n, p = x.shape
        self.c = (x @ torch.ones(p, dtype=x.dtype, device=x.device)) / p - float(mu.sum()) / p
        if sparse is None:
            sparse = int(torch.count_nonzero(x)) < SPARSE_DENSITY * x.numel()
        self.xs = self.xts = None
        if sparse:
            with warnings.catch_warnings():         # torch marks sparse CSR as beta
                warnings.simplefilter('ignore', UserWarning)
                self.xs = x.to_sparse_csr()
                self.xts = x.T.contiguous().to_sparse_csr()

    def _mm(self, a, b):
        import torch
        if a is None:
            return None
        with warnings.catch_warnings():
            warnings.simplefilter('ignore', UserWarning)
            return torch.sparse.mm(a, b)

    def t_mul(self, Q):
        """T @ Q, Q genes x r."""
        xq = self._mm(self.xs, Q) if self.xs is not None else self.x @ Q
        return xq - (self.mu @ Q)[None, :] - self.c[:, None] * Q.sum(dim=0)[None, :]

    def tt_mul(self, Q):
        """T^T @ Q, Q cells x r."""
        xq = self._mm(self.xts, Q) if self.xts is not None else self.x.T @ Q
        return xq - self.mu[:, None] * Q.sum(dim=0)[None, :] - (self.c @ Q)[None, :]


def _orthonormal(A):
    """An orthonormal basis of A's columns: Cholesky QR twice, the r x r
    factorisations on the host; Householder QR on the host when A's Gram
    matrix is not positive definite (rank-deficient iterates)."""
    import torch
    for _ in range(2):
        G = (A.T @ A).cpu().numpy()
        try:
            L = np.linalg.cholesky(G)
        except np.linalg.LinAlgError:
            q, _ = np.linalg.qr(A.cpu().numpy())
            return torch.as_tensor(q, device=A.device)
        Rinv = np.linalg.inv(L.T)
        A = A @ torch.as_tensor(Rinv, dtype=A.dtype, device=A.device)
    return A


def reference_pca(x, mu, n_components, seed=58951, n_oversamples=10, sparse=None):
    """The reference's local PCA of the stacked cells ``x`` (cells x genes, FP64
    tensor, gene means ``mu``): scikit-learn's PCA(n_components,
    random_state=seed) fitted on the double-centred genes x cells matrix.
    Returns (coordinates: cells x k = components_.T, singular values: k, solver).
    Any device."""
    import torch
    n, p = x.shape
    k = int(n_components)
    solver = sklearn_pca_solver(p, n, k)
    if solver != 'randomized':
        return None, None, solver
    T = _Centred(x, mu, sparse)
    r = k + n_oversamples
    n_iter = 7 if k < 0.1 * min(p, n) else 4
    transpose = p < n            # scikit-learn works on M = data^T = T when there are more cells than genes
    mul, tmul = (T.t_mul, T.tt_mul) if transpose else (T.tt_mul, T.t_mul)
    cols = p if transpose else n
    Q = torch.as_tensor(np.random.RandomState(seed).normal(size=(cols, r)), dtype=x.dtype, device=x.device)
    for _ in range(n_iter):
        Q = _orthonormal(mul(Q))
        Q = _orthonormal(tmul(Q))
    Q = _orthonormal(mul(Q))
    B = tmul(Q).T                # r x cols = Q^T M
    Uh, s, Vt = np.linalg.svd(B.cpu().numpy(), full_matrices=False)
    if transpose:
        comp = Q @ torch.as_tensor(Uh[:, :k], dtype=x.dtype, device=x.device)     # cells x k
    else:
        comp = torch.as_tensor(Vt[:k].T.copy(), dtype=x.dtype, device=x.device)  # cells x k
    return _largest_entry_positive(comp), torch.as_tensor(s[:k], dtype=x.dtype, device=x.device), solver


def _largest_entry_positive(comp):
    """scikit-learn's sign convention for components (columns here): the entry of
    largest magnitude of each is positive."""
    import torch
    i = torch.argmax(comp.abs(), dim=0)
    sign = torch.sign(comp[i, torch.arange(comp.shape[1], device=comp.device)])
    return comp * torch.where(sign == 0, torch.ones_like(sign), sign)[None, :]


def compute_pca(m1, m2, n_components, solver='reference'):
    """Returns ``(pca_1, pca_2, singular_values, mean_shift)`` as device tensors
    (FP64): pca_k are the components_.T rows of each day. ``solver``
    'reference' (the default) reproduces the reference's scikit-learn PCA (its
    randomized solver where scikit-learn picks that one, else the exact
    decomposition its full solvers compute); 'exact' decomposes the
    double-centred matrix exactly."""
    torch = N.require_cuda()
    x = torch.cat([torch.as_tensor(dense(m1), device='cuda', dtype=torch.float64),
                   torch.as_tensor(dense(m2), device='cuda', dtype=torch.float64)])
    mean_shift = x.mean(dim=0)
    n_components = min(int(n_components), x.shape[0])
    n1 = m1.shape[0]
    if solver not in ('exact', 'reference'):
        raise ValueError("PCA solver must be 'exact' or 'reference'")
    if solver == 'reference':
        comp, s, _ = reference_pca(x, mean_shift, n_components)
        if comp is not None:
            return comp[:n1], comp[n1:], s, mean_shift
    gram = centred_gram(x, mean_shift)        # genes x genes, FP64 on the device
    # the eigendecomposition of this small (genes x genes) matrix runs in NumPy
    evals, evecs = np.linalg.eigh(gram.cpu().numpy())
    order = np.argsort(evals)[::-1][:n_components].copy()
    s = torch.as_tensor(np.sqrt(np.clip(evals[order], 0.0, None)), device='cuda')
    U = torch.as_tensor(evecs[:, order], device='cuda')
    # V = Xc^T U S^-1 with Xc^T = (x - mean_shift) H: H U = U (U spans the range of a
    # matrix whose rows and columns sum to zero), so V = (x U - mean_shift . U) S^-1
    comp = (x @ U - (mean_shift @ U)[None, :]) / torch.where(s > 0, s, torch.ones_like(s))
    if solver == 'reference':
        comp = _largest_entry_positive(comp)
    return comp[:n1], comp[n1:], s, mean_shift


class FittedPCA:
    """The attributes of the reference's fitted scikit-learn PCA that its callers
    read (ot_model.py:302 takes ``singular_values_``): ``components_`` (k x cells),
    ``singular_values_`` (k), ``n_components_``, ``mean_`` (the per-cell mean over
    genes that scikit-learn removed), all host FP64 arrays."""

    def __init__(self, components, singular_values, mean):
        self.components_ = components
        self.singular_values_ = singular_values
        self.n_components_ = int(singular_values.shape[0])
        self.mean_ = mean


def compute_pca_reference_api(m1, m2, n_components, solver='reference'):
    """``wot.ot.compute_pca`` with the reference's return values (wot/ot/util.py:
    240-255): ``(pca_1, pca_2, pca, mean_shift)`` as host arrays, ``pca`` a
    FittedPCA. Computed on the device by ``compute_pca`` (``solver`` as there)."""
    torch = N.require_cuda()
    a, b, s, mean_shift = compute_pca(m1, m2, n_components, solver=solver)
    comp = torch.cat([a, b])
    x = torch.cat([torch.as_tensor(dense(m1), device='cuda', dtype=torch.float64),
                   torch.as_tensor(dense(m2), device='cuda', dtype=torch.float64)])
    cell_mean = (x - mean_shift[None, :]).mean(dim=1)
    pca = FittedPCA(comp.T.cpu().numpy(), s.cpu().numpy(), cell_mean.cpu().numpy())
    return a.cpu().numpy(), b.cpu().numpy(), pca, mean_shift.cpu().numpy()
