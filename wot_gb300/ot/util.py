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
    reference hands to scikit-learn. Products with T and T^T come from x's
    sparse form and two rank-one terms.

    On the GPU (x a CUDA tensor, as compute_pca makes it) everything runs in
    libwotg: the CSR of x and of its transpose (wotg_csr_count / _fill /
    _transpose, a stable transpose so that every product sums in the same
    order), the products with the rank-one centrings in their epilogue
    (wotg_spmm_centred), the small vector-matrix products (wotg_gemm_f64). For a
    CPU tensor the same operator is formed with torch's sparse products: that
    branch exists for the CPU test suite, which checks the algorithm against
    scikit-learn on a host without a GPU; compute_pca never takes it."""

    def __init__(self, x, mu, sparse=None):
        import torch
        self.x, self.mu = x, mu
        n, p = x.shape
        self.n, self.p = n, p
        self.device = x.is_cuda
        if self.device:
            self._build_device(x.contiguous(), mu.contiguous())
            return
        self.c = (x @ torch.ones(p, dtype=x.dtype, device=x.device)) / p - float(mu.sum()) / p
        if sparse is None:
            sparse = int(torch.count_nonzero(x)) < SPARSE_DENSITY * x.numel()
        self.xs = self.xts = None
        if sparse:
            with warnings.catch_warnings():         # torch marks sparse CSR as beta
                warnings.simplefilter('ignore', UserWarning)
                self.xs = x.to_sparse_csr()
                self.xts = x.T.contiguous().to_sparse_csr()

    def _build_device(self, x, mu):
        import ctypes
        import torch
        lib, st = N.load(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        n, p = self.n, self.p
        f64 = dict(dtype=torch.float64, device='cuda')
        rowptr = torch.empty(n + 1, dtype=torch.int64, device='cuda')
        rowsum = torch.empty(n, **f64)
        N.check(lib.wotg_csr_count(x.data_ptr(), n, p, x.stride(0), rowptr.data_ptr(), rowsum.data_ptr(), st),
                'wotg_csr_count')
        nnz = max(1, int(rowptr[n]))
        colidx = torch.empty(nnz, dtype=torch.int32, device='cuda')
        vals = torch.empty(nnz, **f64)
        N.check(lib.wotg_csr_fill(x.data_ptr(), n, p, x.stride(0), rowptr.data_ptr(), colidx.data_ptr(),
                                  vals.data_ptr(), st), 'wotg_csr_fill')
        t_rowptr = torch.empty(p + 1, dtype=torch.int64, device='cuda')
        t_colidx = torch.empty(nnz, dtype=torch.int32, device='cuda')
        t_vals = torch.empty(nnz, **f64)
        ws = torch.empty(lib.wotg_csr_transpose_workspace_bytes(n, p), dtype=torch.uint8, device='cuda')
        N.check(lib.wotg_csr_transpose(rowptr.data_ptr(), colidx.data_ptr(), vals.data_ptr(), n, p,
                                       t_rowptr.data_ptr(), t_colidx.data_ptr(), t_vals.data_ptr(), ws.data_ptr(),
                                       ws.numel(), st), 'wotg_csr_transpose')
        self.csr = (rowptr, colidx, vals)
        self.csr_t = (t_rowptr, t_colidx, t_vals)
        self.c = rowsum / p - float(mu.sum()) / p
        self.ones_n = torch.ones(n, **f64)
        self.ones_p = torch.ones(p, **f64)
        self.mu = mu

    def _mm(self, a, b):
        import torch
        if a is None:
            return None
        with warnings.catch_warnings():
            warnings.simplefilter('ignore', UserWarning)
            return torch.sparse.mm(a, b)

    def _spmm(self, csr, rows, Q, a, c, b):
        import ctypes
        import torch
        Y = torch.empty((rows, Q.shape[1]), dtype=torch.float64, device='cuda')
        N.check(N.load().wotg_spmm_centred(csr[0].data_ptr(), csr[1].data_ptr(), csr[2].data_ptr(), rows,
                                           Q.data_ptr(), Q.shape[1], a.data_ptr(), c.data_ptr(), b.data_ptr(),
                                           Y.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                'wotg_spmm_centred')
        return Y

    def t_mul(self, Q):
        """T @ Q, Q genes x r."""
        if self.device:
            Q = Q.contiguous()
            return self._spmm(self.csr, self.n, Q, vec_mat(self.mu, Q), self.c, vec_mat(self.ones_p, Q))
        xq = self._mm(self.xs, Q) if self.xs is not None else self.x @ Q
        return xq - (self.mu @ Q)[None, :] - self.c[:, None] * Q.sum(dim=0)[None, :]

    def tt_mul(self, Q):
        """T^T @ Q, Q cells x r."""
        if self.device:
            Q = Q.contiguous()
            return self._spmm(self.csr_t, self.p, Q, vec_mat(self.c, Q), self.mu, vec_mat(self.ones_n, Q))
        xq = self._mm(self.xts, Q) if self.xts is not None else self.x.T @ Q
        return xq - self.mu[:, None] * Q.sum(dim=0)[None, :] - (self.c @ Q)[None, :]


def mat_mul(A, B):
    """A @ B of FP64 CUDA tensors in libwotg's GEMM kernel (wotg_gemm_f64)."""
    import ctypes
    import torch
    A, B = A.contiguous(), B.contiguous()
    M, K = A.shape
    Nc = B.shape[1]
    out = torch.empty((M, Nc), dtype=torch.float64, device='cuda')
    N.check(N.load().wotg_gemm_f64(A.data_ptr(), K, B.data_ptr(), Nc, None, out.data_ptr(), Nc, M, Nc, K,
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), 'wotg_gemm_f64')
    return out


def vec_mat(w, Q):
    """w^T Q (a vector of Q's width) for FP64 CUDA tensors, in libwotg's
    vector-matrix kernel (fixed-order sums over Q's long dimension)."""
    import ctypes
    import torch
    w, Q = w.contiguous(), Q.contiguous()
    K, r = Q.shape
    lib = N.load()
    out = torch.empty(r, dtype=torch.float64, device='cuda')
    ws = torch.empty(lib.wotg_vecmat_workspace_bytes(K, r), dtype=torch.uint8, device='cuda')
    N.check(lib.wotg_vecmat_f64(w.data_ptr(), Q.data_ptr(), K, r, out.data_ptr(), ws.data_ptr(), ws.numel(),
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), 'wotg_vecmat_f64')
    return out


def _orthonormal(A):
    """An orthonormal basis of A's columns: Cholesky QR twice, A^T A and the
    product with R^-1 on the device (libwotg's Gram and GEMM kernels for CUDA
    tensors), the r x r factorisations on the host; Householder QR on the host
    when A's Gram matrix is not positive definite (rank-deficient iterates)."""
    import ctypes
    import torch
    for _ in range(2):
        if A.is_cuda:
            A = A.contiguous()
            n, r = A.shape
            lib = N.load()
            G = torch.empty((r, r), dtype=torch.float64, device='cuda')
            ws = torch.empty(lib.wotg_gram_workspace_bytes(n, r), dtype=torch.uint8, device='cuda')
            N.check(lib.wotg_gram_f64(A.data_ptr(), n, r, G.data_ptr(), ws.data_ptr(), ws.numel(),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), 'wotg_gram_f64')
            G = G.cpu().numpy()
        else:
            G = (A.T @ A).cpu().numpy()
        try:
            L = np.linalg.cholesky(G)
        except np.linalg.LinAlgError:
            q, _ = np.linalg.qr(A.cpu().numpy())
            return torch.as_tensor(q, device=A.device)
        Rinv = torch.as_tensor(np.linalg.inv(L.T), dtype=A.dtype, device=A.device)
        A = mat_mul(A, Rinv) if A.is_cuda else A @ Rinv
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
        U_k = torch.as_tensor(np.ascontiguousarray(Uh[:, :k]), dtype=x.dtype, device=x.device)
        comp = mat_mul(Q, U_k) if x.is_cuda else Q @ U_k                            # cells x k
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
