"""The local PCA's products on libwotg's own kernels (wot/ot/util.py:240-255 as
scikit-learn computes it): the CSR build and its stable transpose exactly, the
centred sparse products and the Gram kernel against FP64 NumPy, and the whole
device reference_pca against the reference's golden output and the oracle's
restatement (singular values to 1e-13 relative, components to 1e-12, as the
CPU tests hold the same routine on CPU tensors)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available()
    _build.build()
    _native.load()


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize('n,p', [(1, 1), (37, 53), (700, 200), (3000, 1000)])
def test_csr_build_transpose_spmm_gram(n, p):
    import torch
    from wot_gb300 import _native as N
    from wot_gb300.ot.util import _Centred, _orthonormal
    rng = np.random.default_rng(n + p)
    X = rng.random((n, p)) * (rng.random((n, p)) < 0.1)
    x = torch.as_tensor(X, device='cuda')
    mu = x.mean(dim=0)
    T = _Centred(x, mu)
    rowptr, colidx, vals = (t.cpu().numpy() for t in T.csr)
    nnz = int(np.count_nonzero(X))
    assert rowptr[-1] == nnz and np.array_equal(np.diff(rowptr), np.count_nonzero(X, axis=1))
    dense = np.zeros((n, p))
    for i in range(n):
        cols = colidx[rowptr[i]:rowptr[i + 1]]
        assert np.all(np.diff(cols) > 0)
        dense[i, cols] = vals[rowptr[i]:rowptr[i + 1]]
    assert np.array_equal(dense, X)
    t_rowptr, t_colidx, t_vals = (t.cpu().numpy() for t in T.csr_t)
    dense_t = np.zeros((p, n))
    for j in range(p):
        rows = t_colidx[t_rowptr[j]:t_rowptr[j + 1]]
        assert np.all(np.diff(rows) > 0)          # stable: rows in order within each column
        dense_t[j, rows] = t_vals[t_rowptr[j]:t_rowptr[j + 1]]
    assert np.array_equal(dense_t, X.T)
    # the centred products: T = x - 1 mu^T - c 1^T
    c = X.mean(axis=1) - X.mean(axis=0).sum() / p
    Tc = X - X.mean(axis=0)[None, :] - c[:, None]
    for r in (1, 40, 64):
        Q = rng.normal(size=(p, r))
        P = rng.normal(size=(n, r))
        np.testing.assert_allclose(T.t_mul(torch.as_tensor(Q, device='cuda')).cpu().numpy(), Tc @ Q,
                                   rtol=1e-12, atol=1e-12 * np.abs(Tc @ Q).max())
        np.testing.assert_allclose(T.tt_mul(torch.as_tensor(P, device='cuda')).cpu().numpy(), Tc.T @ P,
                                   rtol=1e-12, atol=1e-12 * np.abs(Tc.T @ P).max())
    if n >= 64:
        A = rng.normal(size=(n, 40))
        lib = N.load()
        G = torch.empty((40, 40), dtype=torch.float64, device='cuda')
        ws = torch.empty(lib.wotg_gram_workspace_bytes(n, 40), dtype=torch.uint8, device='cuda')
        At = torch.as_tensor(A, device='cuda')
        assert lib.wotg_gram_f64(At.data_ptr(), n, 40, G.data_ptr(), ws.data_ptr(), ws.numel(), _stream()) == 0
        np.testing.assert_allclose(G.cpu().numpy(), A.T @ A, rtol=0, atol=1e-12 * np.abs(A.T @ A).max())
        Qo = _orthonormal(At).cpu().numpy()
        np.testing.assert_allclose(Qo.T @ Qo, np.eye(40), atol=1e-12)


def test_device_reference_pca_equals_the_reference(pair_golden):
    """reference_pca on the GPU (libwotg's CSR, centred products, Gram and
    GEMM kernels) equals the reference's golden PCA, and the oracle's
    restatement on scikit-learn's other (transposed) randomized branch."""
    import torch
    from oracle import ot_model as oom
    from wot_gb300 import synthetic
    from wot_gb300.ot.util import reference_pca
    z = pair_golden
    X, day = z['X'], z['day']
    x = torch.as_tensor(np.vstack([X[day == 0], X[day == 1]]), device='cuda', dtype=torch.float64)
    comp, s, solver = reference_pca(x, x.mean(dim=0), 30)
    assert solver == 'randomized'
    np.testing.assert_allclose(s.cpu().numpy(), z['singular_values'], rtol=1e-13, atol=0)
    np.testing.assert_allclose(comp.cpu().numpy(), np.vstack([z['pca_components_0'], z['pca_components_1']]),
                               rtol=0, atol=1e-12)
    Xb, dayb, _ = synthetic.time_course([1300, 1500], n_genes=1000, n_clusters=6, seed=4)
    a, b, s_ref, _, _ = oom.compute_pca_reference(Xb[dayb == 0], Xb[dayb == 1], 30)
    x = torch.as_tensor(Xb, device='cuda', dtype=torch.float64)
    comp, s, _ = reference_pca(x, x.mean(dim=0), 30)
    np.testing.assert_allclose(s.cpu().numpy(), s_ref, rtol=1e-13, atol=0)
    np.testing.assert_allclose(comp.cpu().numpy(), np.vstack([a, b]), rtol=0, atol=1e-12)
