"""The local PCA as the reference computes it (wot/ot/util.py:240-255:
scikit-learn PCA(30, random_state=58951) on the double-centred genes x cells
matrix), on the CPU:
  * the oracle's restatement (oracle/ot_model.py::compute_pca_reference) equals
    the reference's own output stored in tests/golden/pair_120x150.npz, and
    scikit-learn itself where it is installed (both of its randomized branches:
    fewer and more cells than genes);
  * the product's device-agnostic routine (wot_gb300.ot.util.reference_pca,
    run here on CPU tensors, dense and sparse products) equals both to FP64
    rounding: singular values to 1e-13 relative, components to 1e-12.
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def golden():
    return np.load(os.path.join(ROOT, 'tests', 'golden', 'pair_120x150.npz'))


def _days(z):
    X, day = z['X'], z['day']
    return X[day == 0], X[day == 1]


def test_oracle_reference_pca_matches_the_reference(golden):
    from oracle import ot_model as oom
    m0, m1 = _days(golden)
    a, b, s, _, solver = oom.compute_pca_reference(m0, m1, 30)
    assert solver == 'randomized'
    np.testing.assert_allclose(s, golden['singular_values'], rtol=1e-13, atol=0)
    np.testing.assert_allclose(a, golden['pca_components_0'], rtol=0, atol=1e-12)
    np.testing.assert_allclose(b, golden['pca_components_1'], rtol=0, atol=1e-12)


@pytest.mark.parametrize('cells', [(120, 150), (1300, 1500)])
def test_oracle_reference_pca_matches_sklearn(cells):
    skd = pytest.importorskip('sklearn.decomposition')
    from oracle import ot_model as oom
    from wot_gb300 import synthetic
    X, day, _ = synthetic.time_course(list(cells), n_genes=1000, n_clusters=6, seed=4)
    x = X - X.mean(axis=0)
    pca = skd.PCA(n_components=30, random_state=58951).fit(x.T)
    a, b, s, _, solver = oom.compute_pca_reference(X[day == 0], X[day == 1], 30)
    assert solver == pca._fit_svd_solver == 'randomized'
    np.testing.assert_allclose(s, pca.singular_values_, rtol=1e-13, atol=0)
    np.testing.assert_allclose(np.vstack([a, b]), pca.components_.T, rtol=0, atol=1e-12)


@pytest.mark.parametrize('sparse', [False, True])
def test_product_reference_pca(golden, sparse):
    import torch
    from oracle import ot_model as oom
    from wot_gb300 import synthetic
    from wot_gb300.ot.util import reference_pca
    m0, m1 = _days(golden)
    x = torch.tensor(np.vstack([m0, m1]))
    comp, s, solver = reference_pca(x, x.mean(dim=0), 30, sparse=sparse)
    assert solver == 'randomized'
    np.testing.assert_allclose(s.numpy(), golden['singular_values'], rtol=1e-13, atol=0)
    np.testing.assert_allclose(comp.numpy(), np.vstack([golden['pca_components_0'], golden['pca_components_1']]),
                               rtol=0, atol=1e-12)
    # more cells than genes: scikit-learn's transposed branch
    X, day, _ = synthetic.time_course([1300, 1500], n_genes=1000, n_clusters=6, seed=4)
    a, b, s_ref, _, _ = oom.compute_pca_reference(X[day == 0], X[day == 1], 30)
    x = torch.tensor(X)
    comp, s, solver = reference_pca(x, x.mean(dim=0), 30, sparse=sparse)
    np.testing.assert_allclose(s.numpy(), s_ref, rtol=1e-13, atol=0)
    np.testing.assert_allclose(comp.numpy(), np.vstack([a, b]), rtol=0, atol=1e-12)


def test_solver_choice_follows_sklearn():
    from wot_gb300.ot.util import sklearn_pca_solver
    assert sklearn_pca_solver(1000, 270, 30) == 'randomized'
    assert sklearn_pca_solver(1000, 45000, 30) == 'randomized'
    assert sklearn_pca_solver(1000, 80, 30) == 'covariance_eigh'
    assert sklearn_pca_solver(400, 450, 30) == 'full'
    assert sklearn_pca_solver(1000, 30, 30) == 'covariance_eigh'
    assert sklearn_pca_solver(1000, 600, 500) == 'full'


def test_oracle_pipeline_with_the_reference_pca(golden):
    """The oracle's compute_single_transport_map with the reference's PCA
    reproduces the reference's own cost on the golden pair (median-normalised,
    built from its PCA coordinates), i.e. the whole front of the path."""
    from oracle import ot_model as oom
    m0, m1 = _days(golden)
    a, b, s, _, _ = oom.compute_pca_reference(m0, m1, 30)
    C = oom.compute_default_cost_matrix(a, b, np.diag(s))
    np.testing.assert_allclose(C, golden['C'], rtol=0, atol=1e-10)


def test_oracle_pipeline_reproduces_the_reference_map(golden):
    """From the raw expression matrix: the oracle's compute_single_transport_map
    with the reference's PCA gives the reference's own transport map
    (tmap_dg_default of the golden pair, made by the reference's code) to 1e-12."""
    from oracle import ot_model as oom
    tm, _ = oom.compute_single_transport_map(golden['X'], golden['day'], 0.0, 1.0, growth=golden['growth'],
                                             pca='reference')
    ref = golden['tmap_dg_default']
    assert np.abs(tm - ref).max() <= 1e-12 * np.abs(ref).max()
