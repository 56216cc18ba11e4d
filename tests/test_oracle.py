"""The oracle (FP64 NumPy restatement) pinned against the reference's own
known-answer test, golden vectors produced by the reference's solver module,
and the reference's integer transport-map fixtures. CPU only."""
import ast
import logging

import numpy as np
import pytest

from oracle import optimal_transport as oot
from oracle import ot_model as oom
from oracle import tmap as otm

DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)
CASES = ['dg_default', 'dg_growth3', 'dg_eps01_lam10', 'dg_eps1_lam01', 'dg_tau10', 'dg_maxiter',
         'dg_batch3_tol1e6', 'fi_short', 'fi_tau10', 'fi_growth2']


def solver_of(name):
    return oot.transport_stablev2 if name.startswith('fi') else oot.optimal_transport_duality_gap


def test_kat_identity(kat_golden):
    """tests/test_transport.py:11-33: custom 3x3 cost, epsilon=0.01 -> identity within 0.01."""
    C, G = kat_golden['C'], kat_golden['G']
    for tag, solver in (('dg', oot.optimal_transport_duality_gap), ('fi', oot.transport_stablev2)):
        cfg = dict(DEFAULTS, epsilon=0.01, lambda1=1, lambda2=50)
        tmap, _ = oot.compute_transport_matrix(solver=solver, C=C, G=G.copy(), **cfg)
        assert np.allclose(tmap, np.eye(3), atol=0.01, rtol=0)
        np.testing.assert_allclose(tmap, kat_golden['tmap_' + tag], rtol=1e-12, atol=0)


@pytest.mark.parametrize('name', CASES)
def test_solver_matches_reference(pair_golden, name):
    z = pair_golden
    params = ast.literal_eval(str(z['params_' + name]))
    cfg = dict(DEFAULTS)
    cfg.update(params)
    logging.disable(logging.WARNING)
    try:
        tmap, learned = oot.compute_transport_matrix(solver=solver_of(name), C=z['C'], G=z['G'].copy(), **cfg)
    finally:
        logging.disable(logging.NOTSET)
    ref = z['tmap_' + name]
    assert tmap.shape == ref.shape
    assert np.abs(tmap - ref).max() <= 1e-12 * np.abs(ref).max()
    np.testing.assert_allclose(np.array(learned), z['learned_' + name], rtol=1e-12, atol=0)


def test_cost_matches_reference(pair_golden):
    z = pair_golden
    C = oom.compute_default_cost_matrix(z['pca_components_0'], z['pca_components_1'], np.diag(z['singular_values']))
    np.testing.assert_allclose(C, z['C'], rtol=1e-10, atol=1e-12)
    D = oom.sqeuclidean(z['x0'], z['x1'])
    assert np.median(D) == pytest.approx(float(z['median']), rel=1e-12)


def test_exact_pca_spans_reference_subspace(pair_golden):
    """The reference's randomized PCA and the exact SVD agree on the leading
    singular value to a few percent (they are different solvers)."""
    z = pair_golden
    X, day = z['X'], z['day']
    _, _, s, _ = oom.compute_pca(X[day == 0], X[day == 1], 30)
    assert s[0] == pytest.approx(z['singular_values'][0], rel=0.05)
    assert np.all(np.diff(s) <= 1e-9)


def test_max_iter_quirk(pair_golden):
    """On max_iter the reference returns the coupling without the final / J."""
    z = pair_golden
    cfg = dict(DEFAULTS, max_iter=37)
    st = {}
    logging.disable(logging.WARNING)
    try:
        t = oot.optimal_transport_duality_gap(C=z['C'], G=z['G'], stats=st, **cfg)
    finally:
        logging.disable(logging.NOTSET)
    assert st['max_iter'] and st['iterations'] == 37
    assert t.sum() > z['C'].shape[1] * 0.5 * z['tmap_dg_default'].sum()


def test_zero_growth_raises(pair_golden):
    """A zero source mass makes the duality gap NaN -> RuntimeError (optimal_transport.py:162-163)."""
    z = pair_golden
    G = z['G'].copy()
    G[3] = 0.0
    with np.errstate(all='ignore'), pytest.raises(RuntimeError, match='Overflow encountered'):
        oot.optimal_transport_duality_gap(C=z['C'], G=G, **DEFAULTS)


def _chain(z):
    names = ['t0_t1', 't1_t2', 't2_t3', 't3_t4']
    tmaps = {(float(k), float(k + 1)): z[n + '_X'] for k, n in enumerate(names)}
    return tmaps, [0.0, 1.0, 2.0, 3.0, 4.0]


def test_tmap_restatement_on_integer_maps(chain_golden):
    tmaps, tp = _chain(chain_golden)
    P = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 1.0]])     # 2 populations over the 3 cells of day 4
    back = otm.pull_back(tmaps, tp, P, 4.0, 0.0, normalize=False)
    expect = (tmaps[(0., 1.)] @ tmaps[(1., 2.)] @ tmaps[(2., 3.)] @ tmaps[(3., 4.)] @ P.T).T
    np.testing.assert_array_equal(back, expect)          # integers: exact in FP64
    fwd = otm.push_forward(tmaps, tp, np.ones((1, 4)), 0.0, 2.0, normalize=False)
    np.testing.assert_array_equal(fwd, np.ones((1, 4)) @ tmaps[(0., 1.)] @ tmaps[(1., 2.)])
    np.testing.assert_array_equal(otm.chain(tmaps, [(0., 1.), (1., 2.)]), tmaps[(0., 1.)] @ tmaps[(1., 2.)])
    f = otm.fates(tmaps, tp, P, 4.0)
    assert f.shape == (4 + 2 + 5 + 6 + 3, 2)             # no 'Other': P covers every cell
    np.testing.assert_allclose(f.sum(axis=1), 1.0)


def test_adjoint_reference_fixed_point_and_gradient():
    """oracle/adjoint.py: its fixed-epsilon potential iteration converges to the
    coupling of the reference's solver (numpy oracle at tolerance 1e-12), and
    autograd through unrolled iterations from the optimum equals central finite
    differences of the converged objective."""
    torch = pytest.importorskip('torch')
    from oracle import adjoint as A, optimal_transport as oot
    rng = np.random.default_rng(0)
    I, J, d = 40, 50, 3
    x = torch.tensor(rng.normal(size=(I, d)))
    y = torch.tensor(rng.normal(size=(J, d)))
    logg = torch.tensor(rng.normal(0.0, 0.3, I))
    scale = 1.0 / float(np.median(A.cost(x, y, 1.0).numpy()))
    eps, l1, l2 = 0.1, 1.0, 50.0
    D, ub, vb = A.objective(x, y, logg, eps, l1, l2, scale)
    C = A.cost(x, y, scale).numpy()
    R = oot.optimal_transport_duality_gap(C=C, G=np.exp(logg.numpy()), lambda1=l1, lambda2=l2, epsilon=eps,
                                          batch_size=5, tolerance=1e-12, tau=1e4, epsilon0=1, max_iter=1e7)
    T = np.exp((ub.numpy()[:, None] + vb.numpy()[None, :] - C) / eps) / J
    assert np.abs(T - R).max() <= 1e-6 * np.abs(R).max()
    D2, gx, gy, gl = A.unrolled_gradient(x, y, logg, eps, l1, l2, scale, ub, vb, n_unroll=30)
    assert abs(D2 - D) <= 1e-10 * abs(D)
    coords = [('x', (3, 1)), ('x', (17, 0)), ('y', (7, 2)), ('y', (41, 1)), ('logg', (5,)), ('logg', (30,))]
    fd = A.fd_gradient(x, y, logg, eps, l1, l2, scale, coords, ub, vb, h=1e-5)
    ad = [float({'x': gx, 'y': gy, 'logg': gl}[n][i]) for n, i in coords]
    gmax = max(float(gx.abs().max()), float(gy.abs().max()), float(gl.abs().max()))
    assert max(abs(a - f) for a, f in zip(ad, fd)) <= 1e-6 * gmax


def test_torch_fp64_restatement_matches_numpy_oracle(pair_golden):
    """oracle.torch_ot (the same FP64 reference arithmetic on torch tensors, the
    checker for full-size problems on the GPU) equals the NumPy oracle, which is
    pinned to the reference's golden outputs: couplings, iteration and
    absorption counts, growth iterations, the median-normalised cost."""
    import ast
    import torch
    from oracle import ot_model as oom, optimal_transport as oot, torch_ot as tot
    z = pair_golden
    defaults = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, tolerance=1e-8,
                    max_iter=1e7, batch_size=5)
    for name in ('dg_default', 'dg_growth3', 'dg_eps01_lam10', 'dg_tau10', 'dg_maxiter'):
        cfg = dict(defaults, **ast.literal_eval(str(z['params_' + name])))
        st_n, st_t = {}, {}
        ref, lg_n = oot.compute_transport_matrix(solver=lambda **k: oot.optimal_transport_duality_gap(stats=st_n, **k),
                                                 C=z['C'], G=z['G'].copy(), **cfg)
        got, lg_t = tot.compute_transport_matrix(solver=lambda **k: tot.optimal_transport_duality_gap(stats=st_t, **k),
                                                 C=torch.as_tensor(z['C']), G=torch.as_tensor(z['G']), **cfg)
        assert np.abs(got.numpy() - ref).max() <= 1e-10 * np.abs(ref).max(), name
        assert st_t['iterations'] == st_n['iterations'] and st_t['absorptions'] == st_n['absorptions'], name
        assert np.allclose(np.array([x.numpy() for x in lg_t]), np.array(lg_n), rtol=1e-10, atol=0)
    rng = np.random.default_rng(2)
    a, b = rng.normal(size=(41, 7)), rng.normal(size=(58, 7))
    for (x, y) in ((a, b), (a[:40], b)):   # odd and even entry counts of the median
        np.testing.assert_allclose(tot.default_cost(torch.as_tensor(x), torch.as_tensor(y)).numpy(),
                                   oom.compute_default_cost_matrix(x, y), rtol=1e-13, atol=1e-13)
    v = torch.as_tensor(rng.normal(size=200001))            # the blockwise selection of large tensors
    for k in (1, 100000, 100001, 200001):
        assert tot.kth_smallest(v, k, block=1 << 12) == float(torch.kthvalue(v, k).values)
