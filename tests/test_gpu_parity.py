"""Parity of the CUDA path (through the C ABI) with the reference's FP64 outputs.

Tolerances (tests/parity.py, from the project's parity target):
  COUPLING_TOL  max|T - T_ref| / max|T_ref|                               <= 1e-4
  ELEMENT_TOL   max |T_ij - R_ij| / |R_ij| over |R_ij| >= 1e-6 max|R|     <= 1e-4
  MARGINAL_TOL  max_i |r_i - r_ref_i| / max_i r_ref_i (rows and columns) <= 1e-6
The golden couplings come from the reference's own solver module
(tests/golden/make_golden.py); larger cases are checked against the oracle.
"""
import ast
import logging

import numpy as np
import pytest

from parity import COUPLING_TOL, assert_parity, coupling_err

pytestmark = pytest.mark.gpu

DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)
CASES = ['dg_default', 'dg_growth3', 'dg_eps01_lam10', 'dg_eps1_lam01', 'dg_tau10', 'dg_maxiter',
         'dg_batch3_tol1e6', 'fi_short', 'fi_tau10', 'fi_growth2']


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available(), 'GPU tests need a CUDA device'
    _build.build()
    _native.load()


def quiet(fn, *a, **k):
    logging.disable(logging.WARNING)
    try:
        return fn(*a, **k)
    finally:
        logging.disable(logging.NOTSET)


def test_kat_identity(kat_golden):
    """The reference's known-answer test (tests/test_transport.py:11-33) through the drop-in solvers."""
    from wot_gb300 import ot
    C, G = kat_golden['C'], kat_golden['G']
    for tag, solver in (('dg', ot.optimal_transport_duality_gap), ('fi', ot.transport_stablev2)):
        cfg = dict(DEFAULTS, epsilon=0.01, lambda1=1, lambda2=50)
        tmap, learned = ot.compute_transport_matrix(solver=solver, C=C, G=G.copy(), **cfg)
        assert np.allclose(tmap, np.eye(3), atol=0.01, rtol=0)
        assert_parity(tmap, kat_golden['tmap_' + tag], what=tag)


@pytest.mark.parametrize('name', CASES)
def test_solver_vs_reference_golden(pair_golden, name):
    from wot_gb300 import ot
    z = pair_golden
    params = ast.literal_eval(str(z['params_' + name]))
    cfg = dict(DEFAULTS)
    cfg.update(params)
    solver = ot.transport_stablev2 if name.startswith('fi') else ot.optimal_transport_duality_gap
    tmap, learned = quiet(ot.compute_transport_matrix, solver=solver, C=z['C'], G=z['G'].copy(), **cfg)
    ref = z['tmap_' + name]
    assert tmap.shape == ref.shape and tmap.dtype == np.float64
    assert_parity(tmap, ref, what=name)
    lg = np.array(learned)
    assert lg.shape == z['learned_' + name].shape
    np.testing.assert_allclose(lg, z['learned_' + name], rtol=20 * COUPLING_TOL)


def test_iteration_counts_match_oracle(pair_golden):
    """Same stopping decisions as the FP64 reference on the golden pair."""
    from oracle import optimal_transport as oot
    from wot_gb300.ot import device as D
    z = pair_golden
    for params in ({}, {'epsilon': 0.1, 'lambda1': 0.1}, {'tau': 10.0}):
        cfg = dict(DEFAULTS, **params)
        st = {}
        oot.optimal_transport_duality_gap(C=z['C'], G=z['G'], stats=st, **cfg)
        res = D.solve(D.cost_from_dense(z['C']), z['G'], cfg, 0)
        assert res.stats['iterations'] == st['iterations'], (params, res.stats, st)
        assert res.stats['absorptions'] == st['absorptions']
        assert res.stats['gap'] == pytest.approx(st['gap'], rel=1e-2)


def test_max_iter_warns_and_skips_division(pair_golden, caplog):
    from wot_gb300 import ot
    z = pair_golden
    cfg = dict(DEFAULTS, max_iter=37)
    with caplog.at_level(logging.WARNING, logger='wot'):
        t = ot.optimal_transport_duality_gap(C=z['C'], G=z['G'], **cfg)
    assert 'Reached max_iter' in caplog.text
    assert_parity(t, z['tmap_dg_maxiter'])


def test_zero_growth_raises_like_reference(pair_golden):
    from wot_gb300 import ot
    z = pair_golden
    G = z['G'].copy()
    G[3] = 0.0
    with pytest.raises(RuntimeError, match='Overflow encountered'):
        ot.optimal_transport_duality_gap(z['C'], G, 1, 50, 0.05, 5, 1e-8, 1e4, 1, 1e7)


@pytest.mark.parametrize('shape', [(1, 1), (1, 7), (9, 1), (37, 53), (64, 130), (203, 97)])
def test_edge_shapes_vs_oracle(shape):
    from oracle import optimal_transport as oot
    from wot_gb300 import ot
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    x = rng.normal(size=(shape[0], 5))
    y = rng.normal(size=(shape[1], 5)) + 0.3
    C = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    C = C / np.median(C)
    G = rng.lognormal(0, 0.3, size=shape[0])
    for solver, osolver, extra in ((ot.optimal_transport_duality_gap, oot.optimal_transport_duality_gap, {}),
                                   (ot.transport_stablev2, oot.transport_stablev2,
                                    dict(scaling_iter=250, extra_iter=50))):
        cfg = dict(DEFAULTS, **extra)
        ref, _ = oot.compute_transport_matrix(solver=osolver, C=C, G=G.copy(), **cfg)
        got, _ = ot.compute_transport_matrix(solver=solver, C=C, G=G.copy(), **cfg)
        assert_parity(got, ref, what=(shape, solver.__name__))


def test_cost_kernel_and_median():
    from oracle import ot_model as oom
    from wot_gb300.ot import device as D
    rng = np.random.default_rng(7)
    for (I, J, d) in ((37, 53, 30), (300, 257, 50), (129, 64, 3), (1, 1, 30)):
        x = rng.normal(size=(I, d)).astype(np.float32)
        y = rng.normal(size=(J, d)).astype(np.float32)
        c = D.cost_from_points(x, y)
        C = c.C.cpu().numpy()
        ref = oom.sqeuclidean(x.astype(np.float64), y.astype(np.float64))
        assert np.abs(C[:, :J] - ref).max() <= 1e-5 * ref.max()
        assert np.all(np.isinf(C[:, J:]))
        assert D.median(c) == np.median(C[:, :J].astype(np.float64))


def test_median_ties_and_parity():
    from wot_gb300.ot import device as D
    rng = np.random.default_rng(3)
    for (I, J) in ((1, 2), (2, 3), (5, 7), (64, 64), (101, 99)):
        C = rng.integers(0, 5, size=(I, J)).astype(np.float64) * 0.25
        c = D.cost_from_dense(C)
        assert D.median(c) == np.median(C)


def test_c0_shape_from_points_vs_oracle():
    """The plain method at the small configuration's shape (2000 x 2500 cells,
    30-d local PCA): device cost + median + duality-gap solve vs the oracle on
    the same coordinates."""
    from oracle import ot_model as oom, optimal_transport as oot
    from wot_gb300 import synthetic
    from wot_gb300.ot import device as D
    X, day, growth = synthetic.time_course([2000, 2500], n_genes=1000, n_clusters=6, seed=0)
    x0, x1, s, _ = oom.compute_pca(X[day == 0], X[day == 1], 30)
    a, b = x0 * s, x1 * s
    C = oom.compute_default_cost_matrix(a, b)
    G = growth[day == 0]
    st = {}
    ref = oot.optimal_transport_duality_gap(C=C, G=G, stats=st, **DEFAULTS)
    cost = D.default_cost(a.astype(np.float32), b.astype(np.float32))
    res = D.solve(cost, G, DEFAULTS, 0)
    T = res.tmap.cpu().numpy()
    assert_parity(T, ref)
    assert abs(res.stats['iterations'] - st['iterations']) <= 5


def test_otmodel_end_to_end(pair_golden):
    """The default OTModel (device PCA as the reference computes it, device cost
    and solve) from the raw expression matrix: with growth_iters=1 against the
    reference's own map of the golden pair, and with growth_iters=2 against the
    oracle's restatement of compute_single_transport_map (the reference's PCA,
    its g0..g2 columns)."""
    from oracle import ot_model as oom
    import wot_gb300 as wot
    z = pair_golden
    X, day, growth = z['X'], z['day'], z['growth']
    ids = np.array(['c%d' % i for i in range(len(day))])
    ds = wot.Dataset(X, wot.Frame({'day': day, 'cell_growth_rate': growth}, index=ids))
    tm1 = wot.OTModel(ds).compute_transport_map(0, 1)
    assert_parity(tm1.X, z['tmap_dg_default'], what='default OTModel vs the reference')
    model = wot.OTModel(ds, growth_iters=2)
    tm = model.compute_transport_map(0, 1)
    ref, obs = oom.compute_single_transport_map(X, day, 0.0, 1.0, growth=growth, growth_iters=2, pca='reference')
    assert_parity(tm.X, ref, what='growth_iters=2 vs the oracle')
    assert list(tm.obs.index) == list(ids[day == 0]) and list(tm.var.index) == list(ids[day == 1])
    for k in ('g0', 'g1', 'g2'):
        np.testing.assert_allclose(tm.obs[k], obs[k], rtol=1e-5)


def test_compute_all_transport_maps_roundtrip(tmp_path):
    """tests/test_transport.py:36-64: three days, custom costs, maps written and read back."""
    import wot_gb300 as wot
    rng = np.random.default_rng(0)
    ds = wot.Dataset(rng.random((9, 1000)), wot.Frame({'day': [1, 1, 1, 2, 2, 2, 3, 3, 3]}))
    C = np.array([[0, 100, 100], [100, 0, 100], [100, 100, 0]], dtype=np.float64)
    model = wot.OTModel(ds, epsilon=0.01, lambda1=1, lambda2=50)
    model.compute_all_transport_maps(tmap_out=str(tmp_path / 'tmap'), cost_matrices=[C, C])
    tmm = wot.TransportMapModel.from_directory(str(tmp_path / 'tmap'))
    for pair in ((1.0, 2.0), (2.0, 3.0)):
        assert np.allclose(tmm.get_coupling(*pair).X, np.eye(3), atol=0.01, rtol=0)


def _chain_model(z):
    import wot_gb300 as wot
    names = ['t0_t1', 't1_t2', 't2_t3', 't3_t4']
    tmaps, ids, days = {}, [], []
    for k, n in enumerate(names):
        tmaps[(float(k), float(k + 1))] = wot.Dataset(z[n + '_X'], wot.Frame(index=z[n + '_obs']),
                                                      wot.Frame(index=z[n + '_var']))
        ids += list(z[n + '_obs'])
        days += [float(k)] * len(z[n + '_obs'])
    ids += list(z['t3_t4_var'])
    days += [4.0] * len(z['t3_t4_var'])
    meta = wot.Frame({'day': np.array(days)}, index=np.array(ids))
    return wot.TransportMapModel(tmaps, meta), {k: v.X for k, v in tmaps.items()}


def test_transport_map_model_on_integer_maps(chain_golden):
    from oracle import tmap as otm
    from wot_gb300 import Population
    model, raw = _chain_model(chain_golden)
    tp = [0.0, 1.0, 2.0, 3.0, 4.0]
    P = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 1.0]])
    pops = [Population(4.0, P[0], 'a'), Population(4.0, P[1], 'b')]
    back = model.pull_back(*pops, to_time=0.0, normalize=False, as_list=True)
    np.testing.assert_allclose(np.array([p.p for p in back]), otm.pull_back(raw, tp, P, 4.0, 0.0, normalize=False),
                               rtol=1e-13)
    back_n = model.ancestors(*pops, at_time=1.0, as_list=True)
    np.testing.assert_allclose(np.array([p.p for p in back_n]), otm.pull_back(raw, tp, P, 4.0, 1.0), rtol=1e-13)
    start = Population(0.0, np.ones(4), 's')
    fwd = model.descendants(start, at_time=3.0)
    np.testing.assert_allclose(fwd.p, otm.push_forward(raw, tp, np.ones((1, 4)), 0.0, 3.0)[0], rtol=1e-13)
    f = model.fates(pops)
    np.testing.assert_allclose(f.X, otm.fates(raw, tp, P, 4.0), rtol=1e-12)
    tr = model.trajectories([Population(2.0, np.array([0, 1, 0, 0, 1.0]), 'm')])
    np.testing.assert_allclose(tr.X, otm.trajectories(raw, tp, np.array([[0, 1, 0, 0, 1.0]]), 2.0), rtol=1e-12)
    tt = model.transition_table([Population(1.0, np.array([1.0, 0.0]), 'x')], pops)
    np.testing.assert_allclose(tt.X, otm.transition_table(raw, tp, np.array([[1.0, 0.0]]), 1.0, P, 4.0),
                               rtol=1e-12)
    chained = model.get_coupling(0.0, 2.0)
    np.testing.assert_allclose(chained.X, raw[(0., 1.)] @ raw[(1., 2.)], rtol=1e-13)


def test_lse_matvec_primitive():
    """wotg_lse_matvec against an FP64 log-sum-exp of the same FP32 operands."""
    import ctypes
    import torch
    from wot_gb300 import _native as N
    from wot_gb300.ot import device as D
    rng = np.random.default_rng(11)
    I, J = 77, 131
    C = rng.random((I, J)) * 3
    c = D.cost_from_dense(C)
    C32 = c.C.cpu().numpy()[:, :J].astype(np.float64)
    lib = N.load()
    k2 = np.float32(7.5)
    for axis, n in ((0, c.ldc), (1, I)):
        w = rng.normal(size=n).astype(np.float32)
        if axis == 0:
            w[J:] = 0
        wt = torch.as_tensor(w, device='cuda')
        L = torch.empty(I if axis == 0 else J, dtype=torch.float64, device='cuda')
        ws = torch.empty(lib.wotg_lse_matvec_workspace_bytes(I, J, c.ldc), dtype=torch.uint8, device='cuda')
        st = lib.wotg_lse_matvec(c.C.data_ptr(), I, J, c.ldc, wt.data_ptr(), ctypes.c_float(k2), axis,
                                 L.data_ptr(), ws.data_ptr(), ws.numel(),
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0
        x = (w[:J][None, :] if axis == 0 else w[:, None]).astype(np.float64) - float(k2) * C32
        x = x if axis == 0 else x.T
        m = x.max(axis=1)
        ref = (m + np.log2(np.exp2(x - m[:, None]).sum(axis=1))) * np.log(2.0)
        np.testing.assert_allclose(L.cpu().numpy(), ref, rtol=0, atol=2e-5)


def test_otmodel_reference_pca_reproduces_the_reference_map(pair_golden):
    """OTModel(pca='reference').compute_transport_map from the raw expression
    matrix (device PCA as scikit-learn computes it, device cost and solve)
    against the reference's own map of the golden pair (made by the reference's
    code from the same matrix), within the three parity bounds; the exact PCA
    is the alternative."""
    import wot_gb300 as wot
    z = pair_golden
    X, day, growth = z['X'], z['day'], z['growth']
    ids = np.array(['c%d' % i for i in range(len(day))])
    ds = wot.Dataset(X, wot.Frame({'day': day, 'cell_growth_rate': growth}, index=ids))
    tm = wot.OTModel(ds, pca='reference').compute_transport_map(0, 1)
    assert_parity(tm.X, z['tmap_dg_default'])
    exact = wot.OTModel(ds, pca='exact').compute_transport_map(0, 1)
    assert exact.X.shape == tm.X.shape and coupling_err(exact.X, tm.X) < 1.0
