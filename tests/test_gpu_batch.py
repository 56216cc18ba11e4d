"""Batched solves (wotg_solve_batched): every item against the single-problem
driver on the same device cost (iteration counts within a batch or two,
couplings to 1e-5) and against the oracle's FP64 solve (the parity bounds of
tests/parity.py: couplings to 1e-4 normalised and elementwise, marginals to
the batched pass's BATCHED_MARGINAL_TOL); the multi-RHS half-step against an
FP64 log-sum-exp; the implicit map's pull-back / push-forward against dense
products.
"""
import ctypes
import logging

import numpy as np
import pytest

from parity import assert_parity_batched, coupling_err

pytestmark = pytest.mark.gpu

SAME_DEVICE_TOL = 1e-5
DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available()
    _build.build()
    _native.load()


def _pair(I, J, seed, d=30):
    from wot_gb300 import synthetic
    from wot_gb300.ot import batch as Bt, device as D
    x = synthetic.gaussian_mixture_points(I, d=d, seed=seed)
    y = synthetic.gaussian_mixture_points(J, d=d, seed=seed + 100)
    g = np.random.default_rng(seed).lognormal(0, 0.3, I)
    cost = D.default_cost(x, y)
    return Bt.prepare_pair(cost, g), x, y, g


def test_transpose_cost():
    import torch
    from wot_gb300.ot import device as D
    rng = np.random.default_rng(0)
    for I, J in [(1, 1), (37, 53), (130, 257)]:
        x = rng.normal(size=(I, 5)).astype(np.float32)
        y = rng.normal(size=(J, 5)).astype(np.float32)
        c = D.cost_from_points(x, y)
        CT = D.transpose_cost(c).cpu().numpy()
        C = c.C.cpu().numpy()
        assert CT.shape[1] % 4 == 0
        assert np.array_equal(CT[:, :I], C[:, :J].T)
        assert np.all(np.isinf(CT[:, I:]))


def test_lse_multi_vs_fp64():
    """Several weight rows in one pass (more rows than one register group),
    ragged J, -inf weights, per-row kappa."""
    import torch
    from wot_gb300.ot import device as D
    rng = np.random.default_rng(1)
    I, J, K = 300, 517, 11
    x = rng.normal(size=(I, 8)).astype(np.float32)
    y = rng.normal(size=(J, 8)).astype(np.float32)
    c = D.cost_from_points(x, y)
    ldw = (J + 3) // 4 * 4
    W = rng.normal(scale=30.0, size=(K, ldw)).astype(np.float32)
    W[:, J:] = 0
    W[3, ::7] = -np.inf
    W[5, :] = -np.inf
    W[5, 11] = 2.0
    k2 = rng.uniform(0.5, 40.0, size=K).astype(np.float32)
    L = D.lse_multi(c.C, I, J, c.ldc, torch.as_tensor(W, device='cuda'), k2).cpu().numpy()
    C = c.C.cpu().numpy()[:, :J].astype(np.float64)
    for k in range(K):
        t = W[k, :J].astype(np.float64)[None, :] - float(k2[k]) * C
        m = t.max(axis=1, keepdims=True)
        ref = (m[:, 0] + np.log2(np.exp2(t - m).sum(axis=1))) * np.log(2.0)
        assert np.abs(L[k] - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())


def _solve_single(bp, g, cfg):
    from wot_gb300.ot import device as D
    logging.disable(logging.WARNING)
    try:
        return D.solve(bp.cost, g, cfg, 0, want_tmap=True, want_potentials=True)
    finally:
        logging.disable(logging.NOTSET)


def test_batched_matches_single_driver():
    """A small sweep plus items that take every branch: growth iterations,
    batch size 3, frequent absorptions, max_iter, a tall and a wide pair."""
    from wot_gb300 import _native as N
    from wot_gb300.ot import batch as Bt
    p0 = _pair(300, 420, 1)
    p1 = _pair(650, 380, 2)
    p2 = _pair(128, 1000, 3)
    pairs = [p0[0], p1[0], p2[0]]
    items = []
    for e in (0.05, 0.1):
        for l1 in (1.0, 3.0):
            items.append((0, dict(DEFAULTS, epsilon=e, lambda1=l1)))
    items.append((1, dict(DEFAULTS, growth_iters=2, batch_size=3)))
    items.append((1, dict(DEFAULTS, tau=1.05, epsilon=0.025)))
    items.append((2, dict(DEFAULTS, max_iter=40)))
    items.append((2, dict(DEFAULTS, epsilon=0.02, lambda1=0.3)))
    maps = Bt.solve_batched(pairs, items)
    gs = [p0[3], p1[3], p2[3]]
    for (p, cfg), m in zip(items, maps):
        ref = _solve_single(pairs[p], gs[p], cfg)
        T = m.dense().cpu().numpy()
        R = ref.tmap.cpu().numpy()
        # Two FP32 summation orders can put a stage-exit or duality-gap test that
        # lands within rounding of its threshold on either side: one batch more
        # or less per stage.
        assert abs(m.stats['iterations'] - ref.stats['iterations']) <= 2 * cfg['batch_size'], (cfg, m.stats, ref.stats)
        assert abs(m.stats['checks'] - ref.stats['checks']) <= 2, (cfg, m.stats, ref.stats)
        if cfg['tau'] < 10:
            assert m.stats['absorptions'] > 10 and ref.stats['absorptions'] > 10
        assert abs(m.stats['absorptions'] - ref.stats['absorptions']) <= 2 * cfg['batch_size']
        assert m.stats['hit_max_iter'] == ref.stats['hit_max_iter']
        assert m.status == (N.WOTG_MAX_ITER if cfg['max_iter'] == 40 else N.WOTG_OK)
        assert coupling_err(T, R) <= SAME_DEVICE_TOL, cfg
        rs = m.row_sums.cpu().numpy()
        assert np.abs(rs - R.sum(1)).max() <= SAME_DEVICE_TOL * np.abs(R.sum(1)).max()
        if cfg['growth_iters'] == 2:
            lg = m.learned_growth[1].cpu().numpy()
            assert np.abs(lg - ref.learned_growth[1].cpu().numpy()).max() <= SAME_DEVICE_TOL * np.abs(lg).max()


def test_batched_vs_oracle():
    """Three items of one pair against the FP64 oracle on the same coordinates."""
    from oracle import ot_model as oom, optimal_transport as oot
    from wot_gb300.ot import batch as Bt
    bp, x, y, g = _pair(400, 500, 7)
    C = oom.compute_default_cost_matrix(x.astype(np.float64), y.astype(np.float64))
    cfgs = [dict(DEFAULTS, epsilon=0.025, lambda1=0.3), dict(DEFAULTS, epsilon=0.1, lambda1=10.0),
            dict(DEFAULTS, growth_iters=2)]
    maps = Bt.solve_batched([bp], [(0, c) for c in cfgs])
    for cfg, m in zip(cfgs, maps):
        st = {}
        ref = oot.compute_transport_matrix(solver=oot.optimal_transport_duality_gap, C=C, G=g, stats=st, **cfg)
        R = ref[0]
        T = m.dense().cpu().numpy()
        assert_parity_batched(T, R, what=cfg)


def test_implicit_map_pull_back_push_forward():
    import torch
    from wot_gb300.ot import batch as Bt
    bp, x, y, g = _pair(260, 333, 9)
    m = Bt.solve_batched([bp], [(0, dict(DEFAULTS))])[0]
    T = m.dense().cpu().numpy()
    rng = np.random.default_rng(3)
    pj = (rng.random((8, 333)) < 0.2).astype(np.float64)
    pi = (rng.random((8, 260)) < 0.2).astype(np.float64)
    pull = m.pull_back(pj, normalize=False).cpu().numpy()
    push = m.push_forward(pi, normalize=False).cpu().numpy()
    ref_pull = (T @ pj.T).T
    ref_push = pi @ T
    assert np.abs(pull - ref_pull).max() <= 1e-5 * np.abs(ref_pull).max()
    assert np.abs(push - ref_push).max() <= 1e-5 * np.abs(ref_push).max()


def test_otmodel_batched_sweep_matches_single_maps():
    """OTModel.compute_transport_maps_batched on a 3-day course x 2 parameter
    sets: every map equals OTModel.compute_transport_map with that parameter set."""
    import wot_gb300 as wot
    from wot_gb300 import synthetic
    X, day, growth = synthetic.time_course([300, 350, 280], n_genes=200, n_clusters=4, seed=3)
    ids = np.array(['c%d' % i for i in range(len(day))])
    ds = wot.Dataset(X, wot.Frame({'day': day, 'cell_growth_rate': growth}, index=ids))
    model = wot.OTModel(ds, local_pca=20, form='materialized')
    sweep = [{'epsilon': 0.05, 'lambda1': 1.0}, {'epsilon': 0.1, 'lambda1': 3.0}]
    maps = model.compute_transport_maps_batched(sweep=sweep)
    assert sorted(maps) == [(0.0, 1.0, 0), (0.0, 1.0, 1), (1.0, 2.0, 0), (1.0, 2.0, 1)]
    for (t0, t1, i), m in maps.items():
        ref = wot.OTModel(ds, local_pca=20, form='materialized', **sweep[i]).compute_transport_map(t0, t1)
        R = np.asarray(ref.X)
        T = m.dense().cpu().numpy()
        assert coupling_err(T, R) <= SAME_DEVICE_TOL
