"""Maps held as potentials (ImplicitCoupling): pull-back and push-forward from
the points on the tensor cores (50-d, the packed 64-column form) against dense
products of the same coupling, and a chained pull-back of 8 cell-set indicator
vectors through TransportMapModel on implicit maps against the oracle's dense
chain (oracle/tmap.py, transport_map_model.py:301-365). Tolerance 1e-5 relative
to the largest entry.
"""
import logging

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5
CFG = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
           inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available()
    _build.build()
    _native.load()


def _solve(x, y, g, form='onthefly'):
    from wot_gb300.ot import device as D
    from wot_gb300.ot.implicit import ImplicitCoupling
    cost = D.default_cost(x, y)
    logging.disable(logging.WARNING)
    try:
        res = D.solve(cost, g, CFG, 0, want_tmap=False, want_potentials=True, form=form)
    finally:
        logging.disable(logging.NOTSET)
    return ImplicitCoupling.from_solve(cost, res)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_implicit_points_path_vs_dense():
    from wot_gb300 import synthetic
    x = synthetic.gaussian_mixture_points(300, d=50, seed=21)
    y = synthetic.gaussian_mixture_points(350, d=50, seed=22)
    g = np.random.default_rng(0).lognormal(0, 0.3, 300)
    m = _solve(x, y, g)
    assert m.cost is None  # points only
    T = m.dense().cpu().numpy()
    rng = np.random.default_rng(1)
    pj = (rng.random((8, 350)) < 0.1).astype(np.float64)
    pi = (rng.random((8, 300)) < 0.1).astype(np.float64)
    assert _rel(m.pull_back(pj, normalize=False).cpu().numpy(), (T @ pj.T).T) <= TOL
    assert _rel(m.push_forward(pi, normalize=False).cpu().numpy(), pi @ T) <= TOL
    # row sums of the map agree with the solve's own
    assert _rel(m.pull_back(np.ones(350), normalize=False).cpu().numpy()[0], T.sum(1)) <= TOL


def test_chained_pull_back_on_implicit_maps():
    import wot_gb300 as wot
    from oracle import tmap as otm
    from wot_gb300 import Population, synthetic
    sizes = [260, 310, 220, 280, 240]
    pts = [synthetic.gaussian_mixture_points(n, d=50, seed=30 + t) for t, n in enumerate(sizes)]
    tmaps, dense, ids, days = {}, {}, [], []
    for t in range(len(sizes) - 1):
        g = np.random.default_rng(t).lognormal(0, 0.3, sizes[t])
        m = _solve(pts[t], pts[t + 1], g)
        tmaps[(float(t), float(t + 1))] = m
        dense[(float(t), float(t + 1))] = m.dense().cpu().numpy()
    for t, n in enumerate(sizes):
        ids += ['d%d_c%d' % (t, i) for i in range(n)]
        days += [float(t)] * n
    meta = wot.Frame({'day': np.array(days)}, index=np.array(ids))
    model = wot.TransportMapModel(tmaps, meta)
    tp = [float(t) for t in range(len(sizes))]
    rng = np.random.default_rng(2)
    P = np.zeros((8, sizes[-1]))
    for k in range(8):
        P[k, rng.choice(sizes[-1], 25, replace=False)] = 1.0
    pops = [Population(tp[-1], P[k], 'set%d' % k) for k in range(8)]
    back = np.array([p.p for p in model.pull_back(*pops, to_time=0.0, as_list=True)])
    ref = otm.pull_back(dense, tp, P, tp[-1], 0.0)
    assert _rel(back, ref) <= TOL
    fwd = np.array([p.p for p in model.push_forward(Population(0.0, np.ones(sizes[0]), 'all'), to_time=tp[-1],
                                                     as_list=True)])
    assert _rel(fwd, otm.push_forward(dense, tp, np.ones((1, sizes[0])), 0.0, tp[-1])) <= TOL


@pytest.mark.parametrize('M,Nc,K', [(1, 1, 1), (65, 130, 17), (200, 70, 300), (3, 257, 64)])
def test_gemm_f64_with_row_gather(M, Nc, K):
    """wotg_gemm_f64 (the dense product of chained couplings) against NumPy FP64,
    with the right operand's rows gathered by an index as glue_transport_maps does."""
    import ctypes
    import torch
    from wot_gb300 import _native as N
    rng = np.random.default_rng(M * 7 + Nc)
    A = rng.random((M, K))
    B = rng.random((K + 5, Nc))
    rows = rng.permutation(K + 5)[:K]
    out = torch.empty((M, Nc), dtype=torch.float64, device='cuda')
    At, Bt = torch.as_tensor(A, device='cuda'), torch.as_tensor(B, device='cuda')
    r = torch.as_tensor(rows.astype(np.int64), device='cuda')
    st = N.load().wotg_gemm_f64(At.data_ptr(), K, Bt.data_ptr(), Nc, r.data_ptr(), out.data_ptr(), Nc, M, Nc, K,
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    np.testing.assert_allclose(out.cpu().numpy(), A @ B[rows], rtol=1e-13, atol=0)


def test_glue_rejects_cells_missing_from_the_next_map():
    import wot_gb300 as wot
    from wot_gb300.tmap.util import glue_transport_maps
    t0 = wot.Dataset(np.ones((2, 3)), wot.Frame(index=['a', 'b']), wot.Frame(index=['x', 'y', 'z']))
    t1 = wot.Dataset(np.ones((2, 2)), wot.Frame(index=['x', 'y']), wot.Frame(index=['p', 'q']))
    with pytest.raises(KeyError):
        glue_transport_maps(t0, t1)


@pytest.mark.parametrize('d,k', [(30, 11), (50, 3), (3, 1)])
def test_apply_points_populations_vs_fp64(d, k):
    """wotg_apply_points: k populations through a coupling held as potentials,
    one exp per entry for all of them (eight per launch: 11 takes two), against
    the same sums in FP64: real-valued, indicator and all-zero populations."""
    from wot_gb300 import synthetic
    from wot_gb300.ot import device as D
    I, J = 700, 900
    x = synthetic.gaussian_mixture_points(I, d=d, seed=d)
    y = synthetic.gaussian_mixture_points(J, d=d, seed=d + 1)
    rng = np.random.default_rng(k)
    C = ((x.astype(np.float64)[:, None, :] - y.astype(np.float64)[None, :, :]) ** 2).sum(-1)
    scale = 1.0 / (np.median(C) * 0.05)
    w = rng.normal(size=J) * 3
    b = rng.normal(size=I)
    P = rng.random((k, J))
    P[0] = (P[0] < 0.1)
    if k > 2:
        P[2] = 0.0
    out = D.apply_points(x, y, w, b, P, scale).cpu().numpy()
    z = w[None, :] - scale * C
    m = z.max(axis=1, keepdims=True)
    E = np.exp(z - m)
    ref = np.exp(b[:, None] + m) * (E @ P.T)          # I x k
    ref = ref.T
    for p in range(k):
        if np.abs(ref[p]).max() == 0:
            assert np.all(out[p] == 0)
        else:
            assert _rel(out[p], ref[p]) <= 1e-4, (p, _rel(out[p], ref[p]))
