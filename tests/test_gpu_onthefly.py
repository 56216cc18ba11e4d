"""The on-the-fly (tensor-core) form: the tcgen05 split-precision product,
then whole solves against the materialised form and the oracle.

Tolerances (tests/parity.py): couplings within 1e-4 of the FP64 oracle, as for
the materialised form; small entries and marginals within the on-the-fly
form's own bounds (ONTHEFLY_BOUNDS: the FP16 hi/lo split of the points,
accumulated in FP32 on the tensor cores, sets them); against the materialised
form, couplings within 1e-4 normalised and elementwise. The MMA self-test
checks the FP16 hi/lo product to 5e-6 of max|D| (hi.hi alone: 2e-3).
"""
import ctypes

import numpy as np
import pytest

from parity import assert_parity, assert_parity_onthefly

pytestmark = pytest.mark.gpu

DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available()
    _build.build()
    _native.load()


@pytest.mark.parametrize('terms,tol', [(1, 2e-3), (3, 5e-6)])
def test_tcgen05_split_product(terms, tol):
    import torch
    from wot_gb300 import _native as N
    rng = np.random.default_rng(terms)
    A = rng.normal(size=(128, 32)).astype(np.float32)
    B = rng.normal(size=(128, 32)).astype(np.float32)
    At, Bt = torch.as_tensor(A, device='cuda'), torch.as_tensor(B, device='cuda')
    D = torch.zeros((128, 128), dtype=torch.float32, device='cuda')
    e = torch.zeros(1, dtype=torch.int32, device='cuda')
    st = N.load().wotg_tc_selftest(At.data_ptr(), Bt.data_ptr(), D.data_ptr(), 128, 512, terms, e.data_ptr(),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == 0 and int(e.item()) == 0
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    assert np.abs(D.cpu().numpy() - ref).max() <= tol * np.abs(ref).max()


def _points(I, J, d, seed):
    from wot_gb300 import synthetic
    x = synthetic.gaussian_mixture_points(I, d=d, seed=seed)
    y = synthetic.gaussian_mixture_points(J, d=d, seed=seed + 1)
    g = np.random.default_rng(seed).lognormal(0, 0.3, I)
    return x, y, g


@pytest.mark.parametrize('I,J,d', [(37, 53, 30), (300, 257, 30), (700, 900, 30), (250, 130, 50), (129, 128, 3)])
def test_onthefly_matches_materialized(I, J, d):
    from wot_gb300.ot import device as D
    x, y, g = _points(I, J, d, I + J)
    cost = D.default_cost(x, y)
    for solver, extra in ((0, {}), (1, dict(scaling_iter=200, extra_iter=50))):
        cfg = dict(DEFAULTS, **extra)
        a = D.solve(cost, g, cfg, solver, form='materialized')
        b = D.solve(cost, g, cfg, solver, form='onthefly')
        Ta, Tb = a.tmap.cpu().numpy(), b.tmap.cpu().numpy()
        # the two forms may stop a batch apart, so marginals are not compared here
        assert_parity(Tb, Ta, marginals=False, what=solver)
        if solver == 0:
            assert abs(a.stats['iterations'] - b.stats['iterations']) <= 5


@pytest.mark.parametrize('eps', [0.05, 0.01])
def test_onthefly_vs_oracle_c0_shape(eps):
    from oracle import ot_model as oom, optimal_transport as oot
    from wot_gb300 import synthetic
    from wot_gb300.ot import device as D
    X, day, growth = synthetic.time_course([2000, 2500], n_genes=1000, n_clusters=6, seed=0)
    x0, x1, s, _ = oom.compute_pca(X[day == 0], X[day == 1], 30)
    a, b = x0 * s, x1 * s
    C = oom.compute_default_cost_matrix(a, b)
    G = growth[day == 0]
    cfg = dict(DEFAULTS, epsilon=eps)
    st = {}
    ref = oot.optimal_transport_duality_gap(C=C, G=G, stats=st, **cfg)
    res = D.solve(D.default_cost(a.astype(np.float32), b.astype(np.float32)), G, cfg, 0, form='onthefly')
    T = res.tmap.cpu().numpy()
    assert_parity_onthefly(T, ref, eps, what=eps)
    assert abs(res.stats['iterations'] - st['iterations']) <= 10


@pytest.mark.parametrize('I,J,d', [(37, 53, 30), (300, 1000, 30), (129, 257, 50)])
def test_lse_points_primitive(I, J, d):
    """wotg_lse_points against an FP64 log-sum-exp of the same points."""
    from wot_gb300.ot import device as D
    x, y, _ = _points(I, J, d, 3)
    rng = np.random.default_rng(4)
    w = rng.normal(size=J) * 3
    C = ((x.astype(np.float64)[:, None, :] - y.astype(np.float64)[None, :, :]) ** 2).sum(-1)
    scale = 1.0 / (np.median(C) * 0.05)
    L = D.lse_points(x, y, w, scale).cpu().numpy()
    z = w[None, :] - scale * C
    m = z.max(axis=1)
    ref = m + np.log(np.exp(z - m[:, None]).sum(axis=1))
    np.testing.assert_allclose(L, ref, rtol=0, atol=5e-5 * max(1.0, np.abs(ref).max()))


def test_speculative_form_fallback_matches_materialized():
    """Warm-started iterations from shifted potentials: each side's first
    half-step runs the exact form, the next ones the speculative form with
    offsets far from the new sums (a shift of v by s moves a row's
    log-sum-exp by about (1 - alpha1 alpha2) s / eps per iteration: ~190 in
    base 2 here), so rows take the exact per-row recompute (exact_rows > 0);
    the potentials equal the same iterations on the materialised form."""
    import torch
    from wot_gb300.ot import device as D
    cfg = dict(DEFAULTS, lambda1=0.1)
    x, y, g = _points(700, 900, 30, seed=5)
    cost = D.default_cost(x, y)
    res = D.solve(cost, g, cfg, 0, want_tmap=False, want_potentials=True, form='materialized')
    eps = res.stats['final_epsilon']
    rng = np.random.default_rng(0)
    u0 = res.u_bar.clone()
    v0 = res.v_bar + 20.0 + torch.as_tensor(rng.normal(0.0, 1.0, 900), device='cuda')
    out = {}
    for form in ('materialized', 'onthefly'):
        u, v = u0.clone(), v0.clone()
        _, _, st = D.refine(cost, g, cfg, u, v, eps, 6, form=form)
        out[form] = (u.cpu().numpy(), v.cpu().numpy(), st)
    assert out['onthefly'][2]['exact_rows'] > 0
    assert out['materialized'][2]['exact_rows'] == 0
    for k in (0, 1):
        a, b = out['onthefly'][k], out['materialized'][k]
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()


def test_exp2_rate_is_measured():
    """wotg_exp2_rate: the measured ex2 throughput, the per-element ceiling of every
    half-step form, lies between 1e12 and 1e14 exp2/s on this part."""
    import ctypes
    import torch
    from wot_gb300 import _native
    r = ctypes.c_double(0.0)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert _native.load().wotg_exp2_rate(ctypes.byref(r), st) == 0
    assert 1e12 < r.value < 1e14


def test_lse_points_kernel_timing():
    """wotg_lse_points_timing: both forms of the tensor-core kernel run and time
    positive; the speculative form (sums against the previous log-sum-exp) is no
    slower than the exact form with its running maximum (10 % allowance)."""
    import ctypes
    import torch
    from wot_gb300 import _native, synthetic
    lib = _native.load()
    I, J, d = 3000, 3500, 30
    X = torch.tensor(synthetic.gaussian_mixture_points(I, d=d, seed=3), dtype=torch.float32, device='cuda')
    Y = torch.tensor(synthetic.gaussian_mixture_points(J, d=d, seed=4), dtype=torch.float32, device='cuda')
    w = torch.zeros(J, dtype=torch.float64, device='cuda')
    ws = torch.empty(lib.wotg_lse_points_workspace_bytes(I, J, d), dtype=torch.uint8, device='cuda')
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ms = {}
    for spec in (0, 1):
        r = ctypes.c_float(0.0)
        assert lib.wotg_lse_points_timing(X.data_ptr(), I, d, Y.data_ptr(), J, d, d, 0.05, w.data_ptr(), spec, 10,
                                          ctypes.byref(r), ws.data_ptr(), ws.numel(), st) == 0
        ms[spec] = r.value
    assert ms[0] > 0 and ms[1] > 0
    assert ms[1] <= 1.1 * ms[0]


def test_bounded_wait_runs_out_and_the_device_recovers():
    """A tensor-core half-step whose mbarrier waits get no tries at all: the
    kernel gives up, drains its bulk copies and products, frees its tensor
    memory and reports WOTG_CUDA_ERROR; the next half-steps (the same call with
    the normal budget, and a whole solve) are correct."""
    import ctypes
    import torch
    from wot_gb300 import _native as N
    from wot_gb300.ot import device as D
    lib = N.load()
    I, J, d = 700, 900, 30
    x, y, g = _points(I, J, d, 21)
    w = np.random.default_rng(22).normal(size=J) * 3
    C = ((x.astype(np.float64)[:, None, :] - y.astype(np.float64)[None, :, :]) ** 2).sum(-1)
    scale = 1.0 / (np.median(C) * 0.05)
    X, Y = torch.as_tensor(x, device='cuda'), torch.as_tensor(y, device='cuda')
    wt = torch.as_tensor(w, device='cuda')
    L = torch.zeros(I, dtype=torch.float64, device='cuda')
    ws = torch.empty(lib.wotg_lse_points_workspace_bytes(I, J, d), dtype=torch.uint8, device='cuda')
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(tries):
        return lib.wotg_lse_points_bounded(X.data_ptr(), I, d, Y.data_ptr(), J, d, d, scale, wt.data_ptr(),
                                           L.data_ptr(), tries, ws.data_ptr(), ws.numel(), st)

    assert run(0) == N.WOTG_CUDA_ERROR
    assert 'bounded wait ran out' in lib.wotg_last_error().decode()
    assert run(4000001) == N.WOTG_BADARG
    assert run(4000000) == 0
    z = w[None, :] - scale * C
    m = z.max(axis=1)
    ref = m + np.log(np.exp(z - m[:, None]).sum(axis=1))
    np.testing.assert_allclose(L.cpu().numpy(), ref, rtol=0, atol=5e-5 * max(1.0, np.abs(ref).max()))
    assert run(0) == N.WOTG_CUDA_ERROR
    cost = D.default_cost(x, y)
    a = D.solve(cost, g, DEFAULTS, 0, form='materialized')
    b = D.solve(cost, g, DEFAULTS, 0, form='onthefly')
    assert_parity(b.tmap.cpu().numpy(), a.tmap.cpu().numpy(), marginals=False)


def test_fma_pipe_exp2_meets_its_bound():
    """The FMA-pipe 2^z of the epilogue (range reduction, degree-5 minimax
    polynomial, exponent bits) against FP64 2^z: relative error <= 3e-7 on
    [-125, 126] (the polynomial's 7.5e-8 plus FP32 Horner rounding); beyond the
    clamp, 2^126 (far above the speculative form's safe range, so such a row is
    recomputed exactly) and at most 2^-125; NaN stays NaN."""
    import torch
    from wot_gb300 import _native as N
    lib = N.load()
    z = np.concatenate([np.linspace(-125, 126, 2_000_003), np.linspace(-0.5, 0.5, 100_001),
                        [-np.inf, -1e30, -200.0, -125.5, 126.5, 300.0, 1e30, np.inf, np.nan]]).astype(np.float32)
    zt = torch.as_tensor(z, device='cuda')
    out = torch.empty_like(zt)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.wotg_exp2_fma(zt.data_ptr(), out.data_ptr(), z.size, st) == 0
    r = out.cpu().numpy().astype(np.float64)
    zd = z.astype(np.float64)
    inside = (zd >= -125) & (zd <= 126)
    ref = np.exp2(zd[inside])
    assert (np.abs(r[inside] - ref) / ref).max() <= 3e-7
    above = zd > 126
    assert np.all(r[above] >= 2.0 ** 126 * (1 - 3e-7))
    below = zd < -125
    assert np.all((r[below] >= 0) & (r[below] <= 2.0 ** -125 * (1 + 3e-7)))
    assert np.isnan(r[np.isnan(zd)]).all()
    assert lib.wotg_exp2_fma(zt.data_ptr(), out.data_ptr(), 0, st) == N.WOTG_BADARG
