"""The adjoint (wotg_ot_adjoint via wot_gb300.ot.adjoint.ot_objective): gradient of
the converged unbalanced OT objective with respect to both point sets and the
log-growth rates, on a 500 x 600 problem of 30-d Gaussian-mixture points
(epsilon 0.05, lambda1 1, lambda2 50), against
  * autograd through unrolled FP64 Sinkhorn iterations (oracle/adjoint.py) for
    every coordinate, and
  * central FP64 finite differences of the converged objective on 64 random
    coordinates.
Tolerance: max |g - g_ref| <= 1e-4 max |g_ref| for each block (x, y, log g);
the objective value to 1e-6 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
EPS, L1, L2 = 0.05, 1.0, 50.0


@pytest.fixture(scope='module', autouse=True)
def built():
    import torch
    from wot_gb300 import _build, _native
    assert torch.cuda.is_available()
    _build.build()
    _native.load()


@pytest.fixture(scope='module')
def problem():
    import torch
    from oracle import adjoint as A
    from wot_gb300 import synthetic
    from wot_gb300.ot.adjoint import ot_objective
    I, J = 500, 600
    x = synthetic.gaussian_mixture_points(I, d=30, n_components=10, seed=11)
    y = synthetic.gaussian_mixture_points(J, d=30, n_components=10, seed=12)
    logg = np.random.default_rng(13).normal(0.0, 0.3, I)
    X64 = torch.tensor(x, dtype=torch.float64, device='cuda')
    Y64 = torch.tensor(y, dtype=torch.float64, device='cuda')
    L64 = torch.tensor(logg, dtype=torch.float64, device='cuda')
    scale = 1.0 / float(torch.median(A.cost(X64, Y64, 1.0).reshape(-1)))
    xt = torch.tensor(x, device='cuda', requires_grad=True)
    yt = torch.tensor(y, device='cuda', requires_grad=True)
    lt = torch.tensor(logg, device='cuda', requires_grad=True)
    obj = ot_objective(xt, yt, lt, epsilon=EPS, lambda1=L1, lambda2=L2, cost_scale=scale)
    obj.backward()
    D, ub, vb = A.objective(X64, Y64, L64, EPS, L1, L2, scale)
    return dict(X=X64, Y=Y64, L=L64, scale=scale, obj=float(obj.detach()), gx=xt.grad.double(), gy=yt.grad.double(),
                gl=lt.grad.double(), D=D, ub=ub, vb=vb)


def _rel(g, ref):
    return float((g - ref).abs().max() / ref.abs().max())


def test_adjoint_vs_unrolled_fp64(problem):
    from oracle import adjoint as A
    P = problem
    D2, gx, gy, gl = A.unrolled_gradient(P['X'], P['Y'], P['L'], EPS, L1, L2, P['scale'], P['ub'], P['vb'],
                                         n_unroll=30)
    assert abs(P['obj'] - P['D']) <= 1e-6 * abs(P['D'])
    assert _rel(P['gx'], gx) <= GRAD_TOL
    assert _rel(P['gy'], gy) <= GRAD_TOL
    assert _rel(P['gl'], gl) <= GRAD_TOL


def test_adjoint_vs_finite_differences(problem):
    from oracle import adjoint as A
    P = problem
    rng = np.random.default_rng(5)
    coords = []
    for _ in range(24):
        coords.append(('x', (int(rng.integers(500)), int(rng.integers(30)))))
    for _ in range(24):
        coords.append(('y', (int(rng.integers(600)), int(rng.integers(30)))))
    for _ in range(16):
        coords.append(('logg', (int(rng.integers(500)),)))
    fd = A.fd_gradient(P['X'], P['Y'], P['L'], EPS, L1, L2, P['scale'], coords, P['ub'], P['vb'], h=1e-4)
    g = {'x': P['gx'], 'y': P['gy'], 'logg': P['gl']}
    for name in ('x', 'y', 'logg'):
        sel = [(float(g[name][i]), f) for (n, i), f in zip(coords, fd) if n == name]
        scale = max(abs(f) for _, f in sel)
        err = max(abs(a - f) for a, f in sel)
        assert err <= GRAD_TOL * max(scale, float(g[name].abs().max())), (name, err, scale)


def test_adjoint_directional_derivative_full_size():
    """At the full 10000 x 12000 size (30-d points from a 10-component mixture,
    log g ~ N(0, 0.3^2)), where no FP64 oracle runs: the gradient's directional
    derivative along its own sign pattern, <g, sign(g)> = |g|_1, against the
    central difference of the converged objective (each a full solve + refine)
    with every coordinate moved by 1e-3. Tolerance 1e-3 relative."""
    import torch
    from wot_gb300 import synthetic
    from wot_gb300.ot.adjoint import ot_objective
    I, J, d, h = 10000, 12000, 30, 1e-3
    x = torch.tensor(synthetic.gaussian_mixture_points(I, d=d, n_components=10, seed=31), device='cuda')
    y = torch.tensor(synthetic.gaussian_mixture_points(J, d=d, n_components=10, seed=32), device='cuda')
    lg = torch.tensor(np.random.default_rng(33).normal(0.0, 0.3, I), device='cuda')
    from wot_gb300.ot import device as D
    # the cost scale (1/median of the unperturbed cost) stays fixed across the three objectives
    c = D.cost_from_points(x.float(), y.float())
    scale = 1.0 / D.median(c)
    del c
    xt, yt, lt = (t.clone().requires_grad_(True) for t in (x, y, lg))
    obj = ot_objective(xt, yt, lt, epsilon=EPS, lambda1=L1, lambda2=L2, cost_scale=scale)
    obj.backward()
    sx, sy, sl = torch.sign(xt.grad), torch.sign(yt.grad), torch.sign(lt.grad)
    ana = float(xt.grad.abs().sum() + yt.grad.abs().sum() + lt.grad.abs().sum())
    with torch.no_grad():
        dp = float(ot_objective(x + h * sx, y + h * sy, lg + h * sl, epsilon=EPS, lambda1=L1, lambda2=L2,
                                cost_scale=scale))
        dm = float(ot_objective(x - h * sx, y - h * sy, lg - h * sl, epsilon=EPS, lambda1=L1, lambda2=L2,
                                cost_scale=scale))
    fd = (dp - dm) / (2 * h)
    assert abs(fd - ana) <= 1e-3 * abs(ana), (fd, ana)
