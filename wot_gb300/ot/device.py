"""Device-level API over libwotg: costs, median, solves and population transport.

Buffers are torch tensors on the current CUDA device (torch is used for device
memory and streams only); every computation is a libwotg kernel launched on
``torch.cuda.current_stream()``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from .. import _native as N

# The reference's solver keys (ot_model.py:85-87) and their C types.
_PARAM_KEYS = ('epsilon', 'lambda1', 'lambda2', 'epsilon0', 'tau', 'tolerance', 'max_iter',
               'batch_size', 'scaling_iter', 'inner_iter_max', 'extra_iter', 'growth_iters')
DEFAULTS = {'growth_iters': 1, 'epsilon': 0.05, 'lambda1': 1, 'lambda2': 50, 'epsilon0': 1, 'tau': 10000,
            'scaling_iter': 3000, 'inner_iter_max': 50, 'tolerance': 1e-8, 'max_iter': 1e7,
            'batch_size': 5, 'extra_iter': 1000}


@dataclass
class DeviceCost:
    """FP32 cost on the device, I x ldc with +inf padding; reference cost = scale * C.

    When built from points, ``X`` / ``Y`` keep the FP32 points so that the
    on-the-fly (tensor-core) form can recompute cost tiles."""
    C: object
    I: int
    J: int
    ldc: int
    scale: float = 1.0
    X: object = None
    Y: object = None

    @property
    def shape(self):
        return (self.I, self.J)


@dataclass
class SolveResult:
    tmap: object = None            # I x J FP64 device tensor (or None)
    learned_growth: list = field(default_factory=list)   # growth_iters device tensors of I
    row_sums: object = None        # tmap.sum(axis=1)
    u_bar: object = None
    v_bar: object = None
    stats: dict = field(default_factory=dict)
    status: int = 0


def _torch():
    return N.require_cuda()


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev_f64(x, torch):
    if isinstance(x, torch.Tensor):
        return x.to(device='cuda', dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.float64)), device='cuda')


def _dev_f32(x, torch):
    if isinstance(x, torch.Tensor):
        return x.to(device='cuda', dtype=torch.float32).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(x, dtype=np.float32)), device='cuda')


def cost_from_dense(C) -> DeviceCost:
    """User-supplied dense cost (reference's C, FP64) -> FP32 device cost, scale 1."""
    torch = _torch()
    C64 = _dev_f64(C, torch)
    if C64.dim() != 2:
        raise ValueError('cost matrix must be 2-D')
    I, J = C64.shape
    ldc = N.round_up(J, 4)
    C32 = torch.empty((I, ldc), dtype=torch.float32, device='cuda')
    N.check(N.load().wotg_cost_from_f64(C64.data_ptr(), I, J, C32.data_ptr(), ldc, _stream()),
            'wotg_cost_from_f64')
    return DeviceCost(C32, I, J, ldc, 1.0)


def cost_from_points(x, y) -> DeviceCost:
    """Squared-Euclidean FP32 cost between point sets (rows), unnormalised (scale 1)."""
    torch = _torch()
    X = _dev_f32(x, torch)
    Y = _dev_f32(y, torch)
    if X.dim() != 2 or Y.dim() != 2 or X.shape[1] != Y.shape[1]:
        raise ValueError('points must be 2-D with the same dimension')
    I, d = X.shape
    J = Y.shape[0]
    ldc = N.round_up(J, 4)
    C32 = torch.empty((I, ldc), dtype=torch.float32, device='cuda')
    N.check(N.load().wotg_cost_sqeuclidean(X.data_ptr(), I, X.stride(0), Y.data_ptr(), J, Y.stride(0), d,
                                           C32.data_ptr(), ldc, _stream()), 'wotg_cost_sqeuclidean')
    return DeviceCost(C32, I, J, ldc, 1.0, X, Y)


def median(cost: DeviceCost) -> float:
    """np.median of the valid FP32 cost entries (exact on the FP32 values)."""
    torch = _torch()
    lib = N.load()
    ws = torch.empty(lib.wotg_median_workspace_bytes(), dtype=torch.uint8, device='cuda')
    out = ctypes.c_double(0.0)
    N.check(lib.wotg_median(cost.C.data_ptr(), cost.I, cost.J, cost.ldc, ctypes.byref(out), ws.data_ptr(),
                            ws.numel(), _stream()), 'wotg_median')
    return out.value


def default_cost(x, y) -> DeviceCost:
    """Median-normalised squared-Euclidean cost (wot/ot/ot_model.py:242-253)."""
    c = cost_from_points(x, y)
    med = median(c)
    c.scale = 1.0 / med
    return c


def make_params(cfg: dict, solver: int) -> N.Params:
    p = dict(DEFAULTS)
    p.update({k: cfg[k] for k in _PARAM_KEYS if k in cfg and cfg[k] is not None})
    if cfg.get('tau', 0) is None:
        # the reference compares max(...) > None, which Python 3 rejects
        raise TypeError("'>' not supported between instances of 'numpy.float64' and 'NoneType'")
    return N.Params(epsilon=float(p['epsilon']), lambda1=float(p['lambda1']), lambda2=float(p['lambda2']),
                    epsilon0=float(p['epsilon0']), tau=float(p['tau']), tolerance=float(p['tolerance']),
                    max_iter=float(p['max_iter']), batch_size=int(p['batch_size']),
                    scaling_iter=int(p['scaling_iter']), inner_iter_max=int(p['inner_iter_max']),
                    extra_iter=int(p['extra_iter']), growth_iters=int(p['growth_iters']), solver=int(solver))


FORMS = {'materialized': N.FORM_MATERIALIZED, 'onthefly': N.FORM_ONTHEFLY}
TC_MAX_DIM = 62   # point dimensions the tensor-core half-step packs (two bias columns in 64)


# Below this many cost entries the two forms take about the same time (measured
# on GB300 at 30 dimensions: 1500 x 1800 cells 24 ms streamed against 30 ms on
# the tensor cores per solve, 2500 x 3000 32 ms against 30 ms, 9000 x 10800
# 93 ms against 43 ms), so 'auto' keeps the streamed form there: its exponents
# are exact to the FP32 storage of C, while the tensor-core form's carry the
# error of the points' 22-bit FP16 hi/lo split accumulated in FP32 (about
# kappa |x| |y| 2^-22 per exponent).
TC_AUTO_MIN_ENTRIES = 4_000_000


def resolve_form(cost: DeviceCost, form: str) -> int:
    """'materialized' streams the FP32 cost; 'onthefly' recomputes cost tiles
    from the points on the tensor cores; 'auto' picks the latter when the cost
    was built from points of at most TC_MAX_DIM dimensions and has at least
    TC_AUTO_MIN_ENTRIES entries (where it is the faster form)."""
    if form == 'auto':
        tc = (cost.X is not None and cost.X.shape[1] <= TC_MAX_DIM
              and cost.I * cost.J >= TC_AUTO_MIN_ENTRIES)
        form = 'onthefly' if tc else 'materialized'
    if form not in FORMS:
        raise ValueError("form must be 'auto', 'materialized' or 'onthefly'")
    if form == 'onthefly' and cost.X is None:
        raise ValueError('the on-the-fly form needs a cost built from points')
    return FORMS[form]


def solve(cost: DeviceCost, G, cfg: dict, solver: int = N.SOLVER_DUALITY_GAP, want_tmap: bool = True,
          want_potentials: bool = False, tmap_out=None, form: str = 'materialized') -> SolveResult:
    """All growth iterations of one transport problem on the device
    (wot.ot.compute_transport_matrix, optimal_transport.py:10-33)."""
    torch = _torch()
    lib = N.load()
    params = make_params(cfg, solver)
    I, J = cost.I, cost.J
    Gd = _dev_f64(G, torch).reshape(-1)
    if Gd.numel() != I:
        raise ValueError('G has %d entries for %d source cells' % (Gd.numel(), I))
    gi = max(1, params.growth_iters)
    learned = torch.empty((gi, I), dtype=torch.float64, device='cuda')
    row_sums = torch.empty(I, dtype=torch.float64, device='cuda')
    tmap = None
    if want_tmap:
        tmap = tmap_out if tmap_out is not None else torch.empty((I, J), dtype=torch.float64, device='cuda')
    u_bar = torch.empty(I, dtype=torch.float64, device='cuda') if want_potentials else None
    v_bar = torch.empty(J, dtype=torch.float64, device='cuda') if want_potentials else None
    prob = N.Problem(I=I, J=J, C=cost.C.data_ptr(), ldc=cost.ldc, cost_scale=float(cost.scale),
                     G=Gd.data_ptr())
    if resolve_form(cost, form) == N.FORM_ONTHEFLY:
        prob.X, prob.ldx = cost.X.data_ptr(), cost.X.stride(0)
        prob.Y, prob.ldy = cost.Y.data_ptr(), cost.Y.stride(0)
        prob.d, prob.form = cost.X.shape[1], N.FORM_ONTHEFLY
    nbytes = lib.wotg_problem_workspace_bytes(ctypes.byref(prob))
    if nbytes == 0:
        raise ValueError('invalid transport problem')
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    stats = N.Stats()
    status = lib.wotg_compute_transport_matrix(ctypes.byref(prob), ctypes.byref(params), N.ptr(tmap),
                                               learned.data_ptr(), row_sums.data_ptr(), N.ptr(u_bar),
                                               N.ptr(v_bar), ctypes.byref(stats), ws.data_ptr(), nbytes,
                                               _stream())
    N.check(status, 'wotg_compute_transport_matrix')
    return SolveResult(tmap=tmap, learned_growth=[learned[k] for k in range(gi)], row_sums=row_sums,
                       u_bar=u_bar, v_bar=v_bar, stats=stats.as_dict(), status=status)


def _problem(cost: DeviceCost, Gd, form: str):
    prob = N.Problem(I=cost.I, J=cost.J, C=cost.C.data_ptr(), ldc=cost.ldc, cost_scale=float(cost.scale),
                     G=Gd.data_ptr())
    if resolve_form(cost, form) == N.FORM_ONTHEFLY:
        prob.X, prob.ldx = cost.X.data_ptr(), cost.X.stride(0)
        prob.Y, prob.ldy = cost.Y.data_ptr(), cost.Y.stride(0)
        prob.d, prob.form = cost.X.shape[1], N.FORM_ONTHEFLY
    return prob


def refine(cost: DeviceCost, G, cfg: dict, u_bar, v_bar, eps: float, n_iter: int, form: str = 'materialized'):
    """n_iter warm-started iterations at epsilon `eps` from absorbed potentials
    (in place); polishes a duality-gap solve towards the exact optimum."""
    torch = _torch()
    lib = N.load()
    params = make_params(cfg, N.SOLVER_DUALITY_GAP)
    Gd = _dev_f64(G, torch).reshape(-1)
    prob = _problem(cost, Gd, form)
    nbytes = lib.wotg_problem_workspace_bytes(ctypes.byref(prob))
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    stats = N.Stats()
    N.check(lib.wotg_refine_potentials(ctypes.byref(prob), ctypes.byref(params), float(eps), int(n_iter),
                                       u_bar.data_ptr(), v_bar.data_ptr(), ctypes.byref(stats), ws.data_ptr(),
                                       nbytes, _stream()), 'wotg_refine_potentials')
    return u_bar, v_bar, stats.as_dict()


def ot_adjoint(X, Y, cost_scale: float, eps: float, lambda1: float, lambda2: float, u_bar, v_bar, p,
               want_y: bool = True, want_p: bool = True):
    """(objective, grad_x, grad_y, grad_p) of the converged unbalanced OT dual at
    the potentials (u_bar, v_bar); X, Y FP32 device points."""
    torch = _torch()
    lib = N.load()
    I, d = X.shape
    J = Y.shape[0]
    gx = torch.empty((I, d), dtype=torch.float64, device='cuda')
    gy = torch.empty((J, d), dtype=torch.float64, device='cuda') if want_y else None
    gp = torch.empty(I, dtype=torch.float64, device='cuda') if want_p else None
    nbytes = lib.wotg_ot_adjoint_workspace_bytes(I, J)
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    obj = ctypes.c_double(0.0)
    N.check(lib.wotg_ot_adjoint(X.data_ptr(), I, X.stride(0), Y.data_ptr(), J, Y.stride(0), d, float(cost_scale),
                                float(eps), float(lambda1), float(lambda2), u_bar.data_ptr(), v_bar.data_ptr(),
                                p.data_ptr(), gx.data_ptr(), N.ptr(gy), N.ptr(gp), ctypes.byref(obj),
                                ws.data_ptr(), nbytes, _stream()), 'wotg_ot_adjoint')
    return obj.value, gx, gy, gp


def apply_coupling(X, P, transpose: bool, normalize: bool):
    """push (transpose=False): P @ X; pull (transpose=True): (X @ P.T).T; FP64 on device."""
    torch = _torch()
    Xd = _dev_f64(X, torch)
    Pd = _dev_f64(P, torch)
    if Pd.dim() == 1:
        Pd = Pd.reshape(1, -1)
    I, J = Xd.shape
    k = Pd.shape[0]
    if Pd.shape[1] != (J if transpose else I):
        raise ValueError('population length %d does not match the coupling %s' % (Pd.shape[1], (I, J)))
    out = torch.empty((k, I if transpose else J), dtype=torch.float64, device='cuda')
    N.check(N.load().wotg_apply_coupling_f64(Xd.data_ptr(), I, J, Pd.data_ptr(), k, int(transpose),
                                             int(normalize), out.data_ptr(), _stream()),
            'wotg_apply_coupling_f64')
    return out


def lse_points(x, y, w, scale: float):
    """L_i = log sum_j exp(w_j - scale |x_i - y_j|^2) on the tensor cores (FP64 out)."""
    torch = _torch()
    X = _dev_f32(x, torch)
    Y = _dev_f32(y, torch)
    W = _dev_f64(w, torch).reshape(-1)
    I, d = X.shape
    J = Y.shape[0]
    lib = N.load()
    nbytes = lib.wotg_lse_points_workspace_bytes(I, J, d)
    if nbytes == 0:
        raise ValueError('invalid points for the on-the-fly half-step (d <= 62)')
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    L = torch.empty(I, dtype=torch.float64, device='cuda')
    N.check(lib.wotg_lse_points(X.data_ptr(), I, X.stride(0), Y.data_ptr(), J, Y.stride(0), d, float(scale),
                                W.data_ptr(), L.data_ptr(), ws.data_ptr(), nbytes, _stream()), 'wotg_lse_points')
    return L


def apply_points(x, y, w, bias, P, scale: float):
    """out[k, i] = exp(bias_i) sum_j exp(w_j - scale |x_i - y_j|^2) P[k, j] on the
    tensor cores, one exp per (i, j) for all rows of P (FP64 k x I out)."""
    torch = _torch()
    X = _dev_f32(x, torch)
    Y = _dev_f32(y, torch)
    W = _dev_f64(w, torch).reshape(-1)
    B = _dev_f64(bias, torch).reshape(-1)
    Pd = _dev_f64(P, torch)
    I, d = X.shape
    J = Y.shape[0]
    k = Pd.shape[0]
    lib = N.load()
    nbytes = lib.wotg_apply_points_workspace_bytes(I, J, d)
    if nbytes == 0:
        raise ValueError('invalid points for the on-the-fly form (d <= 62)')
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    out = torch.empty((k, I), dtype=torch.float64, device='cuda')
    N.check(lib.wotg_apply_points(X.data_ptr(), I, X.stride(0), Y.data_ptr(), J, Y.stride(0), d, float(scale),
                                  W.data_ptr(), B.data_ptr(), Pd.data_ptr(), Pd.stride(0), k, out.data_ptr(),
                                  ws.data_ptr(), nbytes, _stream()), 'wotg_apply_points')
    return out


def transpose_cost(cost: DeviceCost):
    """C^T (J x ldct FP32, +inf padding) of a device cost; the column form a batch reads."""
    torch = _torch()
    ldct = N.round_up(cost.I, 4)
    CT = torch.empty((cost.J, ldct), dtype=torch.float32, device='cuda')
    N.check(N.load().wotg_transpose_cost(cost.C.data_ptr(), cost.I, cost.J, cost.ldc, CT.data_ptr(), ldct,
                                         _stream()), 'wotg_transpose_cost')
    return CT


def lse_multi(C, I: int, J: int, ldc: int, W, kappa2):
    """L[k, i] = log sum_j exp2(W[k, j] - kappa2[k] C[i, j]) for K weight rows at once
    (one read of C); W is K x ldw FP32 on the device (ldw >= roundup(J, 4))."""
    torch = _torch()
    lib = N.load()
    K, ldw = W.shape
    k2 = (ctypes.c_float * K)(*[float(x) for x in kappa2])
    nbytes = lib.wotg_lse_matvec_multi_workspace_bytes(I, K)
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    L = torch.empty((K, I), dtype=torch.float64, device='cuda')
    N.check(lib.wotg_lse_matvec_multi(C.data_ptr(), I, J, ldc, W.data_ptr(), ldw, k2, K, L.data_ptr(), I,
                                      ws.data_ptr(), nbytes, _stream()), 'wotg_lse_matvec_multi')
    return L


def coupling_from_potentials(cost: DeviceCost, u_bar, v_bar, eps: float, log_scale: float):
    """Dense FP64 coupling exp((u_bar_i + v_bar_j - scale C_ij) / eps + log_scale)."""
    torch = _torch()
    out = torch.empty((cost.I, cost.J), dtype=torch.float64, device='cuda')
    N.check(N.load().wotg_coupling_from_potentials(cost.C.data_ptr(), cost.I, cost.J, cost.ldc, float(cost.scale),
                                                   float(eps), u_bar.data_ptr(), v_bar.data_ptr(),
                                                   float(log_scale), out.data_ptr(), _stream()),
            'wotg_coupling_from_potentials')
    return out
