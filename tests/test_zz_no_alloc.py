"""The no-allocation solve entry point (wotg_compute_transport_matrix_noalloc).

It serves callers that cannot call cudaMalloc, for example a host whose
device memory is owned by another allocator or pool, or a code path where
cudaMalloc's implicit device synchronisation is not acceptable. It takes the
same inputs and outputs as wotg_compute_transport_matrix and takes its
scratch from a static device array, so its results must match the
workspace entry point call after call. The static array keeps the previous
call's contents, so a call that forgot to reset state would fail the second
comparison.

This file is named to be collected last: when it fails, a run that stops at
the first failure has already run every other test.
"""
import ast
import ctypes

import numpy as np
import pytest

COUPLING_TOL = 1e-4
DEFAULTS = dict(growth_iters=2, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


def _solve_both(lib, N, D, torch, C, G, cfg, solver, noalloc):
    """C: a dense cost (materialised form), or a pair of point sets (x, y) whose
    median-normalised squared distances are the cost (tensor-core form)."""
    if isinstance(C, tuple):
        cost = D.default_cost(*C)
    else:
        cost = D.cost_from_dense(C)
    I, J = cost.I, cost.J
    Gd = torch.as_tensor(np.asarray(G, dtype=np.float64), device='cuda')
    params = D.make_params(cfg, solver)
    prob = N.Problem(I=I, J=J, C=cost.C.data_ptr(), ldc=cost.ldc, cost_scale=float(cost.scale), G=Gd.data_ptr())
    if isinstance(C, tuple):
        prob.X, prob.ldx = cost.X.data_ptr(), cost.X.stride(0)
        prob.Y, prob.ldy = cost.Y.data_ptr(), cost.Y.stride(0)
        prob.d, prob.form = cost.X.shape[1], N.FORM_ONTHEFLY
    gi = params.growth_iters
    out = {'tmap': torch.empty((I, J), dtype=torch.float64, device='cuda'),
           'learned': torch.empty((gi, I), dtype=torch.float64, device='cuda'),
           'rows': torch.empty(I, dtype=torch.float64, device='cuda'),
           'u': torch.empty(I, dtype=torch.float64, device='cuda'),
           'v': torch.empty(J, dtype=torch.float64, device='cuda')}
    stats = N.Stats()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptrs = [out[k].data_ptr() for k in ('tmap', 'learned', 'rows', 'u', 'v')]
    if noalloc:
        st = lib.wotg_compute_transport_matrix_noalloc(ctypes.byref(prob), ctypes.byref(params), *ptrs,
                                                       ctypes.byref(stats), stream)
    else:
        nbytes = lib.wotg_problem_workspace_bytes(ctypes.byref(prob))
        ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
        st = lib.wotg_compute_transport_matrix(ctypes.byref(prob), ctypes.byref(params), *ptrs,
                                               ctypes.byref(stats), ws.data_ptr(), nbytes, stream)
    torch.cuda.synchronize()
    return st, {k: v.cpu().numpy() for k, v in out.items()}, stats.as_dict()


def _err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(pair_golden):
    import torch
    from wot_gb300 import _build, _native as N
    from wot_gb300.ot import device as D
    assert torch.cuda.is_available()
    _build.build()
    lib = N.load()
    z = pair_golden
    rng = np.random.default_rng(5)
    small_C = rng.random((37, 53)) * 2.0
    small_G = rng.lognormal(0, 0.3, 37)
    # tensor-core form: packed point tiles, the error word, the redo counters and
    # the exact-row list also live in the static array
    pts = (rng.normal(size=(300, 30)).astype(np.float32), (rng.normal(size=(420, 30)) + 0.2).astype(np.float32))
    pts_G = rng.lognormal(0, 0.3, 300)
    problems = [
        (z['C'], z['G'], dict(DEFAULTS), N.SOLVER_DUALITY_GAP),
        (z['C'], z['G'], dict(DEFAULTS), N.SOLVER_DUALITY_GAP),       # same problem again
        (pts, pts_G, dict(DEFAULTS, growth_iters=1), N.SOLVER_DUALITY_GAP),
        (small_C, small_G, dict(DEFAULTS, growth_iters=1, scaling_iter=200, extra_iter=40), N.SOLVER_FIXED_ITERS),
        (pts, pts_G, dict(DEFAULTS, growth_iters=1, epsilon=0.02), N.SOLVER_DUALITY_GAP),
    ]
    for C, G, cfg, solver in problems:
        st_a, ref, stats_a = _solve_both(lib, N, D, torch, C, G, cfg, solver, noalloc=False)
        st_b, got, stats_b = _solve_both(lib, N, D, torch, C, G, cfg, solver, noalloc=True)
        assert st_a == 0 and st_b == 0
        # the workspace call replays the final stage's batches as CUDA graphs, the
        # no-alloc call launches them plainly: the same kernels, the same results
        for k in ref:
            assert _err(got[k], ref[k]) <= 1e-12, k
        assert stats_b['iterations'] == stats_a['iterations']
        assert stats_b['exact_rows'] == stats_a['exact_rows']
    # and against the reference's own coupling for the golden pair
    params = ast.literal_eval(str(z['params_dg_default']))
    assert params == {}
    st, got, _ = _solve_both(lib, N, D, torch, z['C'], z['G'], dict(DEFAULTS, growth_iters=1),
                             N.SOLVER_DUALITY_GAP, noalloc=True)
    assert st == 0 and _err(got['tmap'], z['tmap_dg_default']) <= COUPLING_TOL


def test_noalloc_rejects_problems_beyond_its_scratch():
    """Rejected on the host before any device work (checked only where no GPU
    is present, with placeholder pointers that are never dereferenced)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip('run without a GPU: placeholder pointers')
    from wot_gb300 import _build, _native as N
    from wot_gb300.ot import device as D
    _build.build()
    lib = N.load()
    cap = lib.wotg_noalloc_scratch_bytes()
    assert cap == 32 << 20
    I, J = 1 << 20, 64
    assert lib.wotg_solve_workspace_bytes(I, J, J) > cap
    prob = N.Problem(I=I, J=J, C=0x1000, ldc=J, cost_scale=1.0, G=0x2000)
    params = D.make_params(dict(DEFAULTS), N.SOLVER_DUALITY_GAP)
    st = lib.wotg_compute_transport_matrix_noalloc(ctypes.byref(prob), ctypes.byref(params), None, None, None,
                                                   None, None, None, None)
    assert st == N.WOTG_TOO_LARGE
    assert 'static array' in lib.wotg_last_error().decode()
