"""Helpers of the map-analysis path (wot/tmap/util.py:52-94)."""
from __future__ import annotations

import numpy as np

from .. import dataset as ds_


def unique_timepoint(*populations):
    """The single time point shared by all populations (:52-71)."""
    times = set([pop.time for pop in populations])
    if len(times) > 1:
        raise ValueError("Several populations were given, but they are not from the same day")
    if len(times) < 1:
        raise ValueError("No cells found at the given day")
    return list(times)[0]


def glue_transport_maps(tmap_0, tmap_1):
    """Coupling t0->t2 from t0->t1 and t1->t2 (:74-94): X0 @ X1[ids of t1 in tmap_0.var].

    The product runs on the device in libwotg's FP64 GEMM kernel
    (wotg_gemm_f64), which gathers the rows of X1 that tmap_0's columns name.
    A column cell of tmap_0 that is not a row of tmap_1 raises KeyError, as
    indexing the reference's AnnData by it does."""
    import ctypes
    from .. import _native as N
    torch = N.require_cuda()
    cells = ds_.index(tmap_0.var)
    pos = {c: k for k, c in enumerate(ds_.index(tmap_1.obs).tolist())}
    missing = [c for c in cells.tolist() if c not in pos]
    if missing:
        raise KeyError('cells of tmap_0.var missing from tmap_1.obs: %s' % missing[:5])
    idx = torch.as_tensor(np.array([pos[c] for c in cells.tolist()], dtype=np.int64), device='cuda')
    X0 = torch.as_tensor(np.ascontiguousarray(np.asarray(tmap_0.X, dtype=np.float64)), device='cuda')
    X1 = torch.as_tensor(np.ascontiguousarray(np.asarray(tmap_1.X, dtype=np.float64)), device='cuda')
    M, K = X0.shape
    Nc = X1.shape[1]
    out = torch.empty((M, Nc), dtype=torch.float64, device='cuda')
    N.check(N.load().wotg_gemm_f64(X0.data_ptr(), K, X1.data_ptr(), Nc, idx.data_ptr(), out.data_ptr(), Nc, M, Nc,
                                   K, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), 'wotg_gemm_f64')
    result = out.cpu().numpy()
    return ds_.make_result(result, {c: ds_.column(tmap_0.obs, c) for c in ds_.columns(tmap_0.obs)},
                           ds_.index(tmap_0.obs), ds_.index(tmap_1.var), like=tmap_0)
