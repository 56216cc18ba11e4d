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

    The product runs on the device (cuBLAS FP64 GEMM through torch)."""
    from .. import _native as N
    torch = N.require_cuda()
    cells = ds_.index(tmap_0.var)
    pos = {c: k for k, c in enumerate(ds_.index(tmap_1.obs).tolist())}
    idx = np.array([pos.get(c, -1) for c in cells.tolist()], dtype=np.int64)
    X0 = torch.as_tensor(np.asarray(tmap_0.X, dtype=np.float64), device='cuda')
    X1 = torch.as_tensor(np.asarray(tmap_1.X, dtype=np.float64), device='cuda')[torch.as_tensor(idx, device='cuda')]
    result = (X0 @ X1).cpu().numpy()
    return ds_.make_result(result, {c: ds_.column(tmap_0.obs, c) for c in ds_.columns(tmap_0.obs)},
                           ds_.index(tmap_0.obs), ds_.index(tmap_1.var), like=tmap_0)
