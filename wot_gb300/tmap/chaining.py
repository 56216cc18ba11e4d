"""Long-range couplings by chaining consecutive maps (wot/tmap/chaining.py:4-108)."""
from __future__ import annotations

from .util import glue_transport_maps


def chain_transport_maps(tmap_model, pairs_list):
    """Glue the maps of consecutive day pairs (:4-40)."""
    for i in range(len(pairs_list) - 1):
        if pairs_list[i][1] != pairs_list[i + 1][0]:
            raise ValueError("Transport maps cannot be glued together : invalid path")
    for a, b in pairs_list:
        if a >= b:
            raise ValueError("({}, {}) is not a valid transport map : it goes backwards in time".format(a, b))
    tmap_0 = tmap_model.get_coupling(*pairs_list.pop(0))
    while len(pairs_list) > 0:
        tmap_1 = tmap_model.get_coupling(*pairs_list.pop(0))
        tmap_0 = glue_transport_maps(tmap_0, tmap_1)
    return tmap_0


def find_path(t0, t1, available_pairs, timepoints):
    """Longest path of forward day pairs from t0 to t1 (:43-108)."""
    if t0 not in timepoints or t1 not in timepoints:
        raise ValueError("Unable to build path : t0 and t1 must be present in timepoints list")
    if available_pairs is None:
        t0_i = timepoints.index(t0)
        t1_i = timepoints.index(t1)
        return [(timepoints[i], timepoints[i + 1]) for i in range(t0_i, t1_i)]
    reach = {t: [] for t in timepoints}
    for a, b in available_pairs:
        reach[a].append(b)
    reach = {t: sorted(reach[t]) for t in timepoints}
    best = {t: (0, None) for t in timepoints}
    for t in timepoints[timepoints.index(t0):]:
        d, _ = best[t]
        for u in reach[t]:
            if d >= best[u][0]:
                best[u] = (d + 1, t)
    if best[t1][0] == 0:
        raise ValueError("{} is not reachable from {} with the chosen day_pairs".format(t1, t0))
    path = []
    cur = t1
    while cur != t0:
        path.insert(0, (best[cur][1], cur))
        cur = best[cur][1]
    return path
