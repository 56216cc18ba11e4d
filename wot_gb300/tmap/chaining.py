"""Long-range couplings through a chain of day-pair maps (wot/tmap/chaining.py:4-108).

A coupling from day t0 to a later day t1 that no single map covers is the
product of the maps along a chain of day pairs t0 = d_0 < d_1 < ... < d_k = t1.
``find_path`` picks the chain, ``chain_transport_maps`` multiplies along it.
"""
from __future__ import annotations

from .util import glue_transport_maps


def chain_transport_maps(tmap_model, pairs_list):
    """The coupling along ``pairs_list`` (consecutive day pairs, each going
    forward in time), as the product of the models' couplings (:4-40).

    Raises the reference's ValueErrors for a list whose pairs do not link up
    and for a pair that goes backwards; ``pairs_list`` is consumed, as the
    reference consumes it."""
    for (_, end), (start, _) in zip(pairs_list[:-1], pairs_list[1:]):
        if end != start:
            raise ValueError("Transport maps cannot be glued together : invalid path")
    for a, b in pairs_list:
        if not a < b:
            raise ValueError("({}, {}) is not a valid transport map : it goes backwards in time".format(a, b))
    coupling = tmap_model.get_coupling(*pairs_list.pop(0))
    while pairs_list:
        coupling = glue_transport_maps(coupling, tmap_model.get_coupling(*pairs_list.pop(0)))
    return coupling


def find_path(t0, t1, available_pairs, timepoints):
    """The day pairs to chain from t0 to t1 (:43-108).

    Without a pair list: every consecutive pair of ``timepoints`` from t0 to t1.
    With one: the chain through the most days, i.e. the longest chain of
    available forward pairs (a < b) that starts at t0 and ends at t1. The days
    are taken in increasing order, which orders the chains topologically, and
    every day's successors in increasing order; a chain into a day replaces the
    one found before only when it is strictly longer, so of two chains of the
    same length the one through the earlier predecessor day is kept (the
    reference's tie rule, which decides which maps get multiplied).

    Wherever the reference returns a path this returns the same one. The
    reference also lets chains that start at days it cannot reach from t0 take
    part in the search and then fails with a KeyError when such a chain is the
    longest into t1; here only chains from t0 count, so those cases get the
    longest chain from t0 instead. Pairs that do not go forward in time are
    never part of a chain.
    """
    if t0 not in timepoints or t1 not in timepoints:
        raise ValueError("Unable to build path : t0 and t1 must be present in timepoints list")
    if available_pairs is None:
        lo, hi = timepoints.index(t0), timepoints.index(t1)
        return list(zip(timepoints[lo:hi], timepoints[lo + 1:hi + 1]))

    successors = {day: [] for day in timepoints}
    for a, b in available_pairs:
        if a < b:
            successors[a].append(b)
    # longest[day]: edges of the longest chain from t0 to day; previous[day]: the day before it
    longest, previous = {t0: 0}, {}
    for day in timepoints[timepoints.index(t0):]:
        if day not in longest:
            continue                      # no chain from t0 reaches this day
        for nxt in sorted(successors[day]):
            if longest[day] + 1 > longest.get(nxt, 0):
                longest[nxt] = longest[day] + 1
                previous[nxt] = day
    if longest.get(t1, 0) == 0:
        raise ValueError("{} is not reachable from {} with the chosen day_pairs".format(t1, t0))
    path = []
    day = t1
    while day != t0:
        path.append((previous[day], day))
        day = previous[day]
    return path[::-1]
