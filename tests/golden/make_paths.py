"""Golden cases of the reference's day-pair path search (wot/tmap/chaining.py:43-108).

Loads the reference's chaining module by file path from a wot checkout (with a
stand-in for the ``wot`` package it imports at top level, which is not used by
``find_path``), runs ``find_path`` on seeded random sets of forward day pairs
and records, per case, the path it returns or the name of the exception it
raises, in ``tests/golden/find_path_cases.json``.

Usage (the tests only read the json):
    python tests/golden/make_paths.py /path/to/wot-checkout
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_find_path(root):
    stub = types.ModuleType('wot')
    stub.tmap = types.ModuleType('wot.tmap')
    sys.modules.setdefault('wot', stub)
    sys.modules.setdefault('wot.tmap', stub.tmap)
    spec = importlib.util.spec_from_file_location('ref_chaining', os.path.join(root, 'wot', 'tmap', 'chaining.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.find_path


def cases(n_cases=400, seed=0):
    rng = np.random.default_rng(seed)
    for _ in range(n_cases):
        n = int(rng.integers(2, 8))
        timepoints = sorted(float(v) for v in rng.choice(np.arange(0, 20), size=n, replace=False))
        all_pairs = [(a, b) for i, a in enumerate(timepoints) for b in timepoints[i + 1:]]
        keep = rng.random(len(all_pairs)) < rng.uniform(0.2, 0.8)
        pairs = [p for p, k in zip(all_pairs, keep) if k]
        rng.shuffle(pairs)
        if rng.random() < 0.85:        # mostly forward queries, some t1 <= t0
            i0, i1 = sorted(int(v) for v in rng.choice(n, size=2, replace=False))
        else:
            i0, i1 = int(rng.integers(0, n)), int(rng.integers(0, n))
        yield timepoints, [list(p) for p in pairs], timepoints[i0], timepoints[i1]


def main(root):
    find_path = load_find_path(root)
    out = []
    for timepoints, pairs, t0, t1 in cases():
        rec = {'timepoints': timepoints, 'pairs': pairs, 't0': t0, 't1': t1}
        try:
            rec['path'] = [list(p) for p in find_path(t0, t1, [tuple(p) for p in pairs], list(timepoints))]
        except Exception as e:  # noqa: BLE001  (the exception class is the recorded outcome)
            rec['error'] = type(e).__name__
        out.append(rec)
    with open(os.path.join(HERE, 'find_path_cases.json'), 'w') as f:
        json.dump(out, f, separators=(',', ':'))
    print('wrote %d cases: %d paths, errors %s' % (
        len(out), sum('path' in r for r in out),
        sorted({r['error'] for r in out if 'error' in r})))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_paths.py /path/to/wot-checkout')
    main(sys.argv[1])
