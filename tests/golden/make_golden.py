"""Generate the golden fixtures of the transport-map path from the reference itself.

Runs the reference's own solver module (wot/ot/optimal_transport.py, NumPy
only) and ``compute_pca`` (wot/ot/util.py, scikit-learn) loaded by file path
from a wot checkout, on small seeded inputs, and stores inputs and outputs in
``tests/golden/*.npz``. It also converts the reference's orphan integer
transport-map fixtures (tests/inputs/transport_maps/*.csv) into
``chain_maps.npz``.

Usage (needs the wot sources and scikit-learn; the tests only read the npz):
    python tests/golden/make_golden.py /path/to/wot-checkout
"""
from __future__ import annotations

import csv
import importlib.util
import os
import sys
import types

import numpy as np

sys.dont_write_bytecode = True
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from wot_gb300 import synthetic  # noqa: E402

DEFAULTS = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_solver(ref, solver, C, G, params):
    cfg = dict(DEFAULTS)
    cfg.update(params)
    tmap, learned = ref.compute_transport_matrix(solver=solver, C=C, G=np.array(G, dtype=np.float64), **cfg)
    return tmap, np.array(learned)


def main(root):
    ref = _load('ref_optimal_transport', os.path.join(root, 'wot', 'ot', 'optimal_transport.py'))
    sys.modules.setdefault('ot', types.ModuleType('ot'))   # util.py imports POT at top level; unused here
    util = _load('ref_ot_util', os.path.join(root, 'wot', 'ot', 'util.py'))
    import sklearn.metrics

    # 1. the reference's known-answer test (tests/test_transport.py:11-33)
    C = np.array([[0, 100, 100], [100, 0, 100], [100, 100, 0]], dtype=np.float64)
    out = {'C': C, 'G': np.ones(3)}
    for tag, solver in (('dg', ref.optimal_transport_duality_gap), ('fi', ref.transport_stablev2)):
        t, lg = run_solver(ref, solver, C, np.ones(3), dict(epsilon=0.01, lambda1=1, lambda2=50))
        out['tmap_' + tag] = t
    np.savez_compressed(os.path.join(HERE, 'kat_3x3.npz'), **out)

    # 2. a small synthetic day pair: reference PCA + cost + both solvers
    X, day, growth = synthetic.time_course([120, 150], n_genes=1000, n_clusters=6, seed=0)
    m0, m1 = X[day == 0], X[day == 1]
    p0, p1, pca, _ = util.compute_pca(m0, m1, 30)
    S = np.diag(pca.singular_values_)
    x0, x1 = p0.dot(S), p1.dot(S)
    D = sklearn.metrics.pairwise.pairwise_distances(x0, x1, metric='sqeuclidean', n_jobs=1)
    med = np.median(D)
    C = D / med
    G = growth[day == 0]
    cases = {
        'dg_default': (ref.optimal_transport_duality_gap, {}),
        'dg_growth3': (ref.optimal_transport_duality_gap, dict(growth_iters=3)),
        'dg_eps01_lam10': (ref.optimal_transport_duality_gap, dict(epsilon=0.01, lambda1=10)),
        'dg_eps1_lam01': (ref.optimal_transport_duality_gap, dict(epsilon=0.1, lambda1=0.1)),
        'dg_tau10': (ref.optimal_transport_duality_gap, dict(tau=10.0)),
        'dg_maxiter': (ref.optimal_transport_duality_gap, dict(max_iter=37)),
        'dg_batch3_tol1e6': (ref.optimal_transport_duality_gap, dict(batch_size=3, tolerance=1e-6)),
        'fi_short': (ref.transport_stablev2, dict(scaling_iter=300, inner_iter_max=50, extra_iter=100)),
        'fi_tau10': (ref.transport_stablev2, dict(scaling_iter=200, inner_iter_max=30, extra_iter=50, tau=10.0)),
        'fi_growth2': (ref.transport_stablev2, dict(scaling_iter=150, inner_iter_max=50, extra_iter=50,
                                                   growth_iters=2)),
    }
    out = {'X': X, 'day': day, 'growth': growth, 'x0': x0, 'x1': x1, 'pca_components_0': p0,
           'pca_components_1': p1, 'singular_values': pca.singular_values_, 'median': np.array(med),
           'C': C, 'G': G}
    for name, (solver, params) in cases.items():
        import logging
        logging.disable(logging.WARNING)
        t, lg = run_solver(ref, solver, C, G, params)
        logging.disable(logging.NOTSET)
        out['tmap_' + name] = t
        out['learned_' + name] = lg
        out['params_' + name] = np.array(repr(params))
    np.savez_compressed(os.path.join(HERE, 'pair_120x150.npz'), **out)

    # 3. the reference's integer transport-map fixtures
    out = {}
    for name in ('t0_t1', 't1_t2', 't2_t3', 't3_t4'):
        with open(os.path.join(root, 'tests', 'inputs', 'transport_maps', name + '.csv')) as f:
            rows = list(csv.reader(f))
        out[name + '_X'] = np.array([[float(v) for v in r[1:]] for r in rows[1:]])
        out[name + '_obs'] = np.array([r[0] for r in rows[1:]])
        out[name + '_var'] = np.array(rows[0][1:])
    np.savez_compressed(os.path.join(HERE, 'chain_maps.npz'), **out)
    print('wrote', sorted(f for f in os.listdir(HERE) if f.endswith('.npz')))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden.py /path/to/wot-checkout')
    main(sys.argv[1])
