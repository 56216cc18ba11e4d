"""Full-size check of the single-pair workload against the NumPy oracle
(test infrastructure, run once on a GPU host; not part of the test suite).

On the 20,000 x 25,000 pair of the benchmark (same generator, seed and
coordinates), with growth_iters = 1 to bound the CPU time:

* times the NumPy oracle (the reference's solver restated in FP64 NumPy) on the
  whole pair on this host's cores: the measured CPU baseline;
* times the same oracle on 1000 x 1250 random cell subsamples (the benchmark's
  reference-arm sample) and extrapolates by I x J, to check the factor the
  reference arm uses;
* compares, entry by entry and in the marginals, the NumPy oracle's coupling
  with the FP64 torch restatement on the GPU (oracle/torch_ot.py, the checker
  the benchmark uses at full size) and with libwotg's solve in both forms.

    python oracle/fullsize_c1.py OUT.json
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def errors(T, R):
    mx = np.abs(R).max()
    keep = np.abs(R) >= 1e-6 * mx
    return {'coupling_max_rel_err': float(np.abs(T - R).max() / mx),
            'element_max_rel_err': float((np.abs(T[keep] - R[keep]) / np.abs(R[keep])).max()),
            'marginal_max_rel_err': float(max(np.abs(T.sum(1) - R.sum(1)).max() / np.abs(R.sum(1)).max(),
                                              np.abs(T.sum(0) - R.sum(0)).max() / np.abs(R.sum(0)).max()))}


def main(out_path):
    import torch
    import bench
    from oracle import ot_model as oom, optimal_transport as oot, torch_ot as tot
    from wot_gb300 import _build, _native
    from wot_gb300.ot import device as D
    _build.build()
    cfg = dict(bench.CFG, growth_iters=1)
    X, day, growth = bench.make_pair(1)
    a, b = bench.coords_on_device(X, day)
    G = growth[day == 0]
    a_h, b_h = a.double().cpu().numpy(), b.double().cpu().numpy()
    rec = {'shape': [a_h.shape[0], b_h.shape[0]], 'config': cfg, 'cpu_count': os.cpu_count(),
           'blas_threads': bench.blas_threads()}

    # the NumPy oracle on the whole pair (cost + median + solve), on the host's cores
    t0 = time.perf_counter()
    C = oom.compute_default_cost_matrix(a_h, b_h)
    t_cost = time.perf_counter() - t0
    st = {}
    t1 = time.perf_counter()
    R = oot.optimal_transport_duality_gap(C=C, G=G.copy(), stats=st, **cfg)
    t_solve = time.perf_counter() - t1
    rec['numpy_full'] = {'cost_s': t_cost, 'solve_s': t_solve, 'total_s': t_cost + t_solve,
                         'iterations': st['iterations'], 'absorptions': st['absorptions']}
    del C

    # the reference arm's sample and its extrapolation by I x J
    rng = np.random.default_rng(0)
    I_s, J_s = bench.REF_SAMPLE
    times, its = [], []
    for _ in range(3):
        t, it, _, _ = bench.cpu_sample(a_h, b_h, G, I_s, J_s, rng, cfg=cfg)
        times.append(t)
        its.append(it)
    scale = a_h.shape[0] * b_h.shape[0] / (I_s * J_s)
    ext = float(np.mean(times)) * scale
    rec['sample_extrapolation'] = {
        'sample': [I_s, J_s], 'sample_s': times, 'sample_iterations': its, 'extrapolated_total_s': ext,
        'measured_over_extrapolated': (t_cost + t_solve) / ext,
        'per_iteration_measured_over_extrapolated':
            (t_solve / st['iterations']) / (ext / float(np.mean(its)))}

    # the FP64 torch restatement on the GPU, and libwotg in both forms
    st_t = {}
    t2 = time.perf_counter()
    C64 = tot.default_cost(a.double(), b.double())
    Rt = tot.optimal_transport_duality_gap(C=C64, G=torch.as_tensor(G, device='cuda'), stats=st_t, **cfg)
    torch.cuda.synchronize()
    rec['torch_fp64'] = dict(errors(Rt.cpu().numpy(), R), seconds=time.perf_counter() - t2,
                             iterations=st_t['iterations'])
    del C64, Rt
    torch.cuda.empty_cache()
    for form in ('materialized', 'onthefly'):
        res = D.solve(D.default_cost(a, b), G, cfg, _native.SOLVER_DUALITY_GAP, form=form)
        rec['libwotg_' + form] = dict(errors(res.tmap.cpu().numpy(), R), iterations=res.stats['iterations'])
        del res
        torch.cuda.empty_cache()
    with open(out_path, 'w') as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python oracle/fullsize_c1.py OUT.json')
    main(sys.argv[1])
