"""Benchmark of the transport-map hot path on one GB300 (or N replicas).

Workload (one "step" = one transport map): the single-day-pair configuration,
20,000 x 25,000 synthetic cells, 1,000 genes, 20 clusters, local PCA 30,
default wot parameters (epsilon 0.05, lambda1 1, lambda2 50, epsilon0 1,
tau 1e4, tolerance 1e-8, duality-gap solver) and growth_iters = 3. A step runs
the cost kernel, the exact FP32 median, three full duality-gap solves and the
dense FP64 coupling, on device-resident coordinates (value), and the whole
OTModel.compute_transport_map call on host data (e2e).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0). Under torchrun each rank solves its own pair
(seed + rank): weak scaling with no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "OT maps/sec @≤1e-4 coupling err, batched vs plain, 1×GB300; Sinkhorn iter/s"
CFG = dict(growth_iters=3, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
           inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)
I_FULL, J_FULL, GENES, CLUSTERS, PCA_D = 20000, 25000, 1000, 20, 30
SAMPLE = (2000, 2500)          # bounded CPU sample of the same cells
REF_SAMPLE = (1000, 1250)      # per-step sample of the reference arm
WORKLOAD = ('single day pair 20000x25000 cells, 1000 genes, 20 clusters, local_pca=30, growth_iters=3, '
            'duality-gap solver, eps=0.05 lambda1=1 lambda2=50 eps0=1 tau=1e4 tol=1e-8')


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--pair', default=None, help='I,J cells of a smaller pair (profiling runs)')
    ap.add_argument('--pca', type=int, default=None, help='local PCA dimension of the pair workload (profiling runs)')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-parity', action='store_true', help='skip the full-size FP64 parity checks')
    ap.add_argument('--workload', default='pair', choices=['pair', 'course', 'chain', 'adjoint'],
                    help="pair: one 20000x25000 map per step; course: the batched 41-day time course x "
                         "5x5 epsilon/lambda1 sweep (1000 maps) per step; chain: the 60000x60000 map and "
                         "the 20-map chain; adjoint: objective + gradient of a 10000x12000 pair")
    ap.add_argument('--course-days', type=int, default=41)
    ap.add_argument('--no-extra', action='store_true',
                    help='pair workload only: skip the batched-course and chain summaries of the JSON line')
    ap.add_argument('--form', default='auto', choices=['materialized', 'onthefly', 'auto'],
                    help='materialised FP32 cost stream or tensor-core cost recomputation')
    return ap.parse_args()


def dist_env():
    return int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1)), int(os.environ.get('LOCAL_RANK', 0))


def exp2_peak():
    """Measured exp2 throughput of this GPU (the half-steps' per-element ceiling)."""
    import ctypes
    import torch
    from wot_gb300 import _native
    r = ctypes.c_double(0.0)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if _native.load().wotg_exp2_rate(ctypes.byref(r), st) != 0:
        return None
    return r.value


def peaks():
    """(HBM GB/s, dense bf16 TFLOP/s, 'measured' | 'fallback')."""
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), float(p['bf16_tflops']), 'measured'
    except Exception:
        return 6800.0, 1900.0, 'fallback'


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ''
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in getattr(self, 'lines', []):
            f = [x.strip() for x in ln.split(',')]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                for k, n in enumerate(names):
                    if f[5 + k].lower().startswith('active'):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': mx, 'reasons': sorted(reasons),
                'samples': len(sm)}


def make_pair(seed, I=None, J=None):
    from wot_gb300 import synthetic
    X, day, growth = synthetic.time_course([I or I_FULL, J or J_FULL], n_genes=GENES, n_clusters=CLUSTERS,
                                           seed=seed)
    return X, day, growth


def coords_on_device(X, day):
    from wot_gb300.ot.util import compute_pca
    x0, x1, s, _ = compute_pca(X[day == 0], X[day == 1], PCA_D)
    return (x0 * s).float().contiguous(), (x1 * s).float().contiguous()


def cpu_sample(a, b, G, I_s, J_s, rng, stages=None, cfg=None):
    """Oracle (FP64 NumPy restatement) on a random cell subsample; returns
    (seconds, iterations, coupling, (a_s, b_s, G_s)). With ``stages`` (a dict),
    also the split of those seconds into cost and solve, and the subsampled
    rows ('rows': (ri, rj)). ``cfg`` replaces the benchmark's solver
    parameters."""
    from oracle import ot_model as oom, optimal_transport as oot
    ri = np.sort(rng.choice(a.shape[0], I_s, replace=False))
    rj = np.sort(rng.choice(b.shape[0], J_s, replace=False))
    a_s, b_s, G_s = a[ri].astype(np.float64), b[rj].astype(np.float64), G[ri]
    t0 = time.perf_counter()
    C = oom.compute_default_cost_matrix(a_s, b_s)
    if stages is not None:
        stages['cost'] = time.perf_counter() - t0
        stages['rows'] = (ri, rj)
    iters = [0]

    def counting(**kw):
        st = {}
        out = oot.optimal_transport_duality_gap(stats=st, **kw)
        iters[0] += st['iterations']
        return out

    t1 = time.perf_counter()
    T, _ = oot.compute_transport_matrix(solver=counting, C=C, G=G_s.copy(), **(CFG if cfg is None else cfg))
    if stages is not None:
        stages['solve'] = time.perf_counter() - t1
    return time.perf_counter() - t0, iters[0], T, (a_s, b_s, G_s)


def dev_errors(T, R, block=4096):
    """Parity of a device coupling T with the FP64 reference R (torch tensors):
    max|T - R| / max|R|; max |T - R| / |R| over the entries |R| >= 1e-6 max|R|;
    the row and column marginals' max |r - r_ref| / max r_ref. Row blocks keep
    the temporaries small for 60000 x 60000 maps."""
    import torch
    mx = float(R.abs().max())
    ce = ee = 0.0
    for r0 in range(0, R.shape[0], block):
        Rb, Tb = R[r0:r0 + block], T[r0:r0 + block].to(torch.float64)
        d = (Tb - Rb).abs()
        ce = max(ce, float(d.max()) / mx)
        keep = Rb.abs() >= 1e-6 * mx
        if bool(keep.any()):
            ee = max(ee, float((d[keep] / Rb.abs()[keep]).max()))
    rr, rc = R.sum(1), R.sum(0)
    me = max(float((T.sum(1) - rr).abs().max() / rr.abs().max()), float((T.sum(0) - rc).abs().max() / rc.abs().max()))
    return {'coupling_max_rel_err': ce, 'element_max_rel_err': ee, 'marginal_max_rel_err': me}


def fp64_reference(a, b, G, cfg):
    """The reference's solver in FP64 on the GPU (oracle/torch_ot.py, the same
    arithmetic as the NumPy oracle) on the cost of the FP32 coordinates a, b:
    returns (coupling, iterations, seconds)."""
    import torch
    from oracle import torch_ot as tot
    t0 = time.perf_counter()
    C64 = tot.default_cost(a.double(), b.double())
    its = [0]

    def counting(**kw):
        st = {}
        out = tot.optimal_transport_duality_gap(stats=st, **kw)
        its[0] += st['iterations']
        return out

    R, _ = tot.compute_transport_matrix(solver=counting, C=C64, G=torch.as_tensor(G, device='cuda').double(),
                                        **dict(cfg))
    del C64
    torch.cuda.synchronize()
    return R, its[0], time.perf_counter() - t0


def blas_threads():
    for k in ('OPENBLAS_NUM_THREADS', 'OMP_NUM_THREADS', 'MKL_NUM_THREADS'):
        if os.environ.get(k):
            return int(os.environ[k])
    return os.cpu_count() or 1


# The oracle's whole 20000 x 25000 solve, timed once on the GPU host's 16 cores with growth_iters = 1
# (oracle/fullsize_c1.py): too long for a bench step.
CPU_FULL_SIZE = {'growth_iters': 1, 'iterations': 450, 'cost_s': 5.83, 'solve_s': 250.6, 'total_s': 256.4,
                 'cores': 16, 'per_iteration_vs_sample_extrapolation': 1.38}


def run_reference(args):
    """Reference arm: the reference's CPU algorithm (the oracle port; the
    reference itself is not available on the GPU host) on bounded samples of
    the same workload, extrapolated to the full pair by I*J*iterations."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    X, day, growth = make_pair(1)
    from oracle import ot_model as oom
    x0, x1, s, _ = oom.compute_pca(X[day == 0], X[day == 1], PCA_D)
    a, b, G = x0 * s, x1 * s, growth[day == 0]
    rng = np.random.default_rng(0)
    I_s, J_s = REF_SAMPLE
    times, its = [], []
    for k in range(args.warmup + args.steps):
        t, it, _, _ = cpu_sample(a, b, G, I_s, J_s, rng)
        if k >= args.warmup:
            times.append(t)
            its.append(it)
    t_step = float(np.mean(times))
    it_s = float(np.mean(its))
    scale = (I_FULL * J_FULL) / (I_s * J_s)
    # maps/s at full size from the sample's time scaled by I*J. The oracle's whole-pair solve, timed
    # once on the same host's 16 cores, spent 1.38x more time per Sinkhorn iteration than this
    # extrapolation assumes (its iterates no longer fit the caches): the value is an upper bound on
    # the CPU's throughput (the whole-pair run is in the line as cpu_full_size_measured).
    value = 1.0 / (t_step * scale)
    sample = ('%dx%d random cell subsample of the 20000x25000 pair per step (own median), full FP64 oracle '
              'duality-gap solve x3 growth iterations (%.0f iterations); ms_per_step is the measured time of '
              'one such step, value its maps/s extrapolated to the whole pair by I*J' % (I_s, J_s, it_s))
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'maps/s', 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t_step * 1e3,
            'ms_per_map_extrapolated': t_step * scale * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': WORKLOAD, 'I': I_FULL, 'J': J_FULL, 'd': PCA_D},
            'sinkhorn_iter_per_s': it_s / t_step * (I_s * J_s) / (I_FULL * J_FULL),
            'cpu_full_size_measured': CPU_FULL_SIZE,
            'cpu_baseline': {'value': value, 'unit': 'maps/s', 'cores': blas_threads(), 'kind': 'port',
                             'sample': sample},
            'e2e': {'value': value, 'unit': 'maps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)



COURSE_EPS = (0.01, 0.025, 0.05, 0.075, 0.1)
COURSE_L1 = (0.1, 0.3, 1, 3, 10)
COURSE_CFG = dict(growth_iters=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000, inner_iter_max=50,
                  tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


def course_items(n_days):
    """The course's day sizes, pair shapes and items (pair, parameters): every
    consecutive pair x the epsilon x lambda1 grid."""
    from wot_gb300 import synthetic
    sizes = synthetic.log_uniform_day_sizes(n_days, 1000, 30000, seed=2)
    shapes = [(int(sizes[t]), int(sizes[t + 1])) for t in range(n_days - 1)]
    items = [(p, dict(COURSE_CFG, epsilon=e, lambda1=l)) for p in range(n_days - 1) for e in COURSE_EPS
             for l in COURSE_L1]
    return sizes, shapes, items


def course_days(n_days, seed=0, needed=None):
    """Per-day cells of the long synthetic time course (day sizes log-uniform in
    [1000, 30000]), generated in a spawn process pool before any CUDA call;
    with ``needed`` (day indices), only those days (the others are None)."""
    import multiprocessing as mp
    from wot_gb300 import synthetic
    sizes = synthetic.log_uniform_day_sizes(n_days, 1000, 30000, seed=2)
    prof = synthetic.course_profiles(n_days, GENES, CLUSTERS, seed)
    want = sorted(set(range(n_days)) if needed is None else set(needed))
    with mp.get_context('spawn').Pool(max(1, min(16, os.cpu_count() or 1, len(want)))) as pool:
        made = pool.starmap(synthetic.course_day, [(prof, t, int(sizes[t])) for t in want])
    days = [None] * n_days
    for t, d in zip(want, made):
        days[t] = d
    return sizes, days


def run_course_sharded(args, days_data, rank, world, pg):
    """The course under torchrun: the items split over the ranks by estimated
    work (wot_gb300.ot.shard), each rank building the costs of only its own
    pairs and solving its items in one wotg_solve_batched call per step; the
    job's time is the slowest rank's. Strong scaling: the whole course (1000
    maps) is the work at every rank count."""
    import torch
    from wot_gb300 import _build, _native
    from wot_gb300.ot import batch as Bt, device as D, shard
    from wot_gb300.ot.util import compute_pca
    import logging
    logging.disable(logging.WARNING)
    _build.build()
    lib = _native.load()
    sizes, days = days_data
    _, shapes, items = course_items(len(days))
    mine = shard.my_items(shapes, items, rank, world)
    used = sorted({items[k][0] for k in mine})
    local = {p: i for i, p in enumerate(used)}
    pairs = []
    for t in used:
        x0, x1, sv, _ = compute_pca(days[t][0], days[t + 1][0], PCA_D)
        cost = D.default_cost((x0 * sv).float().contiguous(), (x1 * sv).float().contiguous())
        pairs.append(Bt.prepare_pair(cost, days[t][1]))
    my = [(local[items[k][0]], items[k][1]) for k in mine]
    for _ in range(args.warmup):
        maps = Bt.solve_batched(pairs, my)
    torch.cuda.synchronize()
    pg.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    n_launch0 = lib.wotg_launch_count()
    with Clocks(dist_env()[2]) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            maps = Bt.solve_batched(pairs, my)
        ev1.record(stream)
        torch.cuda.synchronize()
    t = shard.max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / args.steps)
    its = shard.gather([(k, int(m.stats['iterations'])) for k, m in zip(mine, maps)])
    if rank != 0:
        return None
    return {'metric': METRIC, 'value': len(items) / t, 'unit': 'maps/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t * 1e3, 'higher_is_better': True, 'scaling': 'strong',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': 'batched time course: %d days (log-uniform 1000-30000 cells), %d pairs x eps %s '
                                   'x lambda1 %s, items split over %d ranks by estimated work'
                                   % (len(days), len(shapes), list(COURSE_EPS), list(COURSE_L1), world),
                       'pairs': len(shapes), 'items': len(items), 'parallelism': 'item shards x %d' % world,
                       'timed': 'each rank: one wotg_solve_batched call over its items, costs resident; '
                                'max over ranks'},
            'sinkhorn_iter_per_s': float(sum(i for _, i in its)) / t,
            'gpu_launches': int(lib.wotg_launch_count() - n_launch0), 'clocks': clk.summary(), 'e2e': None}


def run_course(args, days_data):
    """The batched workload: every consecutive day pair x the 5 x 5 epsilon x
    lambda1 grid in one wotg_solve_batched call per step; the plain driver on
    the items of a stratified subset of pairs (and the batched solver on the same
    subset) for the batched-vs-plain ratio."""
    import torch
    from wot_gb300 import _build, _native
    from wot_gb300.ot import batch as Bt, device as D
    from wot_gb300.ot.util import compute_pca
    import logging
    logging.disable(logging.WARNING)
    _build.build()
    lib = _native.load()
    sizes, days = days_data
    npairs = len(days) - 1
    pairs, pts = [], []
    for t in range(npairs):
        x0, x1, sv, _ = compute_pca(days[t][0], days[t + 1][0], PCA_D)
        a, b = (x0 * sv).float().contiguous(), (x1 * sv).float().contiguous()
        cost = D.default_cost(a, b)
        pairs.append(Bt.prepare_pair(cost, days[t][1]))   # G = growth ** (t1 - t0), t1 - t0 = 1
        pts.append((a, b))
    _, _, items = course_items(len(days))
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        maps = Bt.solve_batched(pairs, items)
    torch.cuda.synchronize()
    n_launch0 = lib.wotg_launch_count()
    with Clocks(0) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            maps = Bt.solve_batched(pairs, items)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.wotg_launch_count() - n_launch0
    t = ev0.elapsed_time(ev1) / 1e3 / args.steps
    # the dominant kernel: one batched pass over every item of every pair, as this batch's autotuner
    # timed it with CUDA events for the configuration it chose (row direction: rows of C)
    import ctypes
    ms_r, ms_c = ctypes.c_float(0.0), ctypes.c_float(0.0)
    kgrw = (ctypes.c_int32 * 4)()
    _native.check(lib.wotg_batch_pass_timing(ctypes.byref(ms_r), ctypes.byref(ms_c), kgrw), 'wotg_batch_pass_timing')
    its = np.array([m.stats['iterations'] for m in maps], dtype=np.float64)
    ij = np.array([m.shape[0] * m.shape[1] for m in maps], dtype=np.float64)
    work = float(np.sum(its * ij * 2))

    # plain driver, item by item, on a stratified subset of pairs (by I*J)
    order = np.argsort([p.cost.I * p.cost.J for p in pairs])
    subset = sorted({int(order[int(q * (npairs - 1))]) for q in (0.1, 0.35, 0.6, 0.85)})
    sub_items = [(subset.index(p), c) for p, c in items if p in subset]
    sub_pairs = [pairs[p] for p in subset]
    Bt.solve_batched(sub_pairs, sub_items)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sub_maps = Bt.solve_batched(sub_pairs, sub_items)
    torch.cuda.synchronize()
    t_sub_batched = time.perf_counter() - t0
    t_plain = {}
    for form in ('auto', 'materialized', 'onthefly'):
        D.solve(sub_pairs[0].cost, sub_pairs[0].G, sub_items[0][1], 0, want_tmap=False, want_potentials=True,
                form=form)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for p, c in sub_items:
            D.solve(sub_pairs[p].cost, sub_pairs[p].G, c, 0, want_tmap=False, want_potentials=True, form=form)
        torch.cuda.synchronize()
        t_plain[form] = time.perf_counter() - t0
    w_sub = float(sum(m.stats['iterations'] * m.shape[0] * m.shape[1] for m in sub_maps))
    w_all = float(np.sum(its * ij))
    best_plain = min(t_plain.values())

    hbm_peak, tf_peak, peak_kind = peaks()
    elems = float(sum(pairs[p].cost.I * pairs[p].cost.J for p, _ in items))
    pass_bytes = float(sum(4 * p.cost.I * p.cost.J for p in pairs))
    exp_pk = exp2_peak()
    t_pass = ms_r.value * 1e-3
    roofline = {'bound': 'hbm', 'achieved': pass_bytes / t_pass / 1e9, 'peak': hbm_peak, 'unit': 'GB/s',
                'frac': pass_bytes / t_pass / 1e9 / hbm_peak, 'traffic': None,
                'kernel': 'pass_kernel<%d,%d,speculative> (rows of C)' % (kgrw[0], kgrw[1]), 'peak_kind': peak_kind,
                'launch_ms': ms_r.value, 'col_launch_ms': ms_c.value,
                'col_kernel': 'pass_kernel<%d,%d,speculative> (rows of CT)' % (kgrw[2], kgrw[3]),
                'element_evaluations_per_launch': elems,
                'element_evaluations_per_s': elems / t_pass, 'exp2_peak_per_s': exp_pk,
                'exp2_frac': (elems / t_pass / exp_pk) if exp_pk else None,
                'note': 'one launch evaluates every item of every pair against the pair\'s cost, read once for '
                        'all its items (the algorithmic bytes); the bound is the one exp2 per element '
                        'evaluation (exp2_frac), not HBM'}
    line = {'metric': METRIC, 'value': len(items) / t, 'unit': 'maps/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': 'batched time course: %d days (log-uniform 1000-30000 cells, 1000 genes, '
                                   '20 clusters, local_pca=30), %d consecutive pairs x eps %s x lambda1 %s, '
                                   'lambda2=50, duality-gap solver; maps returned as potentials'
                                   % (len(days), npairs, list(COURSE_EPS), list(COURSE_L1)),
                       'pairs': npairs, 'items': len(items), 'cells': [int(n) for n in sizes],
                       'l2': 'inputs larger than L2 (FP32 costs and transposes %.1f GB)'
                             % (sum(p.cost.I * p.cost.ldc + p.cost.J * p.CT.stride(0) for p in pairs) * 4 / 1e9),
                       'timed': 'one wotg_solve_batched call over all items, costs resident'},
            'sinkhorn_iter_per_s': float(np.sum(its)) / t, 'iterations_per_map': float(np.mean(its)),
            'max_iterations': int(its.max()),
            'element_evaluations_per_s': work / t,
            'exp2_peak_per_s': exp2_peak(),
            'batched_vs_plain': {
                'subset_pairs': subset, 'subset_items': len(sub_items),
                'batched_s': t_sub_batched, 'plain_auto_s': t_plain['auto'],
                'plain_materialized_s': t_plain['materialized'], 'plain_onthefly_s': t_plain['onthefly'],
                'ratio_vs_best_plain': best_plain / t_sub_batched,
                'plain_maps_per_s_extrapolated': len(items) / (best_plain * w_all / w_sub),
                'ratio_full_extrapolated': (best_plain * w_all / w_sub) / t,
                'note': 'plain = wotg_compute_transport_matrix per item (potentials out), the fastest of the '
                        'auto, on-the-fly and materialised forms over the subset; full-course plain time '
                        'extrapolated from the subset by sum(iterations * I * J)'},
            'gpu_launches': int(launches), 'clocks': clk.summary(), 'peaks': {'kind': peak_kind},
            'roofline': roofline}
    if not args.no_cpu:
        # parity and CPU baseline: the oracle on items of the smallest pair
        from oracle import ot_model as oom, optimal_transport as oot
        p = int(order[0])
        a, b = (x.double().cpu().numpy() for x in pts[p])
        C = oom.compute_default_cost_matrix(a, b)
        G = days[p][1]
        errs, t_cpu, w_cpu = [], 0.0, 0.0
        checks = ((0.05, 1), (0.1, 10)) if getattr(args, 'quick', False) else ((0.01, 0.1), (0.05, 1), (0.1, 10))
        for e, l in checks:
            k = items.index((p, dict(COURSE_CFG, epsilon=e, lambda1=l)))
            st = {}
            t0 = time.perf_counter()
            R = oot.optimal_transport_duality_gap(C=C, G=G.copy(), stats=st, **dict(COURSE_CFG, epsilon=e, lambda1=l))
            t_cpu += time.perf_counter() - t0
            w_cpu += st['iterations'] * C.shape[0] * C.shape[1]
            T = maps[k].dense().cpu().numpy()
            errs.append({'eps': e, 'lambda1': l, 'coupling_max_rel_err': float(np.abs(T - R).max() / np.abs(R).max()),
                         'row_marginal_max_rel_err': float(np.abs(T.sum(1) - R.sum(1)).max() / np.abs(R.sum(1)).max()),
                         'col_marginal_max_rel_err': float(np.abs(T.sum(0) - R.sum(0)).max() / np.abs(R.sum(0)).max()),
                         'iterations_gpu': int(maps[k].stats['iterations']), 'iterations_oracle': int(st['iterations'])})
        line['parity_sample'] = {'pair': p, 'shape': list(C.shape), 'items': errs}
        cpu_value = len(items) / (t_cpu * w_all / w_cpu)
        line['cpu_baseline'] = {'value': cpu_value, 'unit': 'maps/s', 'cores': blas_threads(), 'kind': 'port',
                                'sample': 'oracle FP64 solves of %d items of the smallest pair (%dx%d, %.1f s); '
                                          'extrapolated to all items by sum(iterations * I * J)'
                                          % (len(checks), C.shape[0], C.shape[1], t_cpu)}
    if not getattr(args, 'no_parity', False):
        # FP64 reference parity (the reference's solver restated in FP64 on the GPU): every pair at
        # eps 0.05 / lambda1 1, and the whole eps x lambda1 grid on the three smallest pairs
        smallest = [int(p) for p in order[:3]]
        checks = [(p, 0.05, 1) for p in range(npairs)]
        checks += [(p, e, l) for p in smallest for e in COURSE_EPS for l in COURSE_L1 if (e, l) != (0.05, 1)]
        recs = []
        t0 = time.perf_counter()
        for p, e, l in checks:
            cfg = dict(COURSE_CFG, epsilon=e, lambda1=l)
            k = items.index((p, cfg))
            R, it_ref, _ = fp64_reference(pts[p][0], pts[p][1], days[p][1], cfg)
            T = maps[k].dense()
            r = dev_errors(T, R)
            del R, T
            r.update(pair=p, shape=[int(pairs[p].cost.I), int(pairs[p].cost.J)], eps=e, lambda1=l,
                     iterations_gpu=int(maps[k].stats['iterations']), iterations_oracle=int(it_ref))
            recs.append(r)
        torch.cuda.empty_cache()
        keys = ('coupling_max_rel_err', 'element_max_rel_err', 'marginal_max_rel_err')
        line['parity_full'] = {
            'oracle': 'the reference solver restated in FP64 on the GPU (oracle/torch_ot.py), same coordinates',
            'items': len(recs), 'pairs_at_eps0.05_lambda1_1': npairs, 'full_grid_pairs': smallest,
            'max': {k: max(r[k] for r in recs) for k in keys},
            'iterations_equal': sum(r['iterations_gpu'] == r['iterations_oracle'] for r in recs),
            'iterations_max_abs_diff': max(abs(r['iterations_gpu'] - r['iterations_oracle']) for r in recs),
            'worst_marginal': sorted(recs, key=lambda r: -r['marginal_max_rel_err'])[:3],
            'seconds': time.perf_counter() - t0}
    line['e2e'] = course_e2e(days, sizes) if not getattr(args, 'no_e2e', False) else None
    return line


def course_e2e(days, sizes):
    """The course through the public API on host data: a Dataset of every day's
    expression (host FP32), OTModel(...).compute_transport_maps_batched over
    the consecutive pairs x the 5 x 5 sweep (device PCA, cost and median per
    pair, the batched solve), then every map's potentials read back to the
    host. One timed call."""
    import torch
    import wot_gb300 as wot
    X = np.vstack([d[0] for d in days])
    day = np.concatenate([np.full(len(d[0]), float(t)) for t, d in enumerate(days)])
    growth = np.concatenate([d[1] for d in days])
    ds = wot.Dataset(X, wot.Frame({'day': day, 'cell_growth_rate': growth}, index=np.arange(len(day)).astype(str)))
    sweep = [{'epsilon': e, 'lambda1': l} for e in COURSE_EPS for l in COURSE_L1]
    model = wot.OTModel(ds, growth_iters=1, local_pca=PCA_D)

    def call():
        maps = model.compute_transport_maps_batched(sweep=sweep)
        host = {k: (m.u_bar.cpu().numpy(), m.v_bar.cpu().numpy()) for k, m in maps.items()}
        return maps, host

    # one timed call (the kernels and the batch's autotuning are warm from the device-resident runs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    maps, host = call()
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    d2h = int(sum(u.nbytes + v.nbytes for u, v in host.values()))
    return {'value': len(maps) / t, 'unit': 'maps/s', 'seconds': t,
            'h2d_bytes_per_step': int(X.nbytes + growth.nbytes), 'd2h_bytes_per_step': d2h,
            'api': 'wot_gb300.OTModel(Dataset of %d days).compute_transport_maps_batched(sweep of 25) '
                   '(device PCA + cost per pair + batched solve; potentials to host)' % len(days)}


CHAIN_CFG = dict(growth_iters=1, epsilon=0.05, lambda1=1, lambda2=50, epsilon0=1, tau=10000, scaling_iter=3000,
                 inner_iter_max=50, tolerance=1e-8, max_iter=1e7, batch_size=5, extra_iter=1000)


def chain_days(big=60000, n_chain=21, lo=20000, hi=60000, seed=4):
    """Cells of the large pair (two days of `big` cells) and of a chain of
    n_chain days with log-uniform sizes in [lo, hi], 1000 genes, 20 clusters."""
    import multiprocessing as mp
    from wot_gb300 import synthetic
    sizes = [big, big] + [int(n) for n in synthetic.log_uniform_day_sizes(n_chain, lo, hi, seed=seed)]
    prof = synthetic.course_profiles(len(sizes), GENES, CLUSTERS, seed)
    with mp.get_context('spawn').Pool(min(16, os.cpu_count() or 1)) as pool:
        days = pool.starmap(synthetic.course_day, [(prof, t, n) for t, n in enumerate(sizes)])
    return sizes, days


def run_adjoint(args, data=None):
    """The gradient workload: the converged unbalanced OT objective of a
    10000 x 12000 pair of 30-d points (10-component mixture, log g ~ N(0, 0.3^2),
    eps 0.05, lambda1 1, lambda2 50) and its gradient with respect to both point
    sets and log g, through wot_gb300.ot.adjoint.ot_objective (duality-gap solve,
    400 refinement iterations at the final epsilon, one adjoint pass per side)."""
    import torch
    from wot_gb300 import _native, synthetic
    from wot_gb300.ot import device as D
    from wot_gb300.ot.adjoint import ot_objective
    lib = _native.load()
    I, J, d = 10000, 12000, 30
    x = torch.tensor(synthetic.gaussian_mixture_points(I, d=d, n_components=10, seed=31), device='cuda')
    y = torch.tensor(synthetic.gaussian_mixture_points(J, d=d, n_components=10, seed=32), device='cuda')
    lg = torch.tensor(np.random.default_rng(33).normal(0.0, 0.3, I), device='cuda')
    c = D.cost_from_points(x.float(), y.float())
    scale = 1.0 / D.median(c)
    del c

    def step():
        xt, yt, lt = (t.clone().requires_grad_(True) for t in (x, y, lg))
        obj = ot_objective(xt, yt, lt, epsilon=0.05, lambda1=1.0, lambda2=50.0, cost_scale=scale)
        obj.backward()
        return obj, xt.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    n_launch0 = lib.wotg_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        obj, gx = step()
    ev1.record()
    torch.cuda.synchronize()
    t = ev0.elapsed_time(ev1) / 1e3
    return {'value': args.steps / t, 'unit': 'objective+gradient/s', 'ms_per_step': t / args.steps * 1e3,
            'steps': args.steps, 'warmup': args.warmup, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': 'unbalanced OT objective and its gradient w.r.t. x, y, log g: 10000 x 12000 '
                                   '30-d mixture points, eps 0.05, lambda1 1, lambda2 50, duality-gap solve + '
                                   '400 refinement iterations + adjoint', 'I': I, 'J': J, 'd': d},
            'objective': float(obj), 'grad_x_abs_sum': float(gx.abs().sum()),
            'gpu_launches': int(lib.wotg_launch_count() - n_launch0)}


def run_chain(args, data):
    """The large-pair workload: one 60000 x 60000 map in 50-d local PCA on the
    on-the-fly form, then 20 maps of 20000-60000 cells held as potentials and a
    pull-back of 8 cell-set indicator vectors through all of them."""
    import torch
    import wot_gb300 as wot
    from wot_gb300 import _build, _native, Population
    from wot_gb300.ot import device as D
    from wot_gb300.ot.implicit import ImplicitCoupling
    from wot_gb300.ot.util import compute_pca
    import logging
    logging.disable(logging.WARNING)
    _build.build()
    lib = _native.load()
    sizes, days = data
    d50 = 50
    x0, x1, sv, _ = compute_pca(days[0][0], days[1][0], d50)
    a, b = (x0 * sv).float().contiguous(), (x1 * sv).float().contiguous()
    G = torch.as_tensor(days[0][1], device='cuda')
    stream = torch.cuda.current_stream()

    def step():
        cost = D.default_cost(a, b)
        res = D.solve(cost, G, CHAIN_CFG, 0, want_tmap=False, want_potentials=True, form='onthefly')
        return cost, res

    for _ in range(args.warmup):
        cost, res = step()
        del cost
    torch.cuda.synchronize()
    n_launch0 = lib.wotg_launch_count()
    with Clocks(0) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        iters = 0
        for _ in range(args.steps):
            cost, res = step()
            iters += res.stats['iterations']
            if _ < args.steps - 1:
                del cost
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.wotg_launch_count() - n_launch0
    t = ev0.elapsed_time(ev1) / 1e3 / args.steps
    big = ImplicitCoupling.from_solve(cost, res)
    # FP64 fixed-point residual of the a-update on sampled rows (size-independent
    # convergence check): ubar_i = eps alpha1 (log p_i - log sum_j dy exp((vbar_j - C_ij)/eps))
    rng = np.random.default_rng(0)
    rows = np.sort(rng.choice(sizes[0], 64, replace=False))
    A64, B64 = a[rows].double(), b.double()
    C_rows = cost.scale * ((A64[:, None, :] - B64[None, :, :]) ** 2).sum(-1)
    eps = big.eps
    a1 = CHAIN_CFG['lambda1'] / (CHAIN_CFG['lambda1'] + eps)
    lse = torch.logsumexp(-np.log(sizes[1]) + (big.v_bar[None, :] - C_rows) / eps, dim=1)
    u_fix = eps * a1 * (torch.log(G[rows]) - lse)
    resid = float((u_fix - big.u_bar[rows]).abs().max() / big.u_bar.abs().max())
    del cost, C_rows
    parity_full = None
    if not getattr(args, 'no_parity', False):
        # the whole map against the reference's solver in FP64 (oracle/torch_ot.py, row blocks)
        torch.cuda.empty_cache()
        R, it_ref, t_ref = fp64_reference(a, b, G, CHAIN_CFG)
        T = big.dense()
        parity_full = dict(dev_errors(T, R), shape=[sizes[0], sizes[1]], iterations_gpu=iters // args.steps,
                           iterations_oracle=it_ref, oracle_s=t_ref,
                           oracle='the reference solver restated in FP64 on the GPU (oracle/torch_ot.py)')
        del R, T
        torch.cuda.empty_cache()

    # the chain: 20 maps held as potentials
    chain = []
    t0 = time.perf_counter()
    chain_iters = 0
    chain_elems = 0
    for k in range(2, len(days) - 1):
        y0, y1, sk, _ = compute_pca(days[k][0], days[k + 1][0], d50)
        pa, pb = (y0 * sk).float().contiguous(), (y1 * sk).float().contiguous()
        c = D.default_cost(pa, pb)
        r = D.solve(c, torch.as_tensor(days[k][1], device='cuda'), CHAIN_CFG, 0, want_tmap=False,
                    want_potentials=True, form='onthefly')
        chain.append(ImplicitCoupling.from_solve(c, r))
        chain_iters += r.stats['iterations']
        chain_elems += c.I * c.J
        del c
    torch.cuda.synchronize()
    t_chain = time.perf_counter() - t0
    tmaps = {(float(k), float(k + 1)): m for k, m in enumerate(chain)}
    nd = len(chain) + 1
    ids, dd = [], []
    for k in range(nd):
        n = sizes[k + 2]
        ids += ['d%d_%d' % (k, i) for i in range(n)]
        dd += [float(k)] * n
    model = wot.TransportMapModel(tmaps, wot.Frame({'day': np.array(dd)}, index=np.array(ids)))
    n_last = sizes[-1]
    P = np.zeros((8, n_last))
    for k in range(8):
        P[k, rng.choice(n_last, 500, replace=False)] = 1.0
    pops = [Population(float(nd - 1), P[k], 'set%d' % k) for k in range(8)]
    model.pull_back(*pops, to_time=0.0, as_list=True)
    torch.cuda.synchronize()
    tp0 = time.perf_counter()
    back = model.pull_back(*pops, to_time=0.0, as_list=True)
    torch.cuda.synchronize()
    t_pull = time.perf_counter() - tp0
    # reference: the same maps as dense FP64 products, one map at a time on the device
    ref = torch.as_tensor(P, device='cuda')
    for m in reversed(chain):
        T = m.dense()
        ref = (T @ ref.T).T
        ref = ref / ref.sum(dim=1, keepdim=True)
        del T
    got = torch.as_tensor(np.array([p.p for p in back]), device='cuda')
    pull_err = float((got - ref).abs().max() / ref.abs().max())

    line = {'metric': METRIC, 'value': 1.0 / t, 'unit': 'maps/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': 'large pair %dx%d cells, 50-d local PCA, on-the-fly form (cost tiles recomputed '
                                   'on the tensor cores), duality-gap solver, eps=0.05 lambda1=1 lambda2=50; then a '
                                   'chain of %d maps of %d-%d cells held as potentials and a pull-back of 8 indicator '
                                   'vectors through it' % (sizes[0], sizes[1], len(chain), min(sizes[2:]),
                                                           max(sizes[2:])),
                       'I': sizes[0], 'J': sizes[1], 'd': d50,
                       'timed': 'cost (for the exact median) + median + duality-gap solve, potentials out'},
            'sinkhorn_iter_per_s': iters / args.steps / t, 'iterations_per_map': iters / args.steps,
            'element_evaluations_per_s': 2.0 * sizes[0] * sizes[1] * iters / args.steps / t,
            'fixed_point_residual_sampled_rows': resid, 'parity_full': parity_full,
            'chain': {'maps': len(chain), 'cells': sizes[2:], 'solve_s': t_chain, 'iterations': chain_iters,
                      'pull_back_s': t_pull, 'populations': 8,
                      'pull_back_entries_per_s': chain_elems / t_pull,
                      'pull_back_note': 'each coupling entry of the 20 maps recomputed and exponentiated once '
                                        'for all 8 populations (wotg_apply_points)',
                      'pull_back_max_rel_err_vs_dense_fp64': pull_err},
            'gpu_launches': int(launches), 'clocks': clk.summary(), 'e2e': None}
    return line

def main():
    global I_FULL, J_FULL, WORKLOAD, PCA_D
    args = parse()
    if args.pca:
        PCA_D = int(args.pca)
        WORKLOAD = WORKLOAD.replace('local_pca=30', 'local_pca=%d' % PCA_D)
    if args.workload == 'chain' and args.impl != 'reference':
        data = chain_days()
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps(run_chain(args, data)), flush=True)
        return
    if args.workload == 'adjoint' and args.impl != 'reference':
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps(run_adjoint(args)), flush=True)
        return
    if args.workload == 'course' and args.impl != 'reference':
        rank, world, local = dist_env()
        if world > 1:
            from wot_gb300.ot import shard
            _, shapes, items = course_items(args.course_days)
            mine = shard.my_items(shapes, items, rank, world)
            need = {items[k][0] for k in mine} | {items[k][0] + 1 for k in mine}
            data = course_days(args.course_days, needed=need)
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(local)
            dist.init_process_group('nccl')
            line = run_course_sharded(args, data, rank, world, dist)
            if line is not None:
                print(json.dumps(line), flush=True)
            dist.destroy_process_group()
            return
        data = course_days(args.course_days)
        import torch
        torch.cuda.set_device(local)
        print(json.dumps(run_course(args, data)), flush=True)
        return
    if args.pair:
        I_FULL, J_FULL = (int(v) for v in args.pair.split(','))
        WORKLOAD = WORKLOAD.replace('20000x25000', '%dx%d' % (I_FULL, J_FULL))
    if args.impl == 'reference':
        run_reference(args)
        return
    rank, world, local = dist_env()
    extra = rank == 0 and world == 1 and not args.no_extra and args.pair is None and args.pca is None
    course_data = chain_data = None
    if extra:
        # day data of the two extra workloads (process pools must start before CUDA)
        try:
            course_data = course_days(args.course_days)
            chain_data = chain_days()
        except Exception as e:  # noqa: BLE001
            course_data = chain_data = ('error', repr(e))
    import torch
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
        pg = dist
    from wot_gb300 import _build, _native
    _build.build()
    lib = _native.load()
    import wot_gb300 as wot
    from wot_gb300.ot import device as D

    X, day, growth = make_pair(1 + rank)
    a, b = coords_on_device(X, day)
    G = torch.as_tensor(growth[day == 0], device='cuda')
    tmap = torch.empty((I_FULL, J_FULL), dtype=torch.float64, device='cuda')
    stream = torch.cuda.current_stream()

    def step():
        cost = D.default_cost(a, b)
        return D.solve(cost, G, CFG, _native.SOLVER_DUALITY_GAP, want_tmap=True, tmap_out=tmap, form=args.form)

    for _ in range(args.warmup):
        res = step()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    n_launch0 = lib.wotg_launch_count()
    iters = 0
    with Clocks(local) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            res = step()
            iters += res.stats['iterations']
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.wotg_launch_count() - n_launch0
    t = ev0.elapsed_time(ev1) / 1e3
    if pg:
        tt = torch.tensor([t], device='cuda')
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        t = float(tt.item())
    value = world * args.steps / t

    # dominant kernels, timed live with CUDA events on the launching stream
    import ctypes
    cost = D.default_cost(a, b)
    form = D.resolve_form(cost, args.form)
    sh = ctypes.c_void_p(stream.cuda_stream)
    reps = 20

    def time_launches(fn):
        for _ in range(3):
            fn()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
        for r in range(reps):
            evs[2 * r].record(stream)
            fn()
            evs[2 * r + 1].record(stream)
        torch.cuda.synchronize()
        return float(np.mean([evs[2 * r].elapsed_time(evs[2 * r + 1]) for r in range(reps)])) / 1e3

    hbm_peak, tf_peak, peak_kind = peaks()
    exp_pk = exp2_peak()
    # materialised form: streaming row pass over the FP32 cost (HBM-bound)
    ldc = cost.ldc
    w = torch.zeros(ldc, dtype=torch.float32, device='cuda')
    L = torch.empty(I_FULL, dtype=torch.float64, device='cuda')
    L2 = torch.empty(J_FULL, dtype=torch.float64, device='cuda')
    wr = torch.zeros(I_FULL, dtype=torch.float32, device='cuda')
    ws = torch.empty(lib.wotg_lse_matvec_workspace_bytes(I_FULL, J_FULL, ldc), dtype=torch.uint8, device='cuda')
    k2 = ctypes.c_float(float(cost.scale / CFG['epsilon'] * 1.4426950408889634))
    t_row = time_launches(lambda: lib.wotg_lse_matvec(cost.C.data_ptr(), I_FULL, J_FULL, ldc, w.data_ptr(), k2, 0,
                                                      L.data_ptr(), ws.data_ptr(), ws.numel(), sh))
    t_col = time_launches(lambda: lib.wotg_lse_matvec(cost.C.data_ptr(), I_FULL, J_FULL, ldc, wr.data_ptr(), k2, 1,
                                                      L2.data_ptr(), ws.data_ptr(), ws.numel(), sh))
    alg_bytes = I_FULL * J_FULL * 4 + (J_FULL + I_FULL) * 12
    # DRAM bytes read + written per algorithmic byte of the row pass, from an ncu
    # capture of the same kernel on an 8000 x 10000 pair (traffic grows with I*J)
    traffic_ratio = (320.801280 + 3.477504) / (8000 * 10000 * 4 / 1e6)
    roof_mat = {'bound': 'hbm', 'achieved': alg_bytes / t_row / 1e9, 'peak': hbm_peak, 'unit': 'GB/s',
                'frac': alg_bytes / t_row / 1e9 / hbm_peak, 'traffic': I_FULL * J_FULL * 4 * traffic_ratio,
                'kernel': 'row_pass_kernel (wotg_lse_matvec axis 0)', 'peak_kind': peak_kind,
                'row_pass_ms': t_row * 1e3, 'col_pass_ms': t_col * 1e3,
                'col_pass_GBps': alg_bytes / t_col / 1e9}
    # on-the-fly form: tensor-core half-step from the points
    wj = torch.zeros(J_FULL, dtype=torch.float64, device='cuda')
    wsp = torch.empty(lib.wotg_lse_points_workspace_bytes(I_FULL, J_FULL, PCA_D), dtype=torch.uint8, device='cuda')
    sc = float(cost.scale / CFG['epsilon'])

    def tc_kernel_s(speculative):
        # the tensor-core kernel alone, 20 launches timed with CUDA events on this stream
        r = ctypes.c_float(0.0)
        _native.check(lib.wotg_lse_points_timing(a.data_ptr(), I_FULL, a.stride(0), b.data_ptr(), J_FULL,
                                                 b.stride(0), PCA_D, sc, wj.data_ptr(), speculative, reps,
                                                 ctypes.byref(r), wsp.data_ptr(), wsp.numel(), sh),
                      'wotg_lse_points_timing')
        return r.value * 1e-3

    t_tc = tc_kernel_s(1)        # the form the solve runs once a row's previous LSE is known
    t_tc_exact = tc_kernel_s(0)  # the form of the first half-step after each epsilon change
    t_tc_call = time_launches(lambda: lib.wotg_lse_points(a.data_ptr(), I_FULL, a.stride(0), b.data_ptr(), J_FULL,
                                                          b.stride(0), PCA_D, sc, wj.data_ptr(), L.data_ptr(),
                                                          wsp.data_ptr(), wsp.numel(), sh))
    flops = 2.0 * PCA_D * I_FULL * J_FULL           # algorithmic cross-term contraction
    # DRAM bytes per launch from an ncu capture of this kernel inside this workload's solve
    # (5.89e6 and 5.93e6 B read, 0 written): the packed FP16 hi/lo points, read once
    tc_traffic = (5893888 + 5927168) / 2 / (20000 + 25000) * (I_FULL + J_FULL)
    roof_tc = {'bound': 'tensor', 'achieved': flops / t_tc / 1e12, 'peak': tf_peak, 'unit': 'TFLOP/s',
               'frac': flops / t_tc / 1e12 / tf_peak, 'traffic': tc_traffic,
               'kernel': 'lse_tc_kernel<32> (speculative form, as in the solve)', 'peak_kind': peak_kind,
               'launch_ms': t_tc * 1e3, 'exact_form_launch_ms': t_tc_exact * 1e3,
               'wotg_lse_points_call_ms': t_tc_call * 1e3,
               'executed_mma_tflops': 3 * 2.0 * 32 * I_FULL * J_FULL / t_tc / 1e12,
               'exp_per_s': I_FULL * J_FULL / t_tc,
               'exp2_peak_per_s': exp_pk,
               'exp2_frac': (I_FULL * J_FULL / t_tc / exp_pk) if exp_pk else None,
               'note': 'the exp + FP32 reduction of every cost element (one per element, from TMEM) bounds this '
                       'kernel, not the split-precision MMA (3 FP16 products per contraction step)'}
    roofline = roof_tc if form == _native.FORM_ONTHEFLY else roof_mat
    del cost

    line = {'metric': METRIC, 'value': value, 'unit': 'maps/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t / args.steps * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': WORKLOAD, 'I': I_FULL, 'J': J_FULL, 'd': PCA_D, 'parallelism': 'replicas' if world > 1 else 'single',
                       'l2': ('inputs larger than L2: every step writes the 2.0 GB FP32 cost and the 4.0 GB '
                              'FP64 map, so nothing of one step stays in L2 for the next; the materialised '
                              'form streams the cost every half-step, the on-the-fly form re-reads its 5.8 MB '
                              'of packed points from L2 within a step'),
                       'timed': 'cost + median + 3 duality-gap solves + dense FP64 coupling, coordinates resident'},
            'sinkhorn_iter_per_s': iters / t * world, 'iterations_per_map': iters / args.steps,
            'roofline': roofline, 'roofline_materialized': roof_mat, 'roofline_onthefly': roof_tc,
            'form': 'onthefly' if form == _native.FORM_ONTHEFLY else 'materialized',
            'gpu_launches': int(launches), 'clocks': clk.summary()}

    if not args.no_e2e:
        ids = np.array(['c%d' % i for i in range(len(day))])
        ds = wot.Dataset(X, wot.Frame({'day': day, 'cell_growth_rate': growth}, index=ids))
        model = wot.OTModel(ds, growth_iters=3, form=args.form)
        model.compute_transport_map(0, 1)
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tm = model.compute_transport_map(0, 1)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        if pg:
            tt = torch.tensor([te], device='cuda')
            pg.all_reduce(tt, op=pg.ReduceOp.MAX)
            te = float(tt.item())
        line['e2e'] = {'value': world * args.steps / te, 'unit': 'maps/s',
                       'h2d_bytes_per_step': int(X.shape[0] * X.shape[1] * 8 + I_FULL * 8),
                       'd2h_bytes_per_step': int(I_FULL * J_FULL * 8 + 3 * I_FULL * 8),
                       'api': 'wot_gb300.OTModel(Dataset).compute_transport_map(0, 1) (device PCA + cost + solve)',
                       'last_call_s': getattr(model, 'last_timing', None)}
    if rank == 0 and not args.no_cpu:
        rng = np.random.default_rng(0)
        a_h, b_h, G_h = a.double().cpu().numpy(), b.double().cpu().numpy(), growth[day == 0]
        stages = {}
        t_cpu, it_cpu, T_cpu, (a_s, b_s, G_s) = cpu_sample(a_h, b_h, G_h, SAMPLE[0], SAMPLE[1], rng, stages)
        # the oracle's PCA of the same subsampled cells, timed apart from the solve
        from oracle import ot_model as oom
        ri, rj = stages.pop('rows')
        tp = time.perf_counter()
        oom.compute_pca(X[day == 0][ri], X[day == 1][rj], PCA_D)
        stages['pca'] = time.perf_counter() - tp
        scale = (I_FULL * J_FULL) / (SAMPLE[0] * SAMPLE[1])
        it_gpu = iters / args.steps
        cpu_value = 1.0 / (t_cpu * scale * (it_gpu / it_cpu))
        res_s = D.solve(D.default_cost(a_s.astype(np.float32), b_s.astype(np.float32)), G_s, CFG, 0, form=args.form)
        T_gpu = res_s.tmap.cpu().numpy()
        line['parity_sample'] = {'shape': list(SAMPLE), 'coupling_max_rel_err':
                                 float(np.abs(T_gpu - T_cpu).max() / np.abs(T_cpu).max()),
                                 'iterations_gpu': res_s.stats['iterations'], 'iterations_oracle': it_cpu}
        line['cpu_baseline'] = {'value': cpu_value, 'unit': 'maps/s', 'cores': blas_threads(), 'kind': 'port',
                                'sample': '%dx%d random subsample of the pair, full FP64 oracle solve with 3 growth '
                                          'iterations (%.1f s, %d iterations); extrapolated to 20000x25000 by '
                                          'I*J*iterations' % (SAMPLE[0], SAMPLE[1], t_cpu, it_cpu),
                                'sample_stages_s': {k: round(v, 3) for k, v in stages.items()},
                                'measured_whole_pair': dict(CPU_FULL_SIZE, note='the oracle on the whole '
                                                            '20000x25000 pair, timed once on this host type '
                                                            '(growth_iters=1); per iteration 1.38x the '
                                                            'extrapolation, so value is an upper bound')}
    if rank == 0 and not args.no_parity:
        # the whole pair against the reference's solver in FP64 (same coordinates, all growth iterations)
        G_dev = growth[day == 0]
        R, it_ref, t_ref = fp64_reference(a, b, G_dev, CFG)
        full = {'shape': [I_FULL, J_FULL], 'oracle': 'the reference solver restated in FP64 on the GPU '
                                                     '(oracle/torch_ot.py, equal to the NumPy oracle)',
                'iterations_oracle': it_ref, 'oracle_s': t_ref}
        full[line['form']] = dict(dev_errors(tmap, R), iterations_gpu=int(iters / args.steps))
        other = 'materialized' if line['form'] == 'onthefly' else 'onthefly'
        res_o = D.solve(D.default_cost(a, b), G, CFG, _native.SOLVER_DUALITY_GAP, want_tmap=True, tmap_out=tmap,
                        form=other)
        full[other] = dict(dev_errors(tmap, R), iterations_gpu=int(res_o.stats['iterations']))
        line['parity_full'] = full
        del R
        torch.cuda.empty_cache()

    if extra:
        # the batched time course (one warm-up, one timed batch), the large-pair chain and the gradient
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup, sub.quick = 1, 1, True
        for key, fn, data in (('course', run_course, course_data), ('chain', run_chain, chain_data),
                              ('adjoint', run_adjoint, None)):
            try:
                if isinstance(data, tuple) and len(data) == 2 and isinstance(data[0], str):
                    raise RuntimeError(data[1])
                r = fn(sub, data)
                r.pop('metric', None)
                line[key] = r
            except Exception as e:  # noqa: BLE001
                line[key] = {'error': repr(e)}
            torch.cuda.empty_cache()
    if rank == 0:
        print('summary: ' + json.dumps(summary_of(line)), file=sys.stderr, flush=True)
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


def summary_of(line):
    """The headline figures of the JSON line (printed to stderr beside it)."""
    out = {'pair_maps_per_s': line.get('value'), 'pair_e2e': (line.get('e2e') or {}).get('value'),
           'pair_parity_full': {k: v for k, v in (line.get('parity_full') or {}).items()
                                if k in ('onthefly', 'materialized')}}
    c = line.get('course') or {}
    if 'value' in c:
        out['course'] = {'maps_per_s': c['value'], 'e2e': (c.get('e2e') or {}).get('value'),
                         'ratio_vs_best_plain': c['batched_vs_plain']['ratio_vs_best_plain'],
                         'exp2_frac': (c.get('roofline') or {}).get('exp2_frac'),
                         'parity_max': (c.get('parity_full') or {}).get('max')}
    for k in ('chain', 'adjoint'):
        if 'value' in (line.get(k) or {}):
            out[k] = line[k]['value']
    return out


if __name__ == '__main__':
    main()
