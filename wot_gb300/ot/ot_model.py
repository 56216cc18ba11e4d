"""OTModel — drop-in for wot.ot.OTModel (wot/ot/ot_model.py) on the GPU.

Same constructor keywords, configuration precedence (defaults <- kwargs <-
parameter file, per-pair overrides of epsilon/lambda1/lambda2), solver choice,
day selection, ``g0..gk`` learned-growth columns and output file naming. The
default cost is computed on the device from the local-PCA coordinates
(``wotg_cost_sqeuclidean`` + ``wotg_median``) and never leaves it; a
user-supplied ``cost_matrix`` is uploaded and, as in the reference, NOT
median-normalised.
"""
from __future__ import annotations

import itertools
import logging
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .. import _native as N
from .. import dataset as ds_
from . import device as D
from . import optimal_transport as ot
from .initializer import parse_configuration, parse_parameter_file
from .util import compute_pca

logger = logging.getLogger('wot')


class OTModel:
    """Computes transport maps (wot/ot/ot_model.py:19-114).

    Parameters
    ----------
    matrix : anndata.AnnData or wot_gb300.dataset.Dataset
        Expression matrix with a day column in ``obs``.
    day_field, covariate_field, growth_rate_field : str
        obs column names.
    **kwargs
        ``config``, ``cell_filter``, ``gene_filter``, ``cell_day_filter``,
        ``ncounts``, ``ncells``, ``solver`` ('duality_gap' | 'fixed_iters'),
        ``parameters`` (2-column file), and any ot_config key. The GPU-only
        ``form`` ('auto' | 'materialized' | 'onthefly') picks how the cost is
        read by the Sinkhorn half-steps, and ``pca`` ('reference' | 'exact') how
        the local PCA is computed: the reference's own scikit-learn PCA
        (randomized solver, random_state 58951) reproduced to FP64 rounding (the
        default, so that maps equal the reference's from the expression matrix
        on), or the exact decomposition of the double-centred matrix that the
        randomized solver approximates; neither is part of ot_config.
    """

    def __init__(self, matrix, day_field='day', covariate_field='covariate',
                 growth_rate_field='cell_growth_rate', **kwargs):
        self.matrix = matrix
        self.day_field = day_field
        self.covariate_field = covariate_field
        self.cell_growth_rate_field = growth_rate_field
        self.day_pairs = parse_configuration(kwargs.pop('config', None))
        cell_filter = kwargs.pop('cell_filter', None)
        gene_filter = kwargs.pop('gene_filter', None)
        day_filter = kwargs.pop('cell_day_filter', None)
        ncounts = kwargs.pop('ncounts', None)
        ncells = kwargs.pop('ncells', None)
        # GPU-only knobs, kept out of ot_config: 'auto' | 'materialized' | 'onthefly', and
        # the local PCA: 'reference' (scikit-learn's solver and seed), or the 'exact' decomposition
        self.form = kwargs.pop('form', 'auto')
        self.pca = kwargs.pop('pca', 'reference')
        if self.pca not in ('exact', 'reference'):
            raise ValueError("pca must be 'exact' or 'reference'")
        self.matrix = _filter(self.matrix, cell_filter, gene_filter)
        if day_filter is not None:
            days = [float(day) for day in day_filter.split(',')] if isinstance(day_filter, str) else day_filter
            rows = np.isin(ds_.column(self.matrix.obs, self.day_field), days)
            self.matrix = self.matrix[rows].copy()
        if ncells is not None:
            self.matrix = self._subsample_cells(int(ncells))
        if ncounts is not None:
            self._downsample_counts(ncounts)
        if self.matrix.X.shape[0] == 0:
            raise ValueError('No cells in matrix')

        self.ot_config = {'local_pca': 30, 'growth_iters': 1, 'epsilon': 0.05, 'lambda1': 1, 'lambda2': 50,
                          'epsilon0': 1, 'tau': 10000, 'scaling_iter': 3000, 'inner_iter_max': 50,
                          'tolerance': 1e-8, 'max_iter': 1e7, 'batch_size': 5, 'extra_iter': 1000}
        solver = kwargs.pop('solver', 'duality_gap')
        if solver == 'fixed_iters':
            self.solver = ot.transport_stablev2
        elif solver == 'duality_gap':
            self.solver = ot.optimal_transport_duality_gap
        else:
            raise ValueError('Unknown solver')
        parameters_from_file = kwargs.pop('parameters', None)
        for k in kwargs.keys():
            self.ot_config[k] = kwargs[k]
        if parameters_from_file is not None:
            for k, v in parse_parameter_file(parameters_from_file).items():
                self.ot_config[k] = v
        local_pca = self.ot_config['local_pca']
        if local_pca > self.matrix.X.shape[1]:
            logger.warning("local_pca set to {}, above gene count of {}. Disabling PCA"
                           .format(local_pca, self.matrix.X.shape[1]))
            self.ot_config['local_pca'] = 0
        if self.day_field not in ds_.columns(self.matrix.obs):
            raise ValueError("Days information not available for matrix")
        day = ds_.column(self.matrix.obs, self.day_field).astype(np.float64)
        if np.isnan(day).any():
            self.matrix = self.matrix[~np.isnan(day)]
        # day values as stored (ints stay ints, so file names read tmaps_1_2 like the reference's)
        self.timepoints = sorted(set(ds_.column(self.matrix.obs, self.day_field).tolist()))

    # -- preprocessing options of the constructor (ot_model.py:44-81) --------
    def _subsample_cells(self, ncells):
        obs = self.matrix.obs
        day = ds_.column(obs, self.day_field).astype(np.float64)
        has_cv = self.covariate_field in ds_.columns(obs)
        cv = ds_.column(obs, self.covariate_field) if has_cv else None
        cvs = sorted(set(cv.tolist())) if has_cv else [None]
        index_list = []
        for d in sorted(set(day.tolist())):
            for c in cvs:
                sel = day == d if c is None else (day == d) & (cv == c)
                idx = np.where(sel)[0]
                if len(idx) > ncells:
                    np.random.shuffle(idx)
                    idx = idx[:ncells]
                index_list.append(idx)
        return self.matrix[np.concatenate(index_list)]

    def _downsample_counts(self, ncounts):
        X = ds_.dense(self.matrix.X)
        for i in range(X.shape[0]):
            total = X[i].sum()
            if total > ncounts:
                X[i] = np.random.multinomial(ncounts, X[i] / total, size=1)[0]
        self.matrix.X = X

    def get_covariate_pairs(self):
        """All covariate pairs in the dataset (ot_model.py:116-122)."""
        if self.covariate_field not in ds_.columns(self.matrix.obs):
            raise ValueError("Covariate value not available in dataset")
        covariate = set(ds_.column(self.matrix.obs, self.covariate_field).tolist())
        return itertools.product(covariate, covariate)

    def compute_all_transport_maps(self, tmap_out='tmaps', overwrite=True, output_file_format='h5ad',
                                   with_covariates=False, cost_matrices=None):
        """Computes and writes every transport map (ot_model.py:124-201)."""
        from ..io import check_file_extension, write_dataset, write_learned_growth
        tmap_dir, tmap_prefix = os.path.split(tmap_out) if tmap_out is not None else (None, None)
        tmap_prefix = tmap_prefix or "tmaps"
        tmap_dir = tmap_dir or '.'
        if not os.path.exists(tmap_dir):
            os.makedirs(tmap_dir)
        t = self.timepoints
        day_pairs = self.day_pairs
        if day_pairs is None or len(day_pairs) == 0:
            day_pairs = [(t[i], t[i + 1]) for i in range(len(t) - 1)]
        if with_covariates:
            day_pairs = [(*d, c) for d, c in itertools.product(day_pairs, self.get_covariate_pairs())]
        if not day_pairs:
            logger.info('No day pairs')
            return
        if cost_matrices is None:
            cost_matrices = [None for _ in day_pairs]
        learned_tables = []
        save_learned_growth = self.ot_config.get('growth_iters', 1) > 1
        # each map is written by one background thread while the next one is
        # computed; at most one write is in flight, and a failed write raises
        # here before the next map is handed over (or at the end)
        writer = ThreadPoolExecutor(max_workers=1)
        pending = None
        try:
            for day_pair, cost_matrix in zip(day_pairs, cost_matrices):
                path = tmap_prefix
                if not with_covariates:
                    path += "_{}_{}".format(*day_pair)
                else:
                    path += "_{}_{}_cv{}_cv{}".format(*day_pair)
                output_file = check_file_extension(os.path.join(tmap_dir, path), output_file_format)
                if os.path.exists(output_file) and not overwrite:
                    logger.info('Found existing tmap at ' + output_file + '. ')
                    continue
                if with_covariates:
                    tmap = self.compute_transport_map(day_pair[0], day_pair[1], covariate=day_pair[2],
                                                      cost_matrix=cost_matrix)
                else:
                    tmap = self.compute_transport_map(*day_pair, cost_matrix=cost_matrix)
                if pending is not None:
                    pending.result()
                pending = writer.submit(write_dataset, tmap, output_file, output_format=output_file_format)
                if save_learned_growth:
                    learned_tables.append(tmap.obs)
                tmap = None
            if pending is not None:
                pending.result()
        finally:
            writer.shutdown(wait=True)
        if learned_tables:
            write_learned_growth(learned_tables, os.path.join(tmap_dir, tmap_prefix + '_g.txt'))

    def compute_transport_maps_batched(self, day_pairs=None, sweep=None, rank=0, world=1, group=None):
        """Every day pair (the consecutive days, or ``day_pairs``) for every
        parameter set of ``sweep`` (a list of ot_config overrides, e.g.
        ``[{'epsilon': e, 'lambda1': l} for e in ... for l in ...]``; default:
        the model's own configuration) in one batched solve (no counterpart in
        the reference, which solves them one by one, ot_model.py:124-201).

        Each pair's cost is built on the device as compute_single_transport_map
        does (day selection, local PCA, median-normalised cost, G = g^(t1 - t0));
        the solver is the duality-gap one. Returns a dict
        {(t0, t1, i): ImplicitMap} with i the index into ``sweep``; an
        ImplicitMap holds the map as potentials (``.dense()``, ``.pull_back``,
        ``.push_forward``, ``.row_sums``, ``.stats``).

        With ``world`` > 1 (one process per GPU, ``torch.distributed``
        initialised, ``rank`` this process's rank) the items are split over the
        ranks by estimated work (``shard.solve_sharded``): each rank builds the
        costs of only the pairs its items use and returns only the maps it
        solved. ``self.batch_summary`` then lists every item's key, status,
        iteration count and the rank that holds its map, on every rank."""
        from . import batch as B
        from . import shard as S
        if self.solver is not ot.optimal_transport_duality_gap:
            raise ValueError('batched solves use the duality-gap solver')
        t = self.timepoints
        pairs_days = list(day_pairs) if day_pairs else [(t[i], t[i + 1]) for i in range(len(t) - 1)]
        sweep = list(sweep) if sweep else [{}]
        keys, selections = [], []
        for t0, t1 in pairs_days:
            config = {**self.ot_config, 't0': t0, 't1': t1, 'covariate': None}
            p0, p1 = self.select_pair(config)
            if p0.shape[0] == 0 or p1.shape[0] == 0:
                continue
            keys.append((t0, t1))
            selections.append((p0, p1))

        def build_pair(p):
            (t0, t1), (p0, p1) = keys[p], selections[p]
            local_pca = self.ot_config.get('local_pca')
            if local_pca is not None and local_pca > 0:
                x0, x1, sv, _ = compute_pca(p0.X, p1.X, local_pca, solver=self.pca)
                cost = OTModel.compute_default_cost_matrix(x0, x1, sv)
            else:
                cost = OTModel.compute_default_cost_matrix(p0.X, p1.X)
            if self.cell_growth_rate_field in ds_.columns(p0.obs):
                G = np.power(ds_.column(p0.obs, self.cell_growth_rate_field).astype(np.float64), t1 - t0)
            else:
                G = np.ones(p0.shape[0])
            return B.prepare_pair(cost, G)

        items, names = [], []
        for p, (t0, t1) in enumerate(keys):
            for i, over in enumerate(sweep):
                items.append((p, {**self.ot_config, **over}))
                names.append((t0, t1, i))
        if world > 1:
            shapes = [(p0.shape[0], p1.shape[0]) for p0, p1 in selections]
            maps, summary = S.solve_sharded(shapes, items, build_pair, rank, world, group)
            self.batch_summary = [(names[k], rec) for k, rec in summary]
            return {names[k]: m for k, m in maps.items()}
        maps = B.solve_batched([build_pair(p) for p in range(len(keys))], items)
        self.batch_summary = [(names[k], {'rank': 0, 'status': m.status, 'stats': m.stats})
                              for k, m in enumerate(maps)]
        return dict(zip(names, maps))

    def compute_transport_map(self, t0, t1, covariate=None, cost_matrix=None):
        """Transport map from t0 to t1 (ot_model.py:203-240)."""
        if self.day_pairs is not None:
            if (t0, t1) not in self.day_pairs:
                raise ValueError("Transport map ({},{}) is not present in day_pairs".format(t0, t1))
            local_config = self.day_pairs[(t0, t1)]
        else:
            local_config = {}
        if covariate is None:
            logger.info('Computing transport map from {} to {}'.format(t0, t1))
        else:
            logger.info('Computing transport map from {} {} to {} {}'.format(t0, covariate[0], t1, covariate[1]))
        config = {**self.ot_config, **local_config, 't0': t0, 't1': t1, 'covariate': covariate,
                  'C': cost_matrix}
        return self.compute_single_transport_map(config)

    @staticmethod
    def compute_default_cost_matrix(a, b, eigenvals=None):
        """Median-normalised squared-Euclidean cost (ot_model.py:242-253), on
        the device; returns a DeviceCost (FP32 matrix + FP64 scale 1/median)."""
        torch = N.require_cuda()
        a = torch.as_tensor(ds_.dense(a) if not isinstance(a, torch.Tensor) else a, device='cuda')
        b = torch.as_tensor(ds_.dense(b) if not isinstance(b, torch.Tensor) else b, device='cuda')
        if eigenvals is not None:
            e = torch.as_tensor(eigenvals, device='cuda', dtype=a.dtype)
            a = a @ e if e.dim() == 2 else a * e
            b = b @ e if e.dim() == 2 else b * e
        return D.default_cost(a, b)

    def select_pair(self, config):
        """Day/covariate selection of one pair (ot_model.py:271-292)."""
        t0, t1 = config['t0'], config['t1']
        obs = self.matrix.obs
        day = ds_.column(obs, self.day_field).astype(np.float64)
        covariate = config.get('covariate')
        if covariate is None:
            s0, s1 = day == float(t0), day == float(t1)
        else:
            cv = ds_.column(obs, self.covariate_field)
            s0 = (day == float(t0)) & (cv == covariate[0])
            s1 = (day == float(t1)) & (cv == covariate[1])
        return self.matrix[_as_slice(s0), :], self.matrix[_as_slice(s1), :]

    def compute_single_transport_map(self, config):
        """One transport map (ot_model.py:255-326)."""
        t0 = config.pop('t0', None)
        t1 = config.pop('t1', None)
        if t0 is None or t1 is None:
            raise ValueError("config must have both t0 and t1, indicating target timepoints")
        config['t0'], config['t1'] = t0, t1
        clock = [('start', time.perf_counter())]
        p0, p1 = self.select_pair(config)
        config.pop('t0')
        config.pop('t1')
        config.pop('covariate', None)
        if p0.shape[0] == 0:
            logger.info('No cells at {}'.format(t0))
            return None
        if p1.shape[0] == 0:
            logger.info('No cells at {}'.format(t1))
            return None
        local_pca = config.pop('local_pca', None)
        clock.append(('select', time.perf_counter()))
        if config['C'] is None:
            if local_pca is not None and local_pca > 0:
                x0, x1, s, _ = compute_pca(p0.X, p1.X, local_pca, solver=self.pca)
                config['C'] = OTModel.compute_default_cost_matrix(x0, x1, s)
            else:
                config['C'] = OTModel.compute_default_cost_matrix(p0.X, p1.X)
        C = config['C']
        n0 = C.shape[0]
        delta_days = t1 - t0
        if self.cell_growth_rate_field in ds_.columns(p0.obs):
            config['G'] = np.power(ds_.column(p0.obs, self.cell_growth_rate_field).astype(np.float64), delta_days)
        else:
            config['G'] = np.ones(n0)
        sid = ot.native_solver_id(self.solver)
        cost = C if isinstance(C, D.DeviceCost) else D.cost_from_dense(C)
        clock.append(('pca_cost', time.perf_counter()))
        # the host array of the FP64 map is allocated and its pages faulted in on
        # host threads while the GPU works; the copy into it then runs at link speed
        out = _prefaulted_async(C.shape[0], C.shape[1])
        res = D.solve(cost, config['G'], config, sid, want_tmap=True, form=self.form)
        clock.append(('solve', time.perf_counter()))
        tmap = out.result()
        clock.append(('host_pages_wait', time.perf_counter()))
        N.require_cuda().from_numpy(tmap).copy_(res.tmap)
        clock.append(('copy_to_host', time.perf_counter()))
        learned = [np.asarray(config['G'], dtype=np.float64)] + [g.cpu().numpy() for g in res.learned_growth[1:]]
        learned.append(res.row_sums.cpu().numpy())
        obs_growth = {'g' + str(i): np.power(g, 1.0 / delta_days) for i, g in enumerate(learned)}
        self.last_stats = res.stats
        result = ds_.make_result(tmap, obs_growth, ds_.index(p0.obs), ds_.index(p1.obs), like=self.matrix)
        clock.append(('assemble', time.perf_counter()))
        # seconds per stage of this call (the solve returns after its device work)
        self.last_timing = {k: clock[i + 1][1] - clock[i][1] for i, (k, _) in enumerate(clock[1:])}
        self.last_timing['call'] = clock[-1][1] - clock[0][1]
        return result


def _as_slice(mask):
    """A boolean row mask as a slice when its rows are contiguous (a view of the
    matrix instead of a copy), else the mask."""
    idx = np.flatnonzero(mask)
    if idx.size and idx[-1] - idx[0] + 1 == idx.size:
        return slice(int(idx[0]), int(idx[-1]) + 1)
    return mask


_TOUCH_POOL = None


def _prefaulted_async(rows, cols, parts=8):
    """Future of an uninitialised (rows x cols) FP64 array whose pages have been
    written once (one store per 4 KB, spread over host threads), so that a
    device-to-host copy into it does not stop on first-touch page faults."""
    from concurrent.futures import ThreadPoolExecutor
    global _TOUCH_POOL
    if _TOUCH_POOL is None:
        _TOUCH_POOL = ThreadPoolExecutor(max_workers=parts, thread_name_prefix='wotg-prefault')
    arr = np.empty((int(rows), int(cols)), dtype=np.float64)
    flat = arr.reshape(-1)
    step = 512  # 4 KB of float64
    bounds = np.linspace(0, flat.size, parts + 1).astype(np.int64)

    def touch(a, b):
        flat[a:b:step] = 0.0

    futs = [_TOUCH_POOL.submit(touch, int(bounds[k]), int(bounds[k + 1])) for k in range(parts)]

    class _Result:
        def result(self):
            for f in futs:
                f.result()
            return arr

    return _Result()


def _filter(adata, cell_filter, gene_filter):
    """wot.io.filter_adata restricted to id lists (wot/io/io.py:499-518)."""
    if cell_filter is not None:
        ids = set(_read_ids(cell_filter))
        adata = adata[np.array([i in ids for i in ds_.index(adata.obs)], dtype=bool)]
    if gene_filter is not None:
        ids = set(_read_ids(gene_filter))
        adata = adata[:, np.array([i in ids for i in ds_.index(adata.var)], dtype=bool)]
    return adata


def _read_ids(spec):
    if isinstance(spec, str):
        if os.path.exists(spec):
            with open(spec) as f:
                return [line.strip() for line in f if line.strip()]
        return [spec]
    return list(spec)
