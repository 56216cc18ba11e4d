"""TransportMapModel — drop-in for wot.tmap.TransportMapModel
(wot/tmap/transport_map_model.py) with population transport on the GPU.

The k x n population matrix stays on the device across day steps; each step
is one ``wotg_apply_coupling_f64`` launch (push: ``p @ X``, :290; pull:
``(X @ p.T).T``, :356) with the optional row normalisation fused into it.
Maps may be given as file paths, AnnData / Dataset objects (dense ``X``), or
Dataset objects whose ``X`` is already a CUDA tensor. With ``cache=True``
loaded maps and their device copies are kept.
"""
from __future__ import annotations

import json
import os
import re

import numpy as np

from .. import _native as N
from .. import dataset as ds_
from ..ot import device as D
from ..population import Population
from .chaining import chain_transport_maps, find_path
from .util import unique_timepoint


class TransportMapModel:
    """Operates on pre-computed transport maps (:12-38).

    Parameters
    ----------
    tmaps : dict
        (t0, t1) -> map path or object.
    meta : DataFrame or Frame
        Cell metadata, index = cell ids, column 'day', in map order.
    timepoints, day_pairs : optional
    cache : bool
    """

    def __init__(self, tmaps, meta, timepoints=None, day_pairs=None, cache=False):
        self.tmaps = tmaps
        self.meta = meta
        self.cache = cache
        if timepoints is None:
            timepoints = sorted(set(ds_.column(meta, 'day').tolist()))
        self.timepoints = timepoints
        if day_pairs is None:
            day_pairs = [(timepoints[i], timepoints[i + 1]) for i in range(len(timepoints) - 1)]
        self.day_pairs = day_pairs
        self._device = {}

    # -- fates, transition table, trajectories (:40-143) ---------------------
    def fates(self, populations):
        """Probability of each earlier cell to end in each population (:40-69)."""
        start_day = unique_timepoint(*populations)
        populations = Population.copy(*populations, normalize=False, add_missing=True)
        pop_names = [pop.name for pop in populations]
        results = [np.array([pop.p for pop in populations]).T]
        while self.can_pull_back(*populations):
            populations = self.pull_back(*populations, as_list=True, normalize=False)
            results.insert(0, np.array([pop.p for pop in populations]).T)
        X = np.concatenate(results)
        X /= X.sum(axis=1, keepdims=1)
        keep = ds_.column(self.meta, 'day') <= start_day
        return _result(X, self.meta, keep, pop_names)

    def transition_table(self, start_populations, end_populations):
        """Mass moving between start and end populations (:71-103)."""
        start_time = unique_timepoint(*start_populations)
        start_populations = Population.copy(*start_populations, normalize=False, add_missing=True)
        end_populations = Population.copy(*end_populations, normalize=False, add_missing=True)
        unique_timepoint(*end_populations)
        populations = end_populations
        while self.can_pull_back(*populations) and unique_timepoint(*populations) > start_time:
            populations = self.pull_back(*populations, as_list=True, normalize=False)
        end_p = np.vstack([pop.p for pop in populations])
        start_p = np.vstack([pop.p for pop in start_populations])
        p = start_p @ end_p.T
        p = p / p.sum()
        return ds_.Dataset(p, ds_.Frame(index=[q.name for q in start_populations]),
                           ds_.Frame(index=[q.name for q in end_populations]))

    def trajectories(self, populations):
        """Ancestors and descendants of each population at every day (:105-143)."""
        unique_timepoint(*populations)
        trajectories = []
        populations = Population.copy(*populations, normalize=True, add_missing=False)
        population_names = [p.name for p in populations]
        initial_populations = populations

        def update(head, pops):
            idx = 0 if head else len(trajectories)
            trajectories.insert(idx, np.array([pop.p for pop in pops]).T)

        update(True, populations)
        while self.can_pull_back(*populations):
            populations = self.pull_back(*populations, as_list=True)
            update(True, populations)
        populations = initial_populations
        while self.can_push_forward(*populations):
            populations = self.push_forward(*populations, as_list=True)
            update(False, populations)
        return _result(np.concatenate(trajectories), self.meta, None, population_names)

    # -- couplings (:145-190) -------------------------------------------------
    def get_coupling(self, t0, t1, covariate=None):
        """The map t0 -> t1, loaded, or chained when t0, t1 are not adjacent."""
        if t0 not in self.timepoints or t1 not in self.timepoints:
            raise ValueError("Day pair {}, {} not found".format(t0, t1))
        atomic = (self.day_pairs is not None and (t0, t1) in self.day_pairs) \
            or self.timepoints.index(t1) == self.timepoints.index(t0) + 1
        if not atomic and covariate is not None:
            raise ValueError("Covariate-restricted transport maps can only be atomic")
        if atomic:
            key = (t0, t1) if covariate is None else (t0, t1, str(covariate[0]), str(covariate[1]))
            ds_or_path = self.tmaps.get(key)
            if ds_or_path is None:
                raise ValueError('No transport map found for {}', key)
            if not isinstance(ds_or_path, (str, os.PathLike)):
                return ds_or_path
            from ..io import read_dataset
            ds = read_dataset(ds_or_path)
            if self.cache:
                self.tmaps[key] = ds
            return ds
        path = find_path(t0, t1, self.day_pairs, self.timepoints)
        return chain_transport_maps(self, path)

    def _implicit(self, t0, t1):
        """The map t0 -> t1 when it is held as potentials (ImplicitCoupling)."""
        from ..ot.implicit import ImplicitCoupling
        m = self.tmaps.get((t0, t1))
        return m if isinstance(m, ImplicitCoupling) else None

    def _device_coupling(self, t0, t1):
        key = (t0, t1)
        if key in self._device:
            return self._device[key]
        imp = self._implicit(t0, t1)
        if imp is not None:
            return imp.dense()
        X = self.get_coupling(t0, t1).X
        torch = N.require_cuda()
        if not (isinstance(X, torch.Tensor) and X.is_cuda and X.dtype == torch.float64):
            X = torch.as_tensor(ds_.dense(X), device='cuda')
        if self.cache:
            self._device[key] = X
        return X

    def can_push_forward(self, *populations):
        return self.timepoints.index(unique_timepoint(*populations)) < len(self.timepoints) - 1

    def can_pull_back(self, *populations):
        return self.timepoints.index(unique_timepoint(*populations)) > 0

    def push_forward(self, *populations, to_time=None, normalize=True, as_list=False):
        """Push populations forward through the maps (:235-299)."""
        i = self.timepoints.index(unique_timepoint(*populations))
        j = i + 1 if to_time is None else self.timepoints.index(to_time)
        if i == -1:
            raise ValueError("Timepoint not found")
        if j == -1:
            raise ValueError("Destination timepoint not found")
        if j >= len(self.timepoints):
            raise ValueError("No further timepoints. Unable to push forward")
        if i > j:
            raise ValueError("Destination timepoint is before source. Unable to push forward")
        p = np.vstack([pop.p for pop in populations])
        while i < j:
            imp = self._implicit(self.timepoints[i], self.timepoints[i + 1])
            if imp is not None:
                p = imp.push_forward(p, normalize=normalize)
            else:
                X = self._device_coupling(self.timepoints[i], self.timepoints[i + 1])
                p = D.apply_coupling(X, p, transpose=False, normalize=normalize)
            i += 1
        p = p.cpu().numpy() if not isinstance(p, np.ndarray) else p
        result = [Population(self.timepoints[i], p[k, :]) for k in range(p.shape[0])]
        if len(result) == 1 and not as_list:
            return result[0]
        return result

    def pull_back(self, *populations, to_time=None, normalize=True, as_list=False):
        """Pull populations back through the maps (:301-365)."""
        i = self.timepoints.index(unique_timepoint(*populations))
        j = i - 1 if to_time is None else self.timepoints.index(to_time)
        if i == -1:
            raise ValueError("Timepoint not found")
        if i == 0:
            raise ValueError("No previous timepoints. Unable to pull back")
        if j == -1:
            raise ValueError("Destination timepoint not found")
        if i < j:
            raise ValueError("Destination timepoint is after source. Unable to pull back")
        p = np.vstack([pop.p for pop in populations])
        while i > j:
            imp = self._implicit(self.timepoints[i - 1], self.timepoints[i])
            if imp is not None:
                p = imp.pull_back(p, normalize=normalize)
            else:
                X = self._device_coupling(self.timepoints[i - 1], self.timepoints[i])
                p = D.apply_coupling(X, p, transpose=True, normalize=normalize)
            i -= 1
        p = p.cpu().numpy() if not isinstance(p, np.ndarray) else p
        result = [Population(self.timepoints[i], p[k, :]) for k in range(p.shape[0])]
        if len(result) == 1 and not as_list:
            return result[0]
        return result

    def ancestors(self, *populations, at_time=None, as_list=False):
        """Alias of pull_back (:367-409)."""
        return self.pull_back(*populations, to_time=at_time, as_list=as_list)

    def descendants(self, *populations, at_time=None, as_list=False):
        """Alias of push_forward (:411-453)."""
        return self.push_forward(*populations, to_time=at_time, as_list=as_list)

    # -- populations (:455-615) -----------------------------------------------
    def _day_ids(self, day):
        d = ds_.column(self.meta, 'day')
        return ds_.index(self.meta)[d == day]

    def population_from_ids(self, *ids, at_time):
        """Uniform indicator populations of the given ids at ``at_time`` (:455-507)."""
        day = float(at_time)
        day_ids = self._day_ids(day)
        pos = {c: k for k, c in enumerate(day_ids.tolist())}

        def get_population(ids_el):
            idx = np.array([pos[c] for c in ids_el if c in pos], dtype=np.int64)
            if len(idx) == 0:
                return None
            p = np.zeros(len(day_ids), dtype=np.float64)
            p[idx] = 1.0
            return Population(day, p)

        return [get_population(ids_el) for ids_el in ids]

    def population_from_cell_sets(self, cell_sets, at_time):
        keys = list(cell_sets.keys())
        populations = self.population_from_ids(*[cell_sets[name] for name in keys], at_time=at_time)
        out = []
        for i in range(len(keys)):
            if populations[i] is not None:
                populations[i].name = keys[i]
                out.append(populations[i])
        return out

    def cell_ids(self, population):
        return self._day_ids(population.time)

    def ancestor_census(self, cset_matrix, *populations):
        """Census of ancestors and descendants at every day (:540-574)."""
        initial_populations = populations
        timepoints = []
        census = []

        def update(head, pops):
            x = 0 if head else len(census)
            timepoints.insert(x, unique_timepoint(*pops))
            census.insert(x, self.population_census(cset_matrix, *pops))

        update(True, populations)
        while self.can_pull_back(*populations):
            populations = self.pull_back(*populations, as_list=True)
            update(True, populations)
        populations = initial_populations
        while self.can_push_forward(*populations):
            populations = self.push_forward(*populations, as_list=True)
            update(False, populations)
        census = np.asarray(census)
        if census.ndim == 3:
            census = np.asarray([census[:, i, :] for i in range(census.shape[1])])
        return timepoints, census

    def population_census(self, cell_set_matrix, *populations):
        """P(cell set | population) for each population (:576-615)."""
        day = unique_timepoint(*populations)
        day_ids = self._day_ids(day)
        cs_ids = ds_.index(cell_set_matrix.obs)
        inter = [c for c in cs_ids.tolist() if c in set(day_ids.tolist())]
        Xc = ds_.dense(cell_set_matrix.X)
        if len(inter) == 0:
            return [[0] * Xc.shape[1]] * len(populations)
        pos_p = {c: k for k, c in enumerate(day_ids.tolist())}
        pos_c = {c: k for k, c in enumerate(cs_ids.tolist())}
        pop_indexer = np.array([pos_p[c] for c in inter])
        csm_indexer = np.array([pos_c[c] for c in inter])

        def norm(p):
            return p if np.isclose(np.sum(p), 0) else p / np.sum(p)

        return np.asarray([np.dot(norm(pop.p)[pop_indexer], Xc[csm_indexer, :]) for pop in populations],
                          dtype=np.float64)

    # -- persistence (:617-732) -------------------------------------------------
    def to_json(self, path):
        meta = {'day': ds_.column(self.meta, 'day').tolist(), 'id': ds_.index(self.meta).tolist()}
        day_pairs = list(self.day_pairs)
        paths = [self.tmaps[dp] for dp in day_pairs]
        with open(path, 'w') as f:
            json.dump({'day_pairs': day_pairs, 'paths': paths, 'timepoints': list(self.timepoints),
                       'meta': meta}, f, ensure_ascii=False)

    @staticmethod
    def from_json(index_path):
        with open(index_path) as r:
            info = json.load(r)
        meta = ds_.Frame({'day': info['meta']['day']}, index=info['meta']['id'])
        day_pairs = info['day_pairs']
        tmaps = {tuple(day_pairs[i]): info['paths'][i] for i in range(len(day_pairs))}
        return TransportMapModel(tmaps=tmaps, meta=meta, timepoints=info['timepoints'], day_pairs=day_pairs)

    @staticmethod
    def from_directory(tmap_out, with_covariates=False, cache=False):
        """Index the map files written by compute_all_transport_maps (:651-732)."""
        from ..io import read_ids
        tmap_dir, tmap_prefix = os.path.split(tmap_out)
        tmap_dir = tmap_dir or '.'
        tmap_prefix = tmap_prefix or "tmaps"
        day = r'([0-9]*\.?[0-9]+)'
        ext = r'\.(h5ad|loom|npz)$'
        if with_covariates:
            pattern = re.compile(re.escape(tmap_prefix) + '_{}_{}_cv([a-zA-Z0-9]+)_cv([a-zA-Z0-9]+)'.format(day, day) + ext)
        else:
            pattern = re.compile(re.escape(tmap_prefix) + '_{}_{}'.format(day, day) + ext)
        tmaps = {}
        for f in os.listdir(tmap_dir):
            path = os.path.join(tmap_dir, f)
            if os.path.isfile(path):
                m = pattern.match(f)
                if m is not None:
                    t1, t2 = float(m.group(1)), float(m.group(2))
                    key = (t1, t2, m.group(3), m.group(4)) if with_covariates else (t1, t2)
                    tmaps[key] = path
        if len(tmaps) == 0:
            raise ValueError('No transport maps found in ' + tmap_dir + ' with prefix ' + tmap_prefix)
        day_pairs, timepoints = set(), set()
        keys = sorted(tmaps.keys(), key=lambda x: x[0])
        ids, days = [], []
        for i, key in enumerate(keys):
            t0, t1 = key[0], key[1]
            day_pairs.add((t0, t1))
            timepoints.add(t0)
            timepoints.add(t1)
            if not with_covariates:
                rids, cids = read_ids(tmaps[key])
                ids.extend(rids.tolist())
                days.extend([t0] * len(rids))
                if i == len(keys) - 1:
                    ids.extend(cids.tolist())
                    days.extend([t1] * len(cids))
        meta = ds_.Frame({'day': np.asarray(days, dtype=np.float64)}, index=np.asarray(ids)) if ids else None
        return TransportMapModel(tmaps=tmaps, meta=meta, timepoints=sorted(timepoints), day_pairs=day_pairs,
                                 cache=cache)


def _result(X, meta, keep, names):
    idx = ds_.index(meta)
    day = ds_.column(meta, 'day')
    if keep is not None:
        idx, day = idx[keep], day[keep]
    return ds_.Dataset(X, ds_.Frame({'day': day}, index=idx), ds_.Frame(index=np.asarray(names, dtype=object)))
