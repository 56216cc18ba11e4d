"""Host-side logic that needs no GPU: configuration parsing, populations,
paths, containers, map files and the C-ABI library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

import wot_gb300
from wot_gb300 import Population, _native, io as wio
from wot_gb300.dataset import Dataset, Frame
from wot_gb300.ot import parse_configuration, parse_parameter_file
from wot_gb300.ot.device import make_params
from wot_gb300.tmap import find_path, unique_timepoint

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    with open(os.path.join(ROOT, 'include', 'wotg.h')) as f:
        text = f.read()
    return sorted(set(re.findall(r'^\s*(?:const\s+)?\w[\w\s\*]*?\b(wotg_\w+)\s*\(', text, flags=re.M)))


def test_header_and_binding_agree():
    assert header_symbols() == sorted(_native.EXPORTS)


def test_library_loads_and_exports_everything():
    from wot_gb300 import _build
    _build.build()
    lib = _native.load()
    for name in header_symbols():
        assert hasattr(lib, name), name
    assert lib.wotg_version().decode().startswith('wotg')
    assert lib.wotg_median_workspace_bytes() >= 4096 * 8


def test_params_mapping_and_tau_none():
    p = make_params({'epsilon': 0.01, 'lambda1': 3, 'growth_iters': 2, 'max_iter': 1e7}, 0)
    assert p.epsilon == 0.01 and p.lambda1 == 3.0 and p.lambda2 == 50.0 and p.growth_iters == 2
    assert p.batch_size == 5 and p.tolerance == 1e-8
    with pytest.raises(TypeError):
        make_params({'tau': None}, 1)


def test_parse_configuration(tmp_path):
    assert parse_configuration(None) is None
    # inline tables (wot/io/io.py:553-555: ',' between fields, ';' between rows) and header-less pairs
    assert parse_configuration('t0,t1,epsilon;0,1,0.05;1,2,0.1') == {(0, 1): {'epsilon': 0.05},
                                                                      (1, 2): {'epsilon': 0.1}}
    assert parse_configuration('t0,t1;0,2;2,4') == {(0, 2): {}, (2, 4): {}}
    bare = tmp_path / 'day_pairs.txt'
    bare.write_text('0\t2\n2\t4\n')
    assert parse_configuration(str(bare)) == {(0, 2): {}, (2, 4): {}}
    cfg = parse_configuration.__globals__['parse_per_timepair_configuration'](
        {(0, 1): {'epsilon': 0.1, 'lambda1': 2, 'junk': 5}})
    assert cfg == {(0, 1): {'epsilon': 0.1, 'lambda1': 2}}
    with pytest.raises(ValueError):
        parse_configuration({(0, 1): {}})
    f = tmp_path / 'pairs.txt'
    f.write_text('t0\tt1\tepsilon\n0\t1\t0.1\n1\t2\t0.2\n')
    pairs = parse_configuration(str(f))
    assert pairs[(0, 1)] == {'epsilon': 0.1} and pairs[(1, 2)] == {'epsilon': 0.2}
    pf = tmp_path / 'params.txt'
    pf.write_text('epsilon\t0.02\nlambda1\t4\n')
    assert parse_parameter_file(str(pf)) == {'epsilon': 0.02, 'lambda1': 4}


def test_population_copy_and_other():
    a = Population(1.0, [1.0, 0.0, 0.0, 2.0], 'a')
    b = Population(1.0, [0.0, 3.0, 0.0, 0.0], 'b')
    pops = Population.copy(a, b, normalize=False, add_missing=True)
    assert [p.name for p in pops] == ['a', 'b', 'Other']
    np.testing.assert_array_equal(pops[0].p, [1, 0, 0, 1])
    np.testing.assert_array_equal(pops[2].p, [0, 0, 1, 0])
    pops = Population.copy(a, normalize=True)
    assert pops[0].p.sum() == pytest.approx(1.0)
    pops = Population.copy(a)
    np.testing.assert_array_equal(pops[0].p, a.p)
    assert unique_timepoint(a, b) == 1.0
    with pytest.raises(ValueError):
        unique_timepoint(a, Population(2.0, [1.0]))


def test_find_path():
    tp = [0, 1, 2, 3, 4]
    assert find_path(0, 3, None, tp) == [(0, 1), (1, 2), (2, 3)]
    assert find_path(0, 4, [(0, 2), (2, 4), (0, 1), (1, 2)], tp) == [(0, 1), (1, 2), (2, 4)]
    with pytest.raises(ValueError, match='not reachable'):
        find_path(0, 3, [(0, 1), (1, 2)], tp)
    with pytest.raises(ValueError, match='must be present'):
        find_path(0, 7, [(0, 1)], tp)
    # ties: of two chains of the same length into a day, the one through the earlier predecessor is kept
    assert find_path(0, 3, [(0, 1), (1, 3), (0, 2), (2, 3)], tp) == [(0, 1), (1, 3)]
    assert find_path(0, 4, [(2, 4), (0, 2), (0, 1), (1, 4), (3, 4), (0, 3)], tp) == [(0, 1), (1, 4)]
    assert find_path(0, 4, [(0, 1), (1, 2), (0, 2), (2, 4), (1, 3), (3, 4)], tp) == [(0, 1), (1, 2), (2, 4)]
    # a longer chain starting at a day that t0 does not reach does not count
    assert find_path(0, 3, [(0, 3), (1, 2), (2, 3)], tp) == [(0, 3)]


def _longest_chain_length(t0, t1, pairs):
    """Brute force: edges of the longest chain of forward pairs from t0 to t1."""
    best = -1
    stack = [(t0, 0)]
    while stack:
        day, n = stack.pop()
        if day == t1:
            best = max(best, n)
        stack += [(b, n + 1) for a, b in pairs if a == day and a < b]
    return best


def test_find_path_matches_reference_cases():
    """The reference's own find_path on 400 seeded pair sets
    (tests/golden/make_paths.py): the same path wherever the reference returns
    one, the same ValueError wherever it raises one; where the reference fails
    with a KeyError (a longest chain into t1 that starts at a day t0 cannot
    reach), the longest chain from t0, checked by brute force, or the
    reference's ValueError when no chain from t0 reaches t1."""
    import json
    with open(os.path.join(ROOT, 'tests', 'golden', 'find_path_cases.json')) as f:
        cases = json.load(f)
    kinds = set()
    for c in cases:
        tp, t0, t1 = c['timepoints'], c['t0'], c['t1']
        pairs = [tuple(p) for p in c['pairs']]
        err = c.get('error')
        kinds.add(err or 'path')
        if err == 'ValueError':
            with pytest.raises(ValueError):
                find_path(t0, t1, pairs, tp)
            continue
        if err is None:
            assert find_path(t0, t1, pairs, tp) == [tuple(p) for p in c['path']], c
            continue
        assert err == 'KeyError', c
        if _longest_chain_length(t0, t1, pairs) <= 0:
            with pytest.raises(ValueError, match='not reachable'):
                find_path(t0, t1, pairs, tp)
            continue
        got = find_path(t0, t1, pairs, tp)
        assert got[0][0] == t0 and got[-1][1] == t1 and all(p in pairs for p in got), c
        assert all(a[1] == b[0] for a, b in zip(got[:-1], got[1:])), c
        assert len(got) == _longest_chain_length(t0, t1, pairs), c
    assert kinds == {'path', 'ValueError', 'KeyError'}


def test_dataset_selection():
    ds = Dataset(np.arange(12.).reshape(4, 3), Frame({'day': [0., 0., 1., 1.]}, index=['a', 'b', 'c', 'd']))
    sub = ds[np.array([False, True, True, False]), :]
    assert sub.shape == (2, 3) and list(sub.obs.index) == ['b', 'c']
    np.testing.assert_array_equal(sub.X, [[3, 4, 5], [6, 7, 8]])


def test_map_file_roundtrip(tmp_path):
    ds = Dataset(np.random.default_rng(0).random((3, 4)), Frame({'g0': [1., 2., 3.]}, index=['x', 'y', 'z']),
                 Frame(index=['p', 'q', 'r', 's']))
    path = wio.check_file_extension(str(tmp_path / 'tmaps_1_2'), 'npz')
    wio.write_dataset(ds, path, output_format='npz')
    back = wio.read_dataset(path)
    np.testing.assert_array_equal(back.X, ds.X)
    assert list(back.obs.index) == ['x', 'y', 'z'] and list(back.var.index) == ['p', 'q', 'r', 's']
    np.testing.assert_array_equal(back.obs['g0'], [1., 2., 3.])
    m = wot_gb300.TransportMapModel.from_directory(str(tmp_path / 'tmaps'))
    assert m.timepoints == [1.0, 2.0] and (1.0, 2.0) in m.tmaps
    assert list(m.meta.index) == ['x', 'y', 'z', 'p', 'q', 'r', 's']


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    with pytest.raises(RuntimeError, match='CUDA device'):
        wot_gb300.ot.optimal_transport_duality_gap(np.zeros((2, 2)), np.ones(2), 1, 50, 0.05, 5, 1e-8, 1e4, 1, 1e7)


def test_centred_gram_identity():
    """The PCA's Gram matrix from x^T x (dense and sparse products) equals the
    Gram matrix of the explicitly double-centred matrix (wot/ot/util.py:240-255:
    gene means removed, then each cell centred over genes), to FP64 rounding."""
    import torch
    from wot_gb300.ot.util import centred_gram
    rng = np.random.default_rng(7)
    x = rng.random((900, 150))
    x[rng.random(x.shape) < 0.9] = 0.0
    X = torch.tensor(np.log1p(5 * x))
    mu = X.mean(dim=0)
    xt = (X - mu).T
    xt = xt - xt.mean(dim=0, keepdim=True)
    ref = xt @ xt.T
    for sparse in (False, True, None):
        G = centred_gram(X, mu, sparse=sparse)
        assert float((G - ref).abs().max() / ref.abs().max()) < 1e-13
        assert torch.equal(G, G.T) or float((G - G.T).abs().max()) < 1e-15 * float(ref.abs().max())


def test_invalid_arguments_rejected_before_device_work():
    """Every compute entry point of the C ABI checks its arguments before it
    touches the device: NULL pointers, empty or misaligned shapes and
    non-positive parameters return WOTG_BADARG (the reference's ValueError,
    through _native.check) on a machine without a GPU. No kernel runs here."""
    from wot_gb300 import _build
    _build.build()
    lib = _native.load()
    BAD = _native.WOTG_BADARG
    f = ctypes.c_float
    d = ctypes.c_double(0.0)
    assert lib.wotg_median(None, 10, 10, 12, ctypes.byref(d), None, 0, None) == BAD
    assert lib.wotg_median(None, 10, 10, 10, ctypes.byref(d), None, 0, None) == BAD   # ldc not a multiple of 4
    assert lib.wotg_compute_transport_matrix(None, None, None, None, None, None, None, None, None, 0, None) == BAD
    assert lib.wotg_compute_transport_matrix_noalloc(None, None, None, None, None, None, None, None, None) == BAD
    assert lib.wotg_refine_potentials(None, None, 0.05, 10, None, None, None, None, 0, None) == BAD
    assert lib.wotg_lse_matvec(None, 4, 4, 4, None, f(1.0), 0, None, None, 0, None) == BAD
    assert lib.wotg_lse_points(None, 4, 4, None, 4, 4, 4, 1.0, None, None, None, 0, None) == BAD
    r = ctypes.c_float(0.0)
    assert lib.wotg_lse_points_timing(None, 4, 4, None, 4, 4, 4, 1.0, None, 1, 0, ctypes.byref(r), None, 0,
                                      None) == BAD
    assert lib.wotg_apply_coupling_f64(None, 3, 3, None, 0, 0, 0, None, None) == BAD
    assert lib.wotg_transpose_cost(None, 3, 3, 4, None, 3, None) == BAD
    assert lib.wotg_solve_batched(None, 0, None, 0, None, None, None, None, None, None, None, 0, None) == BAD
    k2 = (ctypes.c_float * 1)(1.0)
    assert lib.wotg_lse_matvec_multi(None, 4, 4, 4, None, 4, k2, 1, None, 4, None, 0, None) == BAD
    assert lib.wotg_coupling_from_potentials(None, 3, 3, 4, 1.0, 0.0, None, None, 0.0, None, None) == BAD
    assert lib.wotg_ot_adjoint(None, 3, 2, None, 3, 2, 2, 1.0, 0.05, 1.0, 50.0, None, None, None, None, None, None,
                               ctypes.byref(d), None, 0, None) == BAD
    assert lib.wotg_exp2_rate(None, None) == BAD
    # workspace queries of impossible shapes are 0
    assert lib.wotg_lse_points_workspace_bytes(0, 5, 4) == 0
    assert lib.wotg_lse_points_workspace_bytes(5, 5, 200) == 0
    # the status -> exception mapping of the reference
    with pytest.raises(ValueError):
        _native.check(BAD, 'x')
    with pytest.raises(ValueError):
        _native.check(_native.WOTG_WORKSPACE, 'x')
    with pytest.raises(RuntimeError, match='Overflow encountered in duality gap'):
        _native.check(_native.WOTG_NONFINITE, 'x')
    assert _native.check(_native.WOTG_MAX_ITER, 'x') == _native.WOTG_MAX_ITER


def test_synthetic_inputs_have_the_stated_distributions():
    """The seeded inputs every measurement uses: about 90 % zero counts,
    log1p(CP10k) values, lognormal(0, 0.3) growth, pure functions of the seed;
    course days are independent of the order they are generated in."""
    from wot_gb300 import synthetic
    X, day, g = synthetic.time_course([600, 700], n_genes=300, n_clusters=6, seed=3)
    assert X.shape == (1300, 300) and sorted(set(day.tolist())) == [0.0, 1.0]
    assert 0.85 <= float((X == 0).mean()) <= 0.95
    assert np.allclose(np.expm1(X).sum(axis=1)[np.expm1(X).sum(axis=1) > 0], 1e4, rtol=1e-9)
    lg = np.log(g)
    assert abs(lg.mean()) < 0.05 and abs(lg.std() - 0.3) < 0.03
    X2, day2, g2 = synthetic.time_course([600, 700], n_genes=300, n_clusters=6, seed=3)
    assert np.array_equal(X, X2) and np.array_equal(g, g2)
    prof = synthetic.course_profiles(5, n_genes=200, n_clusters=8, seed=1)
    a = [synthetic.course_day(prof, t, 300) for t in range(5)]
    b = [synthetic.course_day(prof, t, 300) for t in reversed(range(5))][::-1]
    for (xa, ga), (xb, gb) in zip(a, b):
        assert np.array_equal(xa, xb) and np.array_equal(ga, gb)
    assert 0.8 <= float(np.mean([(x == 0).mean() for x, _ in a])) <= 0.95
    sizes = synthetic.log_uniform_day_sizes(41)
    assert sizes.min() >= 1000 and sizes.max() <= 30000


def test_batch_item_statuses_follow_the_reference(caplog):
    """Per-item outcomes of a batched solve: max_iter items log the reference's
    warning (optimal_transport.py:143-145), a NaN duality gap raises its
    RuntimeError (:162-163) unless asked to keep the batch."""
    import logging
    from wot_gb300.ot.batch import report_statuses
    OK, MAXIT, NAN = _native.WOTG_OK, _native.WOTG_MAX_ITER, _native.WOTG_NONFINITE
    with caplog.at_level(logging.WARNING, logger='wot'):
        assert report_statuses([OK, MAXIT, OK]) == []
    assert any('Reached max_iter' in r.getMessage() for r in caplog.records)
    with pytest.raises(RuntimeError, match='Overflow encountered in duality gap.*items 1, 3'):
        report_statuses([OK, NAN, OK, NAN])
    assert report_statuses([NAN, OK], raise_nonfinite=False) == [0]
    with pytest.raises(RuntimeError, match='status 4'):
        report_statuses([_native.WOTG_CUDA_ERROR])


def test_otmodel_configuration_without_a_gpu(tmp_path, caplog):
    """OTModel's constructor and pair bookkeeping (wot/ot/ot_model.py:37-114,
    203-216) need no device: defaults and their precedence (kwargs, then the
    parameter file), solver choice, local_pca above the gene count, NaN days,
    day and cell filters, per-day subsampling, timepoints, the day_pairs check."""
    import logging
    import wot_gb300 as wot
    rng = np.random.default_rng(0)
    ids = np.array(['c%d' % i for i in range(12)])
    day = np.array([0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, np.nan])
    ds = Dataset(rng.random((12, 5)), Frame({'day': day}, index=ids), Frame(index=np.array(list('abcde'))))
    pf = tmp_path / 'params.txt'
    pf.write_text('epsilon\t0.02\n')
    with caplog.at_level(logging.WARNING, logger='wot'):
        m = wot.OTModel(ds, epsilon=0.1, lambda1=3, parameters=str(pf))
    assert any('Disabling PCA' in r.getMessage() for r in caplog.records)
    assert m.ot_config['local_pca'] == 0 and m.ot_config['epsilon'] == 0.02 and m.ot_config['lambda1'] == 3
    assert m.ot_config['lambda2'] == 50 and m.ot_config['tolerance'] == 1e-8 and m.ot_config['batch_size'] == 5
    assert m.timepoints == [0.0, 1.0, 2.0] and m.matrix.shape[0] == 11          # the NaN day is dropped
    assert m.solver is wot.ot.optimal_transport_duality_gap
    assert wot.OTModel(ds, solver='fixed_iters').solver is wot.ot.transport_stablev2
    with pytest.raises(ValueError, match='Unknown solver'):
        wot.OTModel(ds, solver='other')
    assert wot.OTModel(ds).pca == 'reference' and wot.OTModel(ds, pca='exact').pca == 'exact'
    assert 'pca' not in wot.OTModel(ds, pca='reference').ot_config
    with pytest.raises(ValueError, match='pca'):
        wot.OTModel(ds, pca='randomized')
    with pytest.raises(ValueError, match='Days information'):
        wot.OTModel(ds, day_field='time')
    assert wot.OTModel(ds, cell_day_filter='0,2').timepoints == [0.0, 2.0]
    kept = wot.OTModel(ds, cell_filter=['c1', 'c2', 'c5'])
    assert list(kept.matrix.obs.index) == ['c1', 'c2', 'c5']
    assert wot.OTModel(ds, gene_filter=['b', 'd']).matrix.X.shape[1] == 2
    sub = wot.OTModel(ds, ncells=2)
    assert sorted(np.unique(sub.matrix.obs['day'], return_counts=True)[1].tolist()) == [2, 2, 2]
    with pytest.raises(ValueError, match='No cells'):
        wot.OTModel(ds, cell_filter=['nobody'])
    cf = tmp_path / 'pairs.txt'
    cf.write_text('t0\tt1\tepsilon\n0\t1\t0.1\n')
    pairs = wot.OTModel(ds, config=str(cf))
    with pytest.raises(ValueError, match='not present in day_pairs'):
        pairs.compute_transport_map(1, 2)
    # covariate pairs and covariate-restricted selection (ot_model.py:116-122, 271-292)
    cv = np.array(['a', 'b', 'a', 'b', 'a', 'a', 'b', 'b', 'a', 'b', 'a', 'a'])
    dsc = Dataset(ds.X, Frame({'day': day, 'covariate': cv}, index=ids), ds.var)
    mc = wot.OTModel(dsc)
    assert sorted(mc.get_covariate_pairs()) == [('a', 'a'), ('a', 'b'), ('b', 'a'), ('b', 'b')]
    q0, q1 = mc.select_pair({'t0': 0, 't1': 1, 'covariate': ('b', 'a')})
    assert list(q0.obs.index) == ['c1', 'c3'] and list(q1.obs.index) == ['c4', 'c5']
    with pytest.raises(ValueError, match='Covariate'):
        list(m.get_covariate_pairs())
    # contiguous day rows are selected as views of X
    p0, p1 = m.select_pair({'t0': 0, 't1': 1, 'covariate': None})
    assert p0.X.base is not None and np.shares_memory(p0.X, m.matrix.X)
    assert p0.shape == (4, 5) and p1.shape == (4, 5)


def test_objective_helpers_match_the_reference_forms():
    """wot.ot.fdiv / fdivstar / primal / dual (optimal_transport.py:37-62): the
    device code (run here on CPU tensors) equals the oracle's NumPy restatement,
    zeros of R included; the public functions need a CUDA device."""
    import torch
    from oracle import optimal_transport as oot
    from wot_gb300.ot import optimal_transport as wot_ot
    rng = np.random.default_rng(3)
    I, J, eps, l1, l2 = 7, 9, 0.05, 1.0, 50.0
    C = rng.random((I, J))
    K = np.exp(-C / eps)
    a, b = rng.random(I) + 0.5, rng.random(J) + 0.5
    R = (K.T * a).T * b
    R[2, 3] = 0.0
    dx, dy = np.ones(I) / I, np.ones(J) / J
    p = rng.random(I) + 0.1
    q = np.ones(J) * p.mean()
    T = {k: torch.tensor(v) for k, v in dict(C=C, K=K, R=R, dx=dx, dy=dy, p=p, q=q, a=a, b=b).items()}
    ref_p = oot.primal(C, K, R, dx, dy, p, q, a, b, eps, l1, l2)
    ref_d = oot.dual(C, K, R, dx, dy, p, q, a, b, eps, l1, l2)
    got_p = float(wot_ot._primal(T['C'], T['K'], T['R'], T['dx'], T['dy'], T['p'], T['q'], eps, l1, l2))
    got_d = float(wot_ot._dual(T['K'], T['R'], T['dx'], T['dy'], T['p'], T['q'], T['a'], T['b'], eps, l1, l2))
    assert abs(got_p - ref_p) <= 1e-13 * abs(ref_p) and abs(got_d - ref_d) <= 1e-13 * abs(ref_d)
    x = R @ dy
    assert abs(float(wot_ot._fdiv(l1, T['R'] @ T['dy'], T['p'], T['dx'])) - oot.fdiv(l1, x, p, dx)) <= 1e-14
    u = rng.normal(size=I)
    assert abs(float(wot_ot._fdivstar(l1, torch.tensor(u), T['p'], T['dx'])) - oot.fdivstar(l1, u, p, dx)) <= 1e-14
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError, match='CUDA device'):
            wot_gb300.ot.primal(C, K, R, dx, dy, p, q, a, b, eps, l1, l2)


def test_fma_pipe_exp2_coefficients_meet_their_bound_on_cpu():
    """The FMA-pipe 2^z of the tensor-core epilogue (wotg_common.cuh::ex2_fma2),
    replayed in NumPy FP32 with the coefficients read from the header: the
    round-to-nearest reduction, the degree-5 Horner evaluation with one rounding
    per fused multiply-add, and the exact power of two stay within 3e-7 of
    2^z on [-125, 126] (the GPU test holds the kernel to the same bound)."""
    import re
    src = open(os.path.join(ROOT, 'wot_gb300', 'csrc', 'wotg_common.cuh')).read()
    body = src[src.index('float2 ex2_fma2(float2 z)'):]
    body = body[:body.index('return __fmul2_rn')]
    coef = [float(v) for v in re.findall(r'make_float2\(([0-9.e+-]+)f, \1f\)', body)]
    coef = [c for c in coef if abs(c) < 1e6]                 # drop the 1.5 * 2^23 shift constants
    assert len(coef) == 6                                    # c5 first (Horner order) ... c0
    z = np.concatenate([np.linspace(-125, 126, 1_000_003), np.linspace(-0.5, 0.5, 50_001)]).astype(np.float32)
    t = (z + np.float32(12582912.0)).astype(np.float32)
    n = (t - np.float32(12582912.0)).astype(np.float32)
    f = (z - n).astype(np.float32)
    p = np.float32(coef[0]) * np.ones_like(f)
    for ck in coef[1:]:
        p = (p.astype(np.float64) * f + np.float64(np.float32(ck))).astype(np.float32)   # one rounding per fma
    r = (p.astype(np.float64) * np.exp2(n.astype(np.float64))).astype(np.float32)
    ref = np.exp2(z.astype(np.float64))
    assert np.abs(r.astype(np.float64) / ref - 1).max() <= 3e-7
