"""The benchmark's JSON contract, checked on the CPU: the reference arm (the
oracle on a bounded sample of the pair workload) prints one line with the
keys the contract names, and the course and summary helpers are consistent."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, OPENBLAS_NUM_THREADS='4', OMP_NUM_THREADS='4')
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                          '--warmup', '0'], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ('impl', 'metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better',
                'scaling', 'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e'):
        assert key in line, key
    assert line['impl'] == 'reference' and line['value'] > 0 and line['higher_is_better'] is True
    cb = line['cpu_baseline']
    assert cb['kind'] in ('reference', 'port') and cb['cores'] >= 1 and cb['value'] == line['value']
    assert line['e2e'] == {'value': line['value'], 'unit': line['unit'], 'h2d_bytes_per_step': 0,
                           'd2h_bytes_per_step': 0}
    assert line['config']['I'] == 20000 and line['config']['J'] == 25000


def test_course_items_and_summary():
    sys.path.insert(0, ROOT)
    import bench
    sizes, shapes, items = bench.course_items(41)
    assert len(shapes) == 40 and len(items) == 1000
    assert all(0 <= p < 40 for p, _ in items)
    assert sorted({(c['epsilon'], c['lambda1']) for _, c in items}) == sorted(
        (e, l) for e in bench.COURSE_EPS for l in bench.COURSE_L1)
    s = bench.summary_of({'value': 3.5, 'e2e': {'value': 2.0}, 'parity_full': {'onthefly': {'x': 1}, 'shape': [1]}})
    assert s['pair_maps_per_s'] == 3.5 and s['pair_e2e'] == 2.0 and s['pair_parity_full'] == {'onthefly': {'x': 1}}
