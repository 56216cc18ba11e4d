"""Per-pair configuration parsing (wot/ot/initializer.py:42-183).

Only ``epsilon``, ``lambda1`` and ``lambda2`` survive per-pair parsing, as in
the reference. DataFrame inputs need pandas; dict inputs and 2-column text
files work without it.
"""
from __future__ import annotations


def parse_configuration(config):
    """None | path | DataFrame | dict -> {(t0, t1): {...}} or None (:42-81)."""
    if config is None:
        return None
    if isinstance(config, str):
        return parse_configuration(read_day_pairs(config))
    if hasattr(config, 'columns'):
        cols = list(config.columns)
        if 't' in cols:
            return parse_per_timepoint_configuration(config)
        if 't0' in cols and 't1' in cols:
            return parse_per_timepair_configuration(config)
        raise ValueError("Configuration must have at least a column 't' or two columns 't0' and 't1'")
    if isinstance(config, dict):
        raise ValueError("Not implemented")
    raise ValueError("Unrecognized argument type for configuration. Use DataFrame, dict, str or None")


def parse_per_timepoint_configuration(config):
    """Average per-timepoint parameters over consecutive pairs (:84-123)."""
    if not hasattr(config, 'columns'):
        if isinstance(config, dict):
            raise ValueError("Not implemented")
        raise ValueError("Unrecognized argument type for per-timepoint configuration. Use DataFrame, str or None")
    if 't' not in config.columns:
        raise ValueError("Invalid per-timepoint configuration : must have column t")
    types = ('t', 'epsilon', 'lambda1', 'lambda2')
    rows = sorted(_records(config), key=lambda r: float(r['t']))
    fields = [x for x in config.columns if x != 't' and x in types]
    day_pairs = {}
    for i in range(len(rows) - 1):
        a, b = rows[i], rows[i + 1]
        day_pairs[(float(a['t']), float(b['t']))] = {x: (float(a[x]) + float(b[x])) / 2 for x in fields}
    return day_pairs


def parse_per_timepair_configuration(config):
    """Validate a per-pair table / dict, keep epsilon, lambda1, lambda2 (:135-183)."""
    if hasattr(config, 'columns'):
        if 't0' not in config.columns or 't1' not in config.columns:
            raise ValueError("Invalid per-timepair configuration : must have columns t0 and t1")
        result = {}
        for h in _records(config):
            h = dict(h)
            t0, t1 = h.pop('t0'), h.pop('t1')
            result[(t0, t1)] = h
        return parse_per_timepair_configuration(result)
    if isinstance(config, dict):
        try:
            if not all(isinstance(z, (int, float)) for x, y in config for z in [x, y]):
                raise ValueError("Dictionary keys for config must be pairs of floats")
        except Exception:
            raise ValueError("Dictionnary keys for config must be pairs")
        valid_fields = ['epsilon', 'lambda1', 'lambda2']
        for key in config:
            if not isinstance(config[key], dict):
                raise ValueError("Dictionnary values for config must be dictionnaries")
            selected = config[key]
            config[key] = {x: selected[x] for x in valid_fields if x in selected}
        return config
    raise ValueError("Unrecognized argument type for config. Use DataFrame or dict")


def parse_parameter_file(path):
    """Two-column (name, value) file (:126-132); separator sniffed like pandas' sep=None."""
    result = {}
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            parts = line.split('\t') if '\t' in line else (line.split(',') if ',' in line else line.split())
            result[parts[0].strip()] = _number(parts[1].strip())
    return result


def read_day_pairs(spec):
    """Day-pair table (wot/io/io.py:548-556) as a list-of-records table: a file
    (separator sniffed), or an inline table with ',' between fields and ';'
    between rows, e.g. 't0,t1,epsilon;0,1,0.05;1,2,0.1'. A table without a
    t / t0 / t1 header row is read as (t0, t1) pairs."""
    import os
    from ..dataset import Frame
    if os.path.isfile(spec):
        with open(spec) as f:
            lines = [ln.rstrip('\n') for ln in f if ln.strip()]
        sep = '\t' if '\t' in lines[0] else (',' if ',' in lines[0] else None)
    else:
        lines = [r.strip() for r in str(spec).split(';') if r.strip()]
        sep = ','
    if not lines:
        raise ValueError('empty day-pair table')
    header = lines[0].split(sep)
    if not any(h in ('t', 't0', 't1') for h in header):
        header = ['t0', 't1']
        body = lines
    else:
        body = lines[1:]
    cols = {h: [] for h in header}
    for ln in body:
        for h, v in zip(header, ln.split(sep)):
            cols[h].append(_number(v))
    return _TableWrap(Frame(cols))


class _TableWrap:
    def __init__(self, frame):
        self.frame = frame
        self.columns = frame.columns

    def __len__(self):
        return len(self.frame)


def _records(table):
    if isinstance(table, _TableWrap):
        f = table.frame
        return [{c: f[c][i].item() for c in f.columns} for i in range(len(f))]
    if hasattr(table, 'to_dict'):
        try:
            return table.to_dict(orient='records')
        except TypeError:
            pass
    f = table
    return [{c: f[c][i] for c in f.columns} for i in range(len(f))]


def _number(v):
    try:
        f = float(v)
        return int(f) if f.is_integer() and '.' not in str(v) and 'e' not in str(v).lower() else f
    except ValueError:
        return v
