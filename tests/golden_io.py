"""Load the golden fixtures of tests/golden/ (written by make_golden.py)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _decode(v):
    if isinstance(v, dict):
        if '__nd__' in v:
            return np.array(v['__nd__'], dtype=v['dtype'])
        return {k: _decode(x) for k, x in v.items()}
    if isinstance(v, list):
        return [_decode(x) for x in v]
    return v


def names(prefix):
    return sorted(os.path.basename(p)[:-4]
                  for p in glob.glob(os.path.join(GOLDEN, prefix + '*.npz')))


def load(name):
    """Return (meta, arrays) of one fixture."""
    z = np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False)
    meta = _decode(json.loads(str(z['meta'])))
    arrays = {k: z[k] for k in z.files if k != 'meta'}
    return meta, arrays


def problem(name):
    """Problem dictionary (reference input-file layout) + expected outputs."""
    meta, arrays = load(name)
    material = dict(meta['material'])
    if meta.get('has_fun'):
        values = arrays['fun_values']

        def fun(coord, _v=values):
            return _v.copy()
        material['fun'] = fun
    if 'positions' in material:
        material['positions'] = [np.asarray(p) if isinstance(p, np.ndarray) else p
                                 for p in material['positions']]
    prob = {'name': name, 'physics': meta['physics'], 'material': material,
            'solve': meta['solve'], 'solver': meta['solver'],
            'postprocess': meta['postprocess']}
    expected = {'mat': {}, 'kit': {}, 'normres': {}, 'sol': {}}
    for k, v in arrays.items():
        parts = k.split('__')
        if parts[0] == 'mat':
            expected['mat'].setdefault(parts[1], {})[parts[2]] = v
        elif parts[0] in ('kit', 'normres', 'sol'):
            expected[parts[0]][parts[1]] = v
    return prob, expected
