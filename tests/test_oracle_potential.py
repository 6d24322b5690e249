"""Pin the oracle's potential formulation against the reference (no GPU).

Fixtures tests/golden/pot_*.npz come from the reference's own
homog_GaNi_full_potential / homog_Ga_full_potential
(ffthompy/tensorsLowRank/homogenisation.py:41-127) and from its operator
PDFAFGPfun assembled from the reference's grad, div, DFT, enlarge and project.
"""
import numpy as np
import pytest

import golden_io
import oracle

POT = golden_io.names('pot_')


def _coef(arr, key):
    return arr['A_ga'] if key == 'ga' else arr['A_gani']


@pytest.mark.parametrize('name', POT)
def test_oracle_potential_operator(name):
    meta, arr = golden_io.load(name)
    N = tuple(meta['N'])
    Y = np.array(meta['Y'])
    y = oracle.potential_operator(arr['A_gani'], N, Y)(arr['x'])
    ref = arr['y__gani']
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
    if 'y__ga' in arr:
        Nbar = tuple(2 * n - 1 for n in N)
        y = oracle.potential_operator(arr['A_ga'], N, Y, Nbar)(arr['x'])
        ref = arr['y__ga']
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize('name', POT)
def test_oracle_potential_solve(name):
    meta, arr = golden_io.load(name)
    N = tuple(meta['N'])
    Y = np.array(meta['Y'])
    for key in meta['runs']:
        kw = {}
        if key == 'ga':
            kw['Nbar'] = tuple(2 * n - 1 for n in N)
        if key == 'gani_ga':
            kw['A_post'] = arr['A_ga']
        out = oracle.homog_potential(_coef(arr, key), N, Y, meta['tol'], meta['maxiter'], **kw)
        assert out['info']['kit'] == int(arr['kit__' + key]), key
        assert abs(out['AH'] - float(arr['AH__' + key])) <= 1e-12 * abs(float(arr['AH__' + key]))
        ref = arr['Fu__' + key]
        assert np.abs(out['Fu'] - ref).max() <= 1e-10 * np.abs(ref).max(), key
