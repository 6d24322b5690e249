"""Pin the oracle's other linear solvers (no GPU): the two-term Chebyshev
iteration against the reference's own linear_solver(solver='chebyshev')
runs (tests/golden/solv_*.npz, ffthompy/general/solver.py:206-285), and
BiCG (solver.py:142-204, which does not run on the reference's Tensor
objects as shipped) through its defining property: with ATfun = Afun on the
symmetric FiGFA it reproduces CG iterate for iterate."""
import numpy as np
import pytest

import golden_io
import oracle

SOLV = golden_io.names('solv_')


def _afun(meta, arr):
    N = np.array(meta['N'])
    G, _ = oracle.green_operator('scalar', N, np.ones(N.size), meta['kind'], 1)
    return lambda v: oracle.apply_GA(G, arr['A'], v)


@pytest.mark.parametrize('name', SOLV)
def test_oracle_chebyshev_matches_reference(name):
    meta, arr = golden_io.load(name)
    c = meta['chebyshev']
    x, info = oracle.cheby2term(_afun(meta, arr), arr['B'], np.zeros_like(arr['B']),
                                c['eigrange'], c['tol'], c['maxit'])
    assert info['kit'] == int(arr['kit__chebyshev'])
    assert abs(info['norm_res'] - float(arr['normres__chebyshev'])) <= 1e-12
    np.testing.assert_allclose(x, arr['x__chebyshev'], rtol=0, atol=1e-12)


@pytest.mark.parametrize('name', SOLV)
def test_oracle_bicg_symmetric_is_cg(name):
    meta, arr = golden_io.load(name)
    A = _afun(meta, arr)
    x0 = np.zeros_like(arr['B'])
    xb, ib = oracle.bicg(A, A, arr['B'], x0, 1e-8, 300)
    xc, ic = oracle.cg(A, arr['B'], x0, 1e-8, 300)
    assert ib['kit'] == ic['kit']
    np.testing.assert_allclose(xb, xc, rtol=0, atol=1e-12)
