"""The other linear solvers of linear_solver (ffthompy/general/solver.py:
63-77, 142-204, 206-285) over the fused GPU operator, through the reference's
Tensor / Operator API: Chebyshev against the reference's own runs
(tests/golden/solv_*.npz), BiCG and Richardson against the oracle.

Tolerances: iteration counts equal; solutions to 1e-10 of their max (the
recurrences are the same, only FFT roundoff differs)."""
import numpy as np
import pytest

import golden_io
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

SOLV = golden_io.names('solv_')


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _setup(meta, arr):
    import ffthompy_gb300.projections as proj
    from ffthompy_gb300.tensors import DFT, Operator, Tensor
    N = np.array(meta['N'])
    d = N.size
    Nbar = np.array(meta['Nbar'])
    _, G1, _ = proj.scalar(N, np.ones(d), NyqNul=True, tensor=True)
    if meta['kind'] == 'Ga':
        G1 = G1.enlarge(Nbar)
    FN = DFT(name='FN', inverse=False, N=Nbar)
    FiN = DFT(name='FiN', inverse=True, N=Nbar)
    A = Tensor(name='A', val=arr['A'], order=2, multype=21)
    Afun = Operator(name='FiGFA', mat=[[Operator(name='G', mat=[[FiN, G1, FN]]), A]])
    B = Tensor(name='B', val=arr['B'], order=1)
    x0 = Tensor(N=tuple(Nbar), shape=(d,), Fourier=False)
    return Afun, B, x0


def _oracle_afun(meta, arr):
    N = np.array(meta['N'])
    G, _ = oracle.green_operator('scalar', N, np.ones(N.size), meta['kind'], 1)
    return lambda v: oracle.apply_GA(G, arr['A'], v)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize('name', SOLV)
def test_chebyshev_matches_reference(name):
    from ffthompy_gb300.general.solver import linear_solver
    meta, arr = golden_io.load(name)
    Afun, B, x0 = _setup(meta, arr)
    X, info = linear_solver(Afun, B, x0=x0, par=dict(meta['chebyshev']), solver='chebyshev')
    assert info['kit'] == int(arr['kit__chebyshev'])
    assert abs(info['norm_res'] - float(arr['normres__chebyshev'])) <= 1e-9
    assert _rel(X.val, arr['x__chebyshev']) < 1e-10


@pytest.mark.parametrize('name', SOLV)
def test_bicg_and_richardson_match_oracle(name):
    from ffthompy_gb300.general.solver import linear_solver
    meta, arr = golden_io.load(name)
    Afun, B, x0 = _setup(meta, arr)
    Af = _oracle_afun(meta, arr)
    X, info = linear_solver(Afun, B, ATfun=Afun, x0=x0, par={'tol': 1e-8, 'maxiter': 300},
                            solver='bicg')
    xo, io = oracle.bicg(Af, Af, arr['B'], np.zeros_like(arr['B']), 1e-8, 300)
    assert info['kit'] == io['kit']
    assert _rel(X.val, xo) < 1e-10
    # Richardson with omega = 1/alpha, alpha = the upper end of the spectrum
    alpha = meta['chebyshev']['eigrange'][1]
    X, info = linear_solver(Afun, B, x0=x0, par={'tol': 1e-6, 'maxiter': 5000, 'alpha': alpha},
                            solver='richardson')
    x = np.zeros_like(arr['B'])
    kit, nr = 0, 1e15
    while nr > 1e-6 and kit < 5000:
        kit += 1
        r = arr['B'] - Af(x)
        x = x + r / alpha
        nr = oracle.scal(r, r) ** 0.5
    assert info['kit'] == kit
    assert _rel(X.val, x) < 1e-9
