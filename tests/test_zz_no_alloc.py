"""fhp_energy_matrix_noalloc (fixed in-library scratch, nothing allocated)
against fhp_energy_matrix of a plan holding the same coefficient.

Collected last on purpose: it must also hold after every other GPU test has
run in the same process (library module loaded, torch's allocator warm)."""
import ctypes

import numpy as np
import pytest

from ffthompy_gb300 import _lib

# dim, grid, physics, dv, loads, coefficient kind
CASES = [
    (3, (7, 8, 9), _lib.FHP_SCALAR, 3, 3, _lib.FHP_COEF_ISO),
    (2, (15, 12), _lib.FHP_SCALAR, 2, 2, _lib.FHP_COEF_FULL),
    (3, (5, 6, 7), _lib.FHP_ELASTICITY, 6, 6, _lib.FHP_COEF_SYM),
    (3, (64, 64, 63), _lib.FHP_SCALAR, 3, 3, _lib.FHP_COEF_SYM),  # hundreds of blocks
]


def _ncoef(kind, dv):
    return {_lib.FHP_COEF_ISO: 1, _lib.FHP_COEF_SYM: dv * (dv + 1) // 2,
            _lib.FHP_COEF_FULL: dv * dv}[kind]


def _call_noalloc(lib, dim, N, dv, loads, kind, A, X, add_macro, AH, stream):
    n = (ctypes.c_int * dim)(*N)
    return lib.fhp_energy_matrix_noalloc(dim, n, dv, loads, kind, ctypes.c_void_p(A),
                                         ctypes.c_void_p(X), add_macro, ctypes.c_void_p(AH),
                                         ctypes.c_void_p(stream))


@pytest.mark.gpu
@pytest.mark.parametrize('case', CASES, ids=lambda c: '%dd_%s_k%d' % (c[0], 'x'.join(map(str, c[1])), c[5]))
def test_noalloc_energy_matches_plan_energy(case):
    import torch
    assert torch.cuda.is_available()
    lib = _lib.load()
    dim, N, physics, dv, loads, kind = case
    rng = np.random.default_rng(sum(N) + kind)
    M = int(np.prod(N))
    A_host = rng.uniform(0.5, 2.0, (_ncoef(kind, dv),) + N)
    X_host = rng.standard_normal((loads, dv) + N)
    dev = torch.device('cuda:0')
    A = torch.from_numpy(A_host).to(dev)
    X = torch.from_numpy(X_host).to(dev)
    stream = torch.cuda.current_stream().cuda_stream

    plan = ctypes.c_void_p()
    n = (ctypes.c_int * dim)(*N)
    Y = (ctypes.c_double * dim)(*([1.0] * dim))
    _lib.check(lib.fhp_plan_create(ctypes.byref(plan), dim, n, n, Y, physics, loads, 1.0,
                                   _lib.FHP_F64), 'plan')
    try:
        _lib.check(lib.fhp_set_coefficient(plan, kind, ctypes.c_void_p(A.data_ptr()), 1,
                                           ctypes.c_void_p(stream)), 'coefficient')
        for add_macro in (1, 0):
            ref = np.zeros((loads, loads))
            _lib.check(lib.fhp_energy_matrix(plan, ctypes.c_void_p(X.data_ptr()), add_macro,
                                             ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             ctypes.c_void_p(stream)), 'energy')
            # two calls in a row into the same output: the scratch is reused
            AH = torch.full((loads * loads,), float('nan'), dtype=torch.float64, device=dev)
            for _ in range(2):
                AH.fill_(float('nan'))
                _lib.check(_call_noalloc(lib, dim, N, dv, loads, kind, A.data_ptr(),
                                         X.data_ptr(), add_macro, AH.data_ptr(), stream),
                           'energy (no alloc)')
                torch.cuda.synchronize()
                got = AH.cpu().numpy().reshape(loads, loads)
                assert np.all(np.isfinite(got))
                scale = np.abs(ref).max()
                assert np.abs(got - ref).max() <= 1e-12 * scale, (got, ref)
            assert M > 0
    finally:
        lib.fhp_plan_destroy(plan)


def test_noalloc_energy_rejects_sizes_beyond_its_scratch():
    """Argument checks happen before any CUDA call (runs without a GPU)."""
    import __graft_entry__
    __graft_entry__.build()
    lib = _lib.load()
    dummy = 16  # never dereferenced: the checks fail first
    assert _call_noalloc(lib, 3, (4, 4, 4), 3, 7, _lib.FHP_COEF_ISO, dummy, dummy, 1, dummy,
                         None) == _lib.FHP_BAD_ARG
    assert b'6 x 6' in lib.fhp_last_error()
    assert _call_noalloc(lib, 3, (4, 4, 4), 7, 3, _lib.FHP_COEF_ISO, dummy, dummy, 1, dummy,
                         None) == _lib.FHP_BAD_ARG
    assert _call_noalloc(lib, 3, (4, 4, 4), 3, 3, 9, dummy, dummy, 1, dummy,
                         None) == _lib.FHP_BAD_ARG
    assert _call_noalloc(lib, 3, (4, 0, 4), 3, 3, _lib.FHP_COEF_ISO, dummy, dummy, 1, dummy,
                         None) == _lib.FHP_BAD_ARG
