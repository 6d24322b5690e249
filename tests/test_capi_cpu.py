"""C ABI exports and host logic (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'ffthompy_gb300.h')


def _declared():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(fhp_[a-z_0-9]+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from ffthompy_gb300 import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    from ffthompy_gb300 import _lib
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_status_strings_and_bad_args(lib):
    assert lib.fhp_version() == 100
    assert lib.fhp_status_string(0) == b'ok'
    h = ctypes.c_void_p()
    n = (ctypes.c_int * 2)(5, 5)
    y = (ctypes.c_double * 2)(1., 1.)
    # invalid arguments are rejected before any CUDA call
    assert lib.fhp_plan_create(ctypes.byref(h), 4, n, n, y, 0, 2, 1.0, 0) == 5
    assert lib.fhp_plan_create(ctypes.byref(h), 2, n, n, y, 7, 2, 1.0, 0) == 5
    assert lib.fhp_plan_create(ctypes.byref(h), 2, n, n, y, 0, 2, -1.0, 0) == 5
    assert lib.fhp_plan_create(None, 2, n, n, y, 0, 2, 1.0, 0) == 5
    # plans of several cells: 1..65535 cells
    assert lib.fhp_plan_create_cells(ctypes.byref(h), 2, n, n, y, 0, 2, 1.0, 0, 0) == 5
    assert lib.fhp_plan_create_cells(ctypes.byref(h), 2, n, n, y, 0, 2, 1.0, 0, 65536) == 5
    assert lib.fhp_plan_cells(None) == 0
    assert lib.fhp_homogenize_host_many(None, 1, 1, 1, None, 1e-6, 10, None, None, None,
                                        None) == 5
    assert lib.fhp_apply(None, 1, None, None, None) == 5
    assert b'required' in lib.fhp_last_error()


def test_material_assembly_needs_cuda():
    """Coefficient assembly runs on the GPU only: without CUDA it raises
    instead of falling back to the host."""
    import torch
    from ffthompy_gb300.materials import Material
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    m = Material({'inclusions': ['cube', 'otherwise'], 'positions': [np.zeros(2), ''],
                  'params': [np.full(2, 0.5), ''], 'vals': [np.eye(2) * 5., np.eye(2)],
                  'Y': np.ones(2), 'order': None})
    with pytest.raises(RuntimeError):
        m.get_A_GaNi(np.array([5, 5]))
    with pytest.raises(RuntimeError):
        m.get_A_Ga(np.array([9, 9]))


def test_elastic_tensor_mandel():
    from ffthompy_gb300.mechanics.matcoef import ElasticTensor
    import oracle
    for K, mu in ((1., 1.), (10., 5.), (0.8333, 0.3846)):
        np.testing.assert_allclose(ElasticTensor(bulk=K, mu=mu).mandel,
                                   oracle.mandel_isotropic(K, mu), atol=1e-13)
        np.testing.assert_allclose(ElasticTensor(bulk=K, mu=mu, plane='strain').mandel,
                                   oracle.mandel_isotropic(K, mu, dim=2), atol=1e-13)


def test_coefficient_classification():
    from ffthompy_gb300.engine import coef_kind_of, pack_coefficient
    from ffthompy_gb300 import _lib
    a = np.random.default_rng(0).random((4, 5))
    iso = np.einsum('ij,...->ij...', np.eye(3), a)
    assert coef_kind_of(iso) == _lib.FHP_COEF_ISO
    sym = iso.copy()
    sym[0, 1] = sym[1, 0] = a
    assert coef_kind_of(sym) == _lib.FHP_COEF_SYM
    assert pack_coefficient(sym, _lib.FHP_COEF_SYM).shape == (6, 4, 5)
    full = sym.copy()
    full[0, 2] = 1.
    assert coef_kind_of(full) == _lib.FHP_COEF_FULL
    assert pack_coefficient(full, _lib.FHP_COEF_FULL).shape == (9, 4, 5)


def test_line_plans_factor_configured_sizes():
    """Every configured grid length factors into supported radices or gets a
    Bluestein length that does (checked against the C++ planner's rules)."""
    def factor(n):
        for p in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31):
            while n % p == 0:
                n //= p
        return n == 1
    for n in (5, 9, 15, 29, 45, 63, 89, 125, 127, 253, 255, 509, 511, 1021):
        if not factor(n):
            m = 2 * n - 1
            while not factor(m) or any(m % p == 0 for p in (7, 11, 13, 17, 19, 23, 29, 31)):
                m += 1
            assert m <= 4096


def test_ball_entry_points_reject_bad_arguments(lib):
    """fhp_ball_topology / fhp_ball_characteristic check their arguments
    before any CUDA call."""
    from ffthompy_gb300 import _lib
    n = (ctypes.c_int * 3)(5, 5, 5)
    t = (ctypes.c_double * 15)(*range(15))
    x0 = (ctypes.c_double * 3)(0., 0., 0.)
    Y = (ctypes.c_double * 3)(1., 1., 1.)
    out = ctypes.c_void_p(1 << 20)
    bad = _lib.FHP_BAD_ARG
    assert lib.fhp_ball_topology(4, n, t, x0, Y, 0.2, out, None) == bad
    assert lib.fhp_ball_topology(1, n, t, x0, Y, 0.2, out, None) == bad
    assert lib.fhp_ball_topology(3, n, None, x0, Y, 0.2, out, None) == bad
    z = (ctypes.c_int * 3)(5, 0, 5)
    assert lib.fhp_ball_topology(3, z, t, x0, Y, 0.2, out, None) == bad
    assert lib.fhp_ball_characteristic(None, 0.2, 1.0, t, t, out, None) == bad


def test_outer_accumulate_rejects_bad_arguments(lib):
    from ffthompy_gb300 import _lib
    v = (ctypes.c_double * 40)(*range(40))
    c = ctypes.c_void_p(1 << 20)
    out = ctypes.c_void_p(1 << 30)
    bad = _lib.FHP_BAD_ARG
    assert lib.fhp_outer_accumulate(0, v, c, out, 100, None) == bad
    assert lib.fhp_outer_accumulate(37, v, c, out, 100, None) == bad
    assert lib.fhp_outer_accumulate(4, v, c, out, 0, None) == bad
    assert lib.fhp_outer_accumulate(4, None, c, out, 100, None) == bad
    assert lib.fhp_outer_accumulate(4, v, c, c, 100, None) == bad      # overlap
