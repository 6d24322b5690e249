"""The oracle's per-voxel inverse (get_inverse, ffthompy/trigpol.py:120-159)
against the reference's own outputs (tests/golden/inv_*.npz): bit-identical,
including the Inf / NaN of zero pivots; and the C ABI entry point's argument
checks, which return before any CUDA call."""
import ctypes
import warnings

import numpy as np
import pytest

import golden_io
import oracle

INV = golden_io.names('inv_')


def test_inverse_fixtures_exist():
    assert len(INV) >= 5


@pytest.mark.parametrize('name', INV)
def test_oracle_inverse_is_bit_identical_to_reference(name):
    _, arr = golden_io.load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        inv = oracle.get_inverse(arr['A'])
    np.testing.assert_array_equal(inv, arr['inv'])
    if 'zero_pivot' in name:
        assert not np.isfinite(arr['inv']).all()


def test_host_get_inverse_matches_reference():
    """The package's host restatement (used where no GPU is present)."""
    from ffthompy_gb300.materials import get_inverse
    for name in INV:
        _, arr = golden_io.load(name)
        with warnings.catch_warnings():
            warnings.simplefilter('ignore')
            np.testing.assert_array_equal(get_inverse(arr['A']), arr['inv'])


def test_coefficient_inverse_rejects_bad_arguments():
    import __graft_entry__
    __graft_entry__.build()
    from ffthompy_gb300 import _lib
    lib = _lib.load()
    n = (ctypes.c_int * 3)(4, 4, 4)
    a = ctypes.c_void_p(1 << 20)
    b = ctypes.c_void_p(1 << 30)
    bad = _lib.FHP_BAD_ARG
    assert lib.fhp_coefficient_inverse(3, n, 7, a, b, 0, None) == bad        # d > 6
    assert lib.fhp_coefficient_inverse(3, n, 0, a, b, 0, None) == bad
    assert lib.fhp_coefficient_inverse(4, n, 3, a, b, 0, None) == bad        # dim > 3
    assert lib.fhp_coefficient_inverse(3, n, 3, a, a, 0, None) == bad        # in place
    assert lib.fhp_coefficient_inverse(3, n, 3, a, ctypes.c_void_p((1 << 20) + 8), 1,
                                       None) == bad                            # overlap
    assert b'overlap' in lib.fhp_last_error()
    assert lib.fhp_coefficient_inverse(3, n, 3, None, b, 0, None) == bad
    z = (ctypes.c_int * 3)(4, 0, 4)
    assert lib.fhp_coefficient_inverse(3, z, 3, a, b, 0, None) == bad
