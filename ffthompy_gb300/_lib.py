"""ctypes binding of libffthompy_gb300.so (C ABI in include/ffthompy_gb300.h).

The library is loaded from ffthompy_gb300/_lib/ (built in-tree by
ffthompy_gb300/build.py).  There is no CPU fallback: if the library is
missing or CUDA is unavailable, every entry point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'libffthompy_gb300.so')

FHP_OK, FHP_NONCONVERGED, FHP_BREAKDOWN, FHP_NONFINITE, FHP_TIMEOUT, FHP_BAD_ARG, \
    FHP_OOM, FHP_CUDA = range(8)
FHP_F64, FHP_F32, FHP_MIXED = 0, 1, 2
FHP_SCALAR, FHP_ELASTICITY = 0, 1
FHP_COEF_ISO, FHP_COEF_SYM, FHP_COEF_FULL = 1, 2, 3

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_ll_p = ctypes.POINTER(ctypes.c_longlong)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); the exported C ABI
SIGNATURES = {
    'fhp_version': (ctypes.c_int, []),
    'fhp_status_string': (ctypes.c_char_p, [ctypes.c_int]),
    'fhp_last_error': (ctypes.c_char_p, []),
    'fhp_plan_create': (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _c_int_p, _c_int_p,
                                       _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int]),
    'fhp_plan_create_band': (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _c_int_p,
                                            _c_int_p, _c_double_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_int]),
    'fhp_plan_create_cells': (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _c_int_p,
                                             _c_int_p, _c_double_p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    'fhp_plan_cells': (ctypes.c_int, [_vp]),
    'fhp_plan_destroy': (ctypes.c_int, [_vp]),
    'fhp_plan_set_refinement': (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int]),
    'fhp_plan_set_band_cg': (ctypes.c_int, [_vp, ctypes.c_int]),
    'fhp_cg_solve_many': (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp), ctypes.c_int,
                                          ctypes.POINTER(_vp), ctypes.c_double, ctypes.c_int,
                                          ctypes.POINTER(_vp), _c_int_p, _c_double_p, _c_int_p,
                                          _vp]),
    'fhp_plan_set_integration_kernel': (ctypes.c_int, [_vp, ctypes.c_int]),
    'fhp_separable_char': (ctypes.c_int, [ctypes.c_int, _c_int_p, _c_double_p, _c_double_p, _vp,
                                          _vp]),
    'fhp_plan_autotune': (ctypes.c_int, [_vp, _c_int_p, ctypes.POINTER(ctypes.c_float), _vp]),
    'fhp_richardson_solve': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int, _vp, _c_int_p,
                                            _c_double_p, _c_int_p, _vp]),
    'fhp_chebyshev_solve': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp,
                                           _c_int_p, _c_double_p, _c_int_p, _vp]),
    'fhp_bicg_solve': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                      _vp, _c_int_p, _c_double_p, _c_int_p, _vp]),
    'fhp_plan_query': (ctypes.c_int, [_vp, _c_ll_p, _c_int_p, _c_int_p, _c_int_p]),
    'fhp_set_coefficient': (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, _vp]),
    'fhp_apply': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    'fhp_rhs_macro': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    'fhp_cg_solve': (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                    _vp, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                                    ctypes.c_int, _vp]),
    'fhp_energy_matrix': (ctypes.c_int, [_vp, _vp, ctypes.c_int, _c_double_p, _vp]),
    'fhp_fourier_interp': (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    'fhp_energy_gradient': (ctypes.c_int, [_vp, _vp, ctypes.c_int, _c_double_p, _vp, _vp]),
    'fhp_homogenize_host': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_double,
                                           ctypes.c_int, _c_double_p, _c_int_p, _c_double_p, _vp,
                                           _vp]),
    'fhp_homogenize_host_many': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(_vp), ctypes.c_double, ctypes.c_int,
                                                _c_double_p, _c_int_p, _c_double_p, _vp]),
    'fhp_fft_plan_create': (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _c_int_p,
                                           ctypes.c_int, ctypes.c_int]),
    'fhp_ga_grid_coefficient': (ctypes.c_int, [_vp, _vp, _vp, _c_int_p, _c_double_p, _vp, _vp]),
    'fhp_coefficient_inverse': (ctypes.c_int, [ctypes.c_int, _c_int_p, ctypes.c_int, _vp, _vp,
                                               ctypes.c_int, _vp]),
    'fhp_ball_characteristic': (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double,
                                               _c_double_p, _c_double_p, _vp, _vp]),
    'fhp_outer_accumulate': (ctypes.c_int, [ctypes.c_int, _c_double_p, _vp, _vp,
                                            ctypes.c_longlong, _vp]),
    'fhp_ball_topology': (ctypes.c_int, [ctypes.c_int, _c_int_p, _c_double_p, _c_double_p,
                                         _c_double_p, ctypes.c_double, _vp, _vp]),
    'fhp_profile_enable': (ctypes.c_int, [_vp, ctypes.c_int]),
    'fhp_profile_read': (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, _c_ll_p,
                                        _c_double_p, _c_double_p, _c_int_p]),
    'fhp_plan_launches': (ctypes.c_longlong, [_vp]),
    'fhp_potential_rhs': (ctypes.c_int, [_vp, _vp, _vp]),
    'fhp_potential_apply': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'fhp_potential_cg': (ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_int, _vp, _c_int_p,
                                        _c_double_p, _c_int_p, _c_double_p, ctypes.c_int, _vp]),
    'fhp_potential_field': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'fhp_energy_matrix_noalloc': (ctypes.c_int, [ctypes.c_int, _c_int_p, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, _vp, _vp,
                                                 ctypes.c_int, _vp, _vp]),
}

_lib = None


class FhpError(RuntimeError):
    """A failed call into the CUDA library."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def load():
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError('libffthompy_gb300.so is not built (%s); run '
                          'python -m ffthompy_gb300.build' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, what=''):
    """Raise for a non-OK status, with the library's error message."""
    if status == FHP_OK:
        return
    lib = load()
    msg = '%s: %s (%s)' % (what, lib.fhp_status_string(status).decode(),
                           lib.fhp_last_error().decode())
    if status == FHP_BAD_ARG:
        raise ValueError(msg)
    raise FhpError(status, msg)
