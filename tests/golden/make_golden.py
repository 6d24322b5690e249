"""Generate the golden fixtures under tests/golden/ from the FFTHomPy reference.

This script is the only place that runs the reference.  It imports the
unmodified reference package from the directory given as its first argument
(or, with no argument, from the environment variable FFTHOMPY_REFERENCE),
with a small runtime shim for the NumPy/SciPy/Python names it still uses
(np.int/np.float/np.complex, time.clock, collections.Callable,
scipy.setdiff1d).  It writes plain .npz files (arrays + a JSON metadata
string), so the tests never need the reference at run time.

Fixture families
----------------
ref_<file>_<prob>.npz
    The reference's own golden pickles test_results/python3/<file>_<prob>
    (compared by run_unittests.py:57-64 at delta 1e-9), flattened: the
    problem definition stored in the pickle, the homogenised matrices, the CG
    iteration counts / final residuals and the solution fields.
run_<name>.npz
    Problems this script defines and runs through the reference's
    Problem(...).calculate() (ffthompy/problem.py:70-83): config-1 (2D GaNi
    45^2 square, tol 1e-8), seeded random 'fun' materials on odd, even,
    prime and anisotropic grids, Ga and GaNi, scalar and elasticity.
op_<name>.npz
    Single applications of the reference operator FiGFA = G o A
    (ffthompy/applications.py:24-58) to seeded random fields; this pins the
    Green projection, the Ga scale factor of Tensor.enlarge and the r2c FFT
    conventions independently of CG.

pot_<name>.npz
    The potential formulation (ffthompy/tensorsLowRank/homogenisation.py:
    41-127): A_H, CG iteration counts and the potential Fu of
    homog_GaNi_full_potential / homog_Ga_full_potential, and one application
    of their preconditioned operator.

solv_<name>.npz
    linear_solver with solver='chebyshev' (ffthompy/general/solver.py:
    206-285) on a scalar FiGFA operator: solution, iteration count, final
    relative residual.

inv_<name>.npz
    Per-voxel inverses of get_inverse (ffthompy/trigpol.py:120-159) of
    seeded matrix fields, one with zero pivots (Inf / NaN outputs).

Usage:  python tests/golden/make_golden.py REFERENCE_DIR [pickles|run|op|pot|solv|inv ...]
        FFTHOMPY_REFERENCE=REFERENCE_DIR python tests/golden/make_golden.py
"""
import collections
import collections.abc
import contextlib
import glob
import io
import json
import os
import pickle
import sys
import time

import numpy as np
import scipy

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_DIR = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('FFTHOMPY_REFERENCE')


def _install_shim():
    np.int = int
    np.float = float
    np.complex = complex
    time.clock = time.perf_counter
    collections.Callable = collections.abc.Callable
    scipy.setdiff1d = np.setdiff1d
    os.environ.setdefault('PYTHONDONTWRITEBYTECODE', '1')
    sys.dont_write_bytecode = True
    sys.path.insert(0, REFERENCE_DIR)
    sys.path.insert(0, os.path.join(REFERENCE_DIR, 'examples', 'scalar'))


def _jsonable(v):
    if isinstance(v, np.ndarray):
        return {'__nd__': v.tolist(), 'dtype': str(v.dtype)}
    if isinstance(v, (np.integer,)):
        return int(v)
    if isinstance(v, (np.floating,)):
        return float(v)
    if isinstance(v, dict):
        return {k: _jsonable(x) for k, x in v.items() if not callable(x)}
    if isinstance(v, (list, tuple)):
        return [_jsonable(x) for x in v]
    return v


def _problem_meta(physics, material, solve, solver, postprocess):
    mat = {k: v for k, v in material.items() if k != 'fun'}
    return dict(physics=physics, material=_jsonable(mat), solve=_jsonable(solve),
                solver=_jsonable(solver), postprocess=_jsonable(postprocess),
                has_fun=('fun' in material))


def _flatten_output(out, primaldual, arrays):
    for pd in primaldual:
        for key, val in out['mat_' + pd].items():
            arrays['mat__%s__%s' % (pd, key)] = np.asarray(val, dtype=np.float64)
        res = out['res_' + pd]
        arrays['kit__' + pd] = np.array([r['info']['kit'] for r in res], dtype=np.int64)
        arrays['normres__' + pd] = np.array([float(r['info']['norm_res']) for r in res])
        arrays['sol__' + pd] = np.stack([s.val for s in out['sol_' + pd]])


def _save(name, meta, arrays):
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)
    print('wrote', os.path.relpath(path, HERE), sorted(arrays)[:4], '...')


def golden_pickles():
    """Flatten the reference's own golden pickles (run_unittests.py:46-64)."""
    for path in sorted(glob.glob(os.path.join(REFERENCE_DIR, 'test_results', 'python3', '*'))):
        with open(path, 'rb') as f:
            r = pickle.load(f)
        meta = _problem_meta(r['physics'], r['material'], r['solve'], r['solver'],
                             r['postprocess'])
        arrays = {}
        if 'fun' in r['material']:
            # examples/scalar/from_file.py:411-419: values do not depend on coord
            arrays['fun_values'] = np.asarray(r['material']['fun'](None), dtype=np.float64)
        _flatten_output(r, r['solve']['primaldual'], arrays)
        _save('ref_' + os.path.basename(path), meta, arrays)


def _run_problem(physics, material, solve, solver, postprocess):
    from ffthompy.problem import Problem
    conf_problem = {'name': 'p', 'physics': physics, 'material': material,
                    'solve': solve, 'solver': solver, 'postprocess': postprocess}
    pb = Problem(conf_problem, None)
    with contextlib.redirect_stdout(io.StringIO()):
        t0 = time.perf_counter()
        pb.calculate()
        t1 = time.perf_counter()
    return pb, t1 - t0


def _fun_material(values, Y, order=0, P=None):
    values = np.asarray(values, dtype=np.float64)
    grid = values.shape[2:]

    def fun(coord):
        assert tuple(coord.shape[1:]) == tuple(grid), (coord.shape, grid)
        return values.copy()
    mat = {'fun': fun, 'Y': np.asarray(Y, dtype=np.float64), 'order': order,
           'P': np.array(grid if P is None else P)}
    return mat


def _iso_field(dim, a):
    return np.einsum('ij,...->ij...', np.eye(dim), a)


def _elastic_field(bulk, mu):
    from ffthompy.mechanics.matcoef import ElasticTensor
    dim = bulk.ndim
    D = dim * (dim + 1) // 2
    out = np.zeros((D, D) + bulk.shape)
    plane = None if dim == 3 else 'strain'
    for idx in np.ndindex(*bulk.shape):
        out[(slice(None), slice(None)) + idx] = ElasticTensor(
            bulk=float(bulk[idx]), mu=float(mu[idx]), plane=plane).mandel
    return out


def run_cases():
    rng = np.random.default_rng(20261203)
    cases = []

    # config-1: 2D GaNi 45^2, centred square 0.6, 11*I / 1*I, tol 1e-8
    dim = 2
    N = np.array([45, 45])
    mat_sq = {'inclusions': ['square', 'otherwise'], 'positions': [np.zeros(dim), ''],
              'params': [0.6 * np.ones(dim), ''], 'vals': [11 * np.eye(dim), np.eye(dim)],
              'Y': np.ones(dim), 'order': None}
    cases.append(('cfg1_square45', 'scalar', mat_sq,
                  {'kind': 'GaNi', 'N': N, 'primaldual': ['primal', 'dual']},
                  {'kind': 'CG', 'tol': 1e-8, 'maxiter': 1e3},
                  [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': None},
                   {'kind': 'Ga', 'order': 0, 'P': N}], None))

    # seeded random isotropic 'fun' materials, scalar
    for name, Nl, Y, kind, tol in [
            ('s2_gani_15', [15, 15], [1., 1.], 'GaNi', 1e-8),
            ('s2_ga_15', [15, 15], [1., 1.], 'Ga', 1e-8),          # Nbar = 29 (prime)
            ('s2_gani_even_12', [12, 12], [1., 1.], 'GaNi', 1e-8),  # Nyquist zeroing
            ('s2_ga_even_8', [8, 8], [1., 1.], 'Ga', 1e-8),         # Nbar = 15
            ('s2_gani_aniso', [9, 21], [1., 2.5], 'GaNi', 1e-9),
            ('s2_ga_aniso', [7, 11], [2., 1.], 'Ga', 1e-9),          # Nbar = 13 x 21
            ('s3_gani_7', [7, 7, 7], [1., 1., 1.], 'GaNi', 1e-8),
            ('s3_ga_7', [7, 7, 7], [1., 1., 1.], 'Ga', 1e-8),       # Nbar = 13
            ('s3_gani_aniso', [5, 9, 6], [1., 1.5, 0.7], 'GaNi', 1e-8),
            ('s3_ga_aniso', [5, 7, 9], [1., 1., 1.], 'Ga', 1e-8)]:
        Nl = np.array(Nl)
        d = Nl.size
        a = 1. + 99. * (rng.random(tuple(Nl)) < 0.3) * rng.random(tuple(Nl))
        values = _iso_field(d, a)
        pp = [{'kind': 'GaNi'}] if kind == 'GaNi' else [{'kind': 'Ga'}]
        if kind == 'GaNi':
            pp.append({'kind': 'Ga', 'order': 0, 'P': Nl})
        cases.append((name, 'scalar', _fun_material(values, Y),
                      {'kind': kind, 'N': Nl, 'primaldual': ['primal', 'dual']},
                      {'kind': 'CG', 'tol': tol, 'maxiter': 1e3}, pp, values))

    # a full (anisotropic, symmetric positive definite) scalar coefficient
    Nl = np.array([11, 9])
    B = rng.standard_normal((2, 2) + tuple(Nl))
    values = np.einsum('ik...,jk...->ij...', B, B) + 0.5 * _iso_field(2, np.ones(tuple(Nl)))
    cases.append(('s2_full_gani', 'scalar', _fun_material(values, [1., 1.]),
                  {'kind': 'GaNi', 'N': Nl, 'primaldual': ['primal', 'dual']},
                  {'kind': 'CG', 'tol': 1e-9, 'maxiter': 1e3},
                  [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': 0, 'P': Nl}], values))

    # elasticity with random isotropic phases (Mandel 6x6 / 3x3)
    for name, Nl, kind in [('e3_gani_5', [5, 5, 5], 'GaNi'), ('e3_ga_5', [5, 5, 5], 'Ga'),
                           ('e3_gani_7', [7, 7, 7], 'GaNi'),
                           ('e2_gani_9', [9, 9], 'GaNi'), ('e2_ga_7', [7, 7], 'Ga')]:
        Nl = np.array(Nl)
        incl = rng.random(tuple(Nl)) < 0.35
        bulk = np.where(incl, 5.5556, 0.8333)
        mu = np.where(incl, 4.1667, 0.3846)
        values = _elastic_field(bulk, mu)
        pp = [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': 0, 'P': Nl}] if kind == 'GaNi' \
            else [{'kind': 'Ga'}]
        cases.append((name, 'elasticity', _fun_material(values, np.ones(Nl.size)),
                      {'kind': kind, 'N': Nl, 'primaldual': ['primal', 'dual']},
                      {'kind': 'CG', 'tol': 1e-8, 'maxiter': 1e3}, pp, values))

    for name, physics, material, solve, solver, pp, values in cases:
        pb, seconds = _run_problem(physics, material, solve, solver, pp)
        meta = _problem_meta(physics, material, solve, solver, pp)
        meta['reference_seconds'] = seconds
        arrays = {}
        if values is not None:
            arrays['fun_values'] = values
        _flatten_output(pb.output, solve['primaldual'], arrays)
        _save('run_' + name, meta, arrays)


def operator_cases():
    """Single G o A applications (ffthompy/applications.py:24-58)."""
    import ffthompy.projections as proj
    from ffthompy.tensors import Tensor, DFT, Operator
    rng = np.random.default_rng(7)
    for name, physics, Nl, Y, kind in [
            ('s2_gani_9', 'scalar', [9, 9], [1., 1.], 'GaNi'),
            ('s2_ga_9', 'scalar', [9, 9], [1., 1.], 'Ga'),
            ('s2_gani_even_10', 'scalar', [10, 8], [1., 2.], 'GaNi'),
            ('s2_ga_even_6', 'scalar', [6, 7], [1., 1.], 'Ga'),
            ('s3_gani_5x7x9', 'scalar', [5, 7, 9], [1., 2., 1.5], 'GaNi'),
            ('s3_ga_5', 'scalar', [5, 5, 5], [1., 1., 1.], 'Ga'),
            ('e2_gani_9', 'elasticity', [9, 9], [1., 1.], 'GaNi'),
            ('e3_gani_5x7x9', 'elasticity', [5, 7, 9], [1., 1., 1.], 'GaNi'),
            ('e3_ga_5', 'elasticity', [5, 5, 5], [1., 1., 1.], 'Ga')]:
        N = np.array(Nl)
        d = N.size
        Nbar = N if kind == 'GaNi' else 2 * N - 1
        dv = d if physics == 'scalar' else d * (d + 1) // 2
        if physics == 'scalar':
            _, G1, G2 = proj.scalar(N, np.array(Y), NyqNul=True, tensor=True)
            Gs = [G1, G2]
        else:
            _, G1h, G1s, G2h, G2s = proj.elasticity(N, np.array(Y), NyqNul=True)
            Gs = [G1h + G1s, G2h + G2s]
        if kind == 'Ga':
            Gs = [G.enlarge(Nbar) for G in Gs]
        FN = DFT(name='FN', inverse=False, N=Nbar)
        FiN = DFT(name='FiN', inverse=True, N=Nbar)
        B = rng.standard_normal((dv, dv) + tuple(Nbar))
        Aval = np.einsum('ik...,jk...->ij...', B, B) + np.einsum(
            'ij,...->ij...', np.eye(dv), np.ones(tuple(Nbar)))
        A = Tensor(name='A', val=Aval, order=2, N=Nbar, multype=21)
        x = Tensor(name='x', val=rng.standard_normal((dv,) + tuple(Nbar)), order=1, N=Nbar)
        arrays = {'A': Aval, 'x': x.val}
        for ip, G in enumerate(Gs):
            GN = Operator(name='G', mat=[[FiN, G, FN]])
            Afun = Operator(name='FiGFA', mat=[[GN, A]])
            arrays['y%d' % (ip + 1)] = Afun(x).val
        meta = dict(physics=physics, N=Nl, Y=Y, kind=kind, Nbar=[int(v) for v in Nbar])
        _save('op_' + name, meta, arrays)


def solver_cases():
    """The two-term Chebyshev iteration of linear_solver (ffthompy/general/
    solver.py:206-285, eigrange = the coefficient bounds) on the scalar
    Galerkin operator of a seeded random material.  (BiCG, solver.py:142-204,
    does not run on Tensor / Operator objects as shipped: it forms R.T*Rs,
    and Tensor has no .T for vectors, and alp*ATfun*Ps multiplies an Operator
    by a float first; the tests pin it by its oracle restatement.)"""
    import ffthompy.projections as proj
    from ffthompy.general.solver import linear_solver
    from ffthompy.tensors import Tensor, DFT, Operator
    rng = np.random.default_rng(11)
    for name, Nl, kind in [('s2_gani_15', [15, 15], 'GaNi'), ('s2_ga_9', [9, 9], 'Ga'),
                           ('s3_gani_7', [7, 7, 7], 'GaNi')]:
        N = np.array(Nl)
        d = N.size
        Nbar = N if kind == 'GaNi' else 2 * N - 1
        _, G1, _ = proj.scalar(N, np.ones(d), NyqNul=True, tensor=True)
        if kind == 'Ga':
            G1 = G1.enlarge(Nbar)
        FN = DFT(name='FN', inverse=False, N=Nbar)
        FiN = DFT(name='FiN', inverse=True, N=Nbar)
        a = 1. + 9. * (rng.random(tuple(Nbar)) < 0.4)
        Aval = np.einsum('ij,...->ij...', np.eye(d), a)
        A = Tensor(name='A', val=Aval, order=2, N=Nbar, multype=21)
        GN = Operator(name='G', mat=[[FiN, G1, FN]])
        Afun = Operator(name='FiGFA', mat=[[GN, A]])
        E = np.zeros(d)
        E[0] = 1.
        EN = Tensor(name='EN', N=Nbar, shape=(d,), Fourier=False)
        EN.set_mean(E)
        B = Afun(-EN)
        arrays = {'A': Aval, 'B': B.val}
        # the spectrum of FiGFA on its range: the coefficient bounds times the
        # Ga scale prod(Nbar)/prod(N) of the enlarged projection
        sc = float(np.prod(Nbar)) / float(np.prod(N))
        eig = [sc * float(a.min()), sc * float(a.max())]
        for solver, par in [('chebyshev', {'tol': 1e-6, 'maxit': 2000, 'eigrange': eig})]:
            x0 = Tensor(N=Nbar, shape=(d,), Fourier=False)
            with contextlib.redirect_stdout(io.StringIO()):
                X, info = linear_solver(Afun, B, ATfun=Afun, x0=x0, par=dict(par),
                                        solver=solver, callback=None)
            arrays['x__' + solver] = X.val
            arrays['kit__' + solver] = np.array(int(info['kit']))
            arrays['normres__' + solver] = np.array(float(info['norm_res']))
        meta = dict(N=Nl, kind=kind, Nbar=[int(v) for v in Nbar],
                    chebyshev={'tol': 1e-6, 'maxit': 2000, 'eigrange': eig})
        _save('solv_' + name, meta, arrays)


def _stub_ttpy():
    """ffthompy.tensorsLowRank imports ttpy (absent here) at module level; the
    full potential solvers used below never call it, so empty stand-in
    modules satisfy the imports."""
    import types

    class _Absent(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith('__'):
                raise AttributeError(name)
            return type(name, (), {})
    for m in ('tt', 'tt.core', 'tt.core.vector', 'tt.core.tools', 'tt.core.matrix'):
        sys.modules.setdefault(m, _Absent(m))


def potential_cases():
    """The potential formulation with the 1/|xi| preconditioner:
    homog_GaNi_full_potential and homog_Ga_full_potential
    (ffthompy/tensorsLowRank/homogenisation.py:41-127), run on reference
    Material coefficients (E = e_0, as the reference does), plus single
    applications of their preconditioned operator PDFAFGPfun built from the
    same reference primitives (grad, div, DFT, enlarge, project)."""
    _stub_ttpy()
    import ffthompy.tensorsLowRank.homogenisation as H
    from ffthompy import Struct
    from ffthompy.materials import Material
    from ffthompy.tensors import DFT, Tensor, grad, div
    rng = np.random.default_rng(31)
    cases = []
    for dim in (2, 3):
        mat = {'inclusions': ['square', 'otherwise'], 'positions': [np.zeros(dim), ''],
               'params': [0.6 * np.ones(dim), ''], 'vals': [10 * np.eye(dim), np.eye(dim)],
               'Y': np.ones(dim), 'P': dim * (5,), 'order': 0}
        cases.append(('s%d_square5' % dim, mat, np.array(dim * [5])))
    for name, Nl in [('s2_fun9', [9, 9]), ('s3_fun5', [5, 5, 5]), ('s3_fun_aniso', [5, 7, 9]),
                     ('s2_fun_even8', [8, 8]), ('s2_fun_even6x7', [6, 7])]:
        Nl = np.array(Nl)
        a = 1. + 49. * (rng.random(tuple(Nl)) < 0.35) * rng.random(tuple(Nl))
        cases.append((name, _fun_material(_iso_field(Nl.size, a), np.ones(Nl.size)), Nl))
    for name, mconf, N in cases:
        d = N.size
        even = bool(np.any(N % 2 == 0))
        pars = Struct(dim=d, N=tuple(int(n) for n in N), Y=np.ones(d),
                      solver=dict(tol=1e-8, maxiter=200))
        mat = Material(mconf)
        Agani = mat.get_A_GaNi(N, primaldual='primal')
        Aga = mat.get_A_Ga(2 * N - 1, primaldual='primal')
        arrays = {'A_gani': Agani.val, 'A_ga': Aga.val}
        runs = [('gani', lambda: H.homog_GaNi_full_potential(Agani, None, pars))]
        if not even:
            runs += [('gani_ga', lambda: H.homog_GaNi_full_potential(Agani, Aga, pars)),
                     ('ga', lambda: H.homog_Ga_full_potential(Aga, pars))]
        for key, fn in runs:
            with contextlib.redirect_stdout(io.StringIO()):
                r = fn()
            arrays['AH__' + key] = np.array(float(r.AH))
            arrays['kit__' + key] = np.array(int(r.info['kit']))
            arrays['normres__' + key] = np.array(float(r.info['norm_res']))
            arrays['Fu__' + key] = r.Fu.val
        # one application of PDFAFGPfun to a seeded Hermitian spectrum
        x = Tensor(name='x', val=np.fft.rfftn(rng.standard_normal(tuple(N))), order=0,
                   N=N, Fourier=True)
        P = H.get_preconditioner(N, pars)
        F, iF = DFT(name='FN', inverse=False, N=N), DFT(name='FiN', inverse=True, N=N)
        arrays['x'] = x.val
        arrays['y__gani'] = (P * (-div(F(Agani * iF(grad(P * x)))))).val
        if not even:
            Nbar = 2 * N - 1
            F2, iF2 = DFT(name='FN', inverse=False, N=Nbar), DFT(name='FiN', inverse=True, N=Nbar)
            FAX = F2(Aga * iF2(grad(P * x).enlarge(Nbar))).project(N)
            arrays['y__ga'] = (P * (-div(FAX))).val
        meta = dict(N=[int(n) for n in N], Y=[1.] * d, tol=1e-8, maxiter=200, even=even,
                    runs=[k for k, _ in runs])
        _save('pot_' + name, meta, arrays)


def inverse_cases():
    """Per-voxel inverses of the reference's get_inverse (ffthompy/trigpol.py:
    120-159): seeded matrices a + d I (symmetric and not) for d = 1, 2, 3, 6 on
    1D-3D grids, and a field with zero pivots at some voxels (Inf / NaN)."""
    from ffthompy.trigpol import get_inverse
    rng = np.random.default_rng(17)
    cases = [('d1_1d_7', 1, (7,), 'full'), ('d2_2d_5x4', 2, (5, 4), 'sym'),
             ('d3_3d_3x4x5', 3, (3, 4, 5), 'full'), ('d6_3d_4x3x5', 6, (4, 3, 5), 'sym'),
             ('d3_2d_6x5_zero_pivot', 3, (6, 5), 'zero')]
    for name, d, N, kind in cases:
        A = rng.standard_normal((d, d) + N)
        if kind == 'sym':
            A = 0.5 * (A + A.transpose((1, 0) + tuple(range(2, 2 + len(N)))))
        A = A + np.einsum('ij,...->ij...', d * np.eye(d), np.ones(N))
        if kind == 'zero':
            A[0, 0, 1, 2] = 0.
            A[1, 1, 3, 0] = A[1, 0, 3, 0] * A[0, 1, 3, 0] / A[0, 0, 3, 0]
            A[0, 0, 5, 4] = 0.
            A[0, 1, 5, 4] = 0.
        arrays = {'A': A, 'inv': np.asarray(get_inverse(A), dtype=np.float64)}
        _save('inv_' + name, dict(d=d, N=list(N), kind=kind), arrays)


if __name__ == '__main__':
    if not REFERENCE_DIR or not os.path.isdir(REFERENCE_DIR):
        sys.exit('make_golden.py: give the FFTHomPy source directory as the first argument '
                 'or in FFTHOMPY_REFERENCE')
    _install_shim()
    import warnings
    warnings.simplefilter('ignore')
    only = sys.argv[2:] if len(sys.argv) > 2 else ['pickles', 'run', 'op', 'pot', 'solv',
                                                   'inv']
    if 'pickles' in only:
        golden_pickles()
    if 'run' in only:
        run_cases()
    if 'op' in only:
        operator_cases()
    if 'pot' in only:
        potential_cases()
    if 'solv' in only:
        solver_cases()
    if 'inv' in only:
        inverse_cases()
