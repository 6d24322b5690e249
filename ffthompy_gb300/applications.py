"""Homogenisation drivers, mirroring ffthompy/applications.py.

scalar(problem) (applications.py:11-90) and elasticity(problem)
(applications.py:93-176): for the primal and/or dual formulation, build the
coefficient (GaNi: nodal values on N; Ga: exact integration on 2N-1), the
Green projection (G1 primal / G2 dual, scaled by prod(2N-1)/prod(N) for Ga),
solve FiGFA X = FiGFA(-E) for every unit macroscopic load by CG and
postprocess.  Differences from the reference, by design:
  * all d (scalar) or d(d+1)/2 (elasticity) loads are solved together in one
    batched GPU CG (each load keeps its own CG scalars and stopping test);
  * the per-iteration CallBack residual (solver_pp.py:13-24) is taken from the
    CG recursion instead of an extra operator application;
  * Ga solves use the band representation by default: the CG fields are
    stored on the N grid (they are band-limited trigonometric polynomials) and
    the coefficient on a smooth integration grid >= 2N-1; the operator and
    the inner products equal the reference's on the 2N-1 grid.
    solve['ga_mode'] = 'full' runs CG on the 2N-1 grid as the reference does.
"""
import time

import numpy as np
import torch

from .engine import nice_size, shared_plan
from .general.solver_pp import CallBack
from .materials import Material
from .postprocess import Solutions, postprocess


def _solve(pb, physics):
    N = np.asarray(pb.solve['N'], dtype=np.int64)
    kind = pb.solve['kind']
    if kind == 'GaNi':
        Nbar = N
    elif kind == 'Ga':
        Nbar = 2 * N - 1
    else:
        raise NotImplementedError('solve kind %s' % kind)
    precision = pb.solve.get('precision', 'f64')
    tol = float(pb.solver.get('tol', 1e-6))
    maxiter = int(pb.solver.get('maxiter', 1e3))
    if str(pb.solver.get('kind', 'CG')).lower() != 'cg':
        raise NotImplementedError('solver %s' % pb.solver.get('kind'))
    ga_mode = pb.solve.get('ga_mode', 'band')
    phases = pb.output.setdefault('time', {}).setdefault('phases', {})
    for primaldual in pb.solve['primaldual']:
        t0 = time.time()
        tp = _phase_clock()
        mat = Material(pb.material)
        proj = 1 if primaldual == 'primal' else 2
        if kind == 'GaNi':
            A = mat.get_A_GaNi(N, primaldual)
            plan = shared_plan(tuple(N), pb.Y, physics=physics, precision=precision)
        elif ga_mode == 'full':
            A = mat.get_A_Ga(Nbar=Nbar, primaldual=primaldual)
            plan = shared_plan(tuple(Nbar), pb.Y, physics=physics, band=tuple(N),
                               precision=precision)
        else:
            integ = tuple(nice_size(n) for n in Nbar)
            A = mat.get_A_Ga(Nbar=Nbar, primaldual=primaldual, grid=integ)
            plan = shared_plan(tuple(N), pb.Y, physics=physics, integ=integ,
                               precision=precision)
        ph = phases.setdefault(primaldual, {})
        ph['coefficient_s'] = tp()
        plan.set_coefficient(A.data)
        plan._coef_tensor = A
        B = plan.rhs_macro(proj)
        X, info = plan.cg(B, None, tol=tol, maxiter=maxiter, proj=proj)
        ph['solve_s'] = tp()
        results = []
        t_solve = time.time() - t0
        for l in range(plan.nloads):
            cb = CallBack(A=None, B=None)
            cb.record_log(info['res_log'][l])
            results.append({'cb': cb, 'info': {'kit': info['kit'][l],
                                               'norm_res': info['norm_res'][l],
                                               'status': info['status'][l],
                                               'time': [[t_solve, t_solve, t_solve]]}})
        out_grid = tuple(N) if kind == 'GaNi' else tuple(Nbar)
        postprocess(pb, A, mat, Solutions(plan, X, pb.Y, out_grid), results, primaldual)
        ph['postprocess_s'] = tp()


def _phase_clock():
    """Seconds since the previous call, with the device synchronised at each
    call so that a phase's GPU work is charged to it."""
    last = [time.perf_counter()]

    def lap():
        torch.cuda.synchronize()
        now = time.perf_counter()
        dt, last[0] = now - last[0], now
        return dt
    return lap


def scalar(problem):
    _solve(problem, 'scalar')


def elasticity(problem):
    _solve(problem, 'elasticity')
