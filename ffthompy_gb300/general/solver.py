"""Linear solvers, mirroring ffthompy/general/solver.py.

linear_solver(Afun, B, ATfun, x0, par, solver, callback) -> (x, info)
(solver.py:8-60).  When Afun is a fused G o A Operator and solver is 'CG',
the whole solve runs on the GPU in one library call (fhp_cg_solve: batched
CG with FP64 reductions, absolute stopping test sqrt(<R,R>) <= tol,
solver.py:80-139).  Other operators use the same CG recurrence written with
Tensor arithmetic on the device.  'richardson' / 'iterative' (63-77),
'bicg' (142-204) and 'chebyshev' (206-285) over a fused Operator run in one
library call each (fhp_richardson_solve, fhp_bicg_solve,
fhp_chebyshev_solve): the recurrences in fused kernels with per-load scalars
on the device and one CUDA-graph replay per iteration, no host
synchronisation per scalar.  Other operators use Tensor arithmetic.
"""
import time

import numpy as np

from ..tensors.objects import Tensor
from ..tensors.operators import Operator
from .solver_pp import CallBack


def _defaults(par):
    par = {} if par is None else par
    par.setdefault('tol', 1e-6)
    par.setdefault('maxiter', int(1e3))
    return par


def linear_solver(Afun, B, ATfun=None, x0=None, par=None, solver=None, callback=None):
    t0 = (time.process_time(), time.perf_counter(), time.time())
    if x0 is None:
        x0 = B.zeros_like()
    par = _defaults(par)
    kind = (solver or 'CG').lower()
    if kind == 'cg':
        x, info = CG(Afun, B, x0=x0, par=par, callback=callback)
    elif kind in ('iterative', 'richardson'):
        x, info = richardson(Afun, B, x0, par=par, callback=callback)
    elif kind == 'bicg':
        x, info = BiCG(Afun, ATfun if ATfun is not None else Afun, B, x0, par=par,
                       callback=callback)
    elif kind in ('chebyshev', 'cheby'):
        x, info = cheby2TERM(Afun, B, x0, par=par, callback=callback)
    else:
        raise NotImplementedError('This kind (%s) of linear solver is not implemented' % solver)
    t1 = (time.process_time(), time.perf_counter(), time.time())
    info['time'] = [[t1[i] - t0[i] for i in range(3)]]
    return x, info


def CG(Afun, B, x0, par=None, callback=None):
    par = _defaults(par)
    if isinstance(Afun, Operator) and Afun.kind == 'GA' and isinstance(B, Tensor):
        plan = Afun.plan()
        zero_start = float(x0.data.abs().max()) == 0.0
        xd, info = plan.cg(B.data[None], None if zero_start else x0.data[None],
                           tol=par['tol'], maxiter=par['maxiter'], proj=Afun.projection.proj)
        x = x0.copy(name='x', val=xd[0])
        log = info['res_log'][0]
        if isinstance(callback, CallBack):
            callback.record_log(log)
        elif callback is not None:
            callback(x)
        return x, {'kit': info['kit'][0], 'norm_res': info['norm_res'][0]}
    return _cg_generic(Afun, B, x0, par, callback)


def _cg_generic(Afun, B, x0, par, callback):
    """solver.py:80-139 with device Tensor arithmetic."""
    if callback is not None:
        callback(x0)
    scal = par.get('scal', lambda X, Y: X * Y)
    x = x0
    R = B - Afun(x0)
    P = R
    rr = scal(R, R)
    res = {'kit': 0, 'norm_res': np.double(rr) ** 0.5}
    while res['norm_res'] > par['tol'] and res['kit'] < par['maxiter']:
        res['kit'] += 1
        AP = Afun(P)
        alp = float(rr / scal(P, AP))
        x = x + alp * P
        R = R - alp * AP
        rrnext = scal(R, R)
        bet = rrnext / rr
        rr = rrnext
        P = R + bet * P
        res['norm_res'] = np.double(rr) ** 0.5
        if callback is not None:
            callback(x)
    if res['kit'] == 0:
        res['norm_res'] = 0
    return x, res


def _fused(Afun, B):
    return isinstance(Afun, Operator) and Afun.kind == 'GA' and isinstance(B, Tensor)


def _device_solve(kind, Afun, B, x0, par, callback, p0=0., p1=0., maxiter=None):
    plan = Afun.plan()
    zero_start = float(x0.data.abs().max()) == 0.0
    xd, info = plan.solve_other(kind, B.data[None], None if zero_start else x0.data[None],
                                tol=par['tol'],
                                maxiter=par['maxiter'] if maxiter is None else maxiter,
                                proj=Afun.projection.proj, p0=p0, p1=p1)
    x = x0.copy(name='x', val=xd[0])
    if callback is not None and not isinstance(callback, CallBack):
        callback(x)
    return x, {'kit': info['kit'][0], 'norm_res': info['norm_res'][0]}


def richardson(Afun, B, x0, par=None, callback=None):
    """solver.py:63-77."""
    if _fused(Afun, B) and par.get('norm', 'L2') in ('L2', 2):
        par = _defaults(par)
        return _device_solve('richardson', Afun, B, x0, par, callback, p0=1. / par['alpha'])
    omega = 1. / par['alpha']
    res = {'norm_res': 1e15, 'kit': 0}
    x = x0
    while res['norm_res'] > par['tol'] and res['kit'] < par['maxiter']:
        res['kit'] += 1
        residuum = B - Afun(x)
        x = x + omega * residuum
        res['norm_res'] = residuum.norm()
        if callback is not None:
            callback(x)
    return x, res


def BiCG(Afun, ATfun, B, x0, par=None, callback=None):
    """BiConjugate gradients, solver.py:142-204 (shadow residual updated with
    ATfun, stop on sqrt(<R, Rs>) <= tol).  The reference forms <R, Rs> as
    R.T*Rs, which its Tensor class does not support; here it is the scalar
    product.  With a fused Operator as its own transpose (the symmetric
    G o A) the whole recurrence runs in the CUDA library (fhp_bicg_solve);
    otherwise with Tensor arithmetic."""
    par = _defaults(par)
    if _fused(Afun, B) and ATfun is Afun and 'scal' not in par:
        return _device_solve('bicg', Afun, B, x0, par, callback)
    scal = par.get('scal', lambda X, Y: X * Y)
    x = x0
    R = B - Afun(x0)
    Rs = R
    rr = float(scal(R, Rs))
    P, Ps = R, Rs
    res = {'kit': 0, 'norm_res': rr ** 0.5}
    while res['norm_res'] > par['tol'] and res['kit'] < par['maxiter']:
        res['kit'] += 1
        AP = Afun(P)
        alp = rr / float(scal(AP, Ps))
        x = x + alp * P
        R = R - alp * AP
        Rs = Rs - alp * ATfun(Ps)
        rrnext = float(scal(R, Rs))
        bet = rrnext / rr
        rr = rrnext
        P = R + bet * P
        Ps = Rs + bet * Ps
        res['norm_res'] = rr ** 0.5
        if callback is not None:
            callback(x)
    if res['kit'] == 0:
        res['norm_res'] = 0
    return x, res


def cheby2TERM(A, B, x0, M=None, par=None, callback=None):
    """Chebyshev two-term iteration, solver.py:206-285: par['eigrange'] is
    the eigenvalue interval, par['maxit'] the iteration limit (default 1e7),
    norm_res the residual norm relative to the initial one."""
    par = {} if par is None else par
    par.setdefault('tol', 1e-06)
    par.setdefault('maxit', 1e7)
    if 'eigrange' not in par:
        raise NotImplementedError('It is necessary to calculate eigenvalues.')
    Egv = par['eigrange']
    if _fused(A, B) and M is None:
        return _device_solve('chebyshev', A, B, x0, par, callback, p0=Egv[0], p1=Egv[1],
                             maxiter=int(min(par['maxit'], 2 ** 31 - 1)))
    res = {'kit': 0}
    bnrm2 = float(B * B) ** 0.5
    Ib = 1.0 / bnrm2
    x = x0
    r = B - A(x)
    r0 = np.double(r * r) ** 0.5
    res['norm_res'] = Ib * r0
    if res['norm_res'] < par['tol']:
        return x, res
    d = (Egv[1] + Egv[0]) / 2.0
    c = (Egv[1] - Egv[0]) / 2.0
    v = 0 * x0
    w = 0.
    while res['norm_res'] > par['tol'] and res['kit'] < par['maxit']:
        res['kit'] += 1
        x_prev = x
        if res['kit'] == 1:
            p = 0.
            w = 1 / d
        elif res['kit'] == 2:
            p = -(1 / 2) * (c / d) * (c / d)
            w = 1 / (d - c * c / 2 / d)
        else:
            p = -(c * c / 4) * w * w
            w = 1 / (d - c * c * w / 4)
        v = r - p * v
        x = x_prev + w * v
        r = B - A(x)
        res['norm_res'] = (1.0 / r0) * r.norm()
        if callback is not None:
            callback(x)
    if res['kit'] == 0:
        res['norm_res'] = 0
    return x, res
