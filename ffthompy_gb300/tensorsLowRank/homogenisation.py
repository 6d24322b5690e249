"""Potential formulation with the 1/|xi| preconditioner, mirroring
ffthompy/tensorsLowRank/homogenisation.py:41-127 and 296-300.

The unknown is the scalar potential u of the fluctuation field, in the 'r'
Fourier form of the grid N; CG runs on P (-div F A iF grad) P with
P = 1/|2 pi xi|, whose iterates are the gradient-formulation iterates in
another basis.  Every step (right-hand side, operator, CG, field and A_H)
runs in libffthompy_gb300.so; this module only builds the plans.

homog_GaNi_full_potential(Agani, Aga, pars): solve with the nodal coefficient
    on N; A_H with Agani, or with the Ga coefficient Aga on 2N-1 when given.
homog_Ga_full_potential(Aga, pars): solve with the Ga coefficient on
    Nbar = 2N-1 (N odd); A_H with Aga.
Both take the reference's pars (pars.Y, pars.solver = {'tol', 'maxiter'}) and
return a Struct with AH, Fu (the potential, 'r' half spectrum), info and time.
As in the reference, the load is E = e_0 and AH is its scalar energy; the
keyword loads=d solves all unit loads together and AH is then the d x d
matrix.  pars.precision ('f64' default, 'f32') selects the working precision.
"""
import time

import numpy as np
import torch

from ..engine import GalerkinPlan


class Struct(dict):
    """Attribute access to a dict (ffthompy/general/base.py:84-276 Struct)."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k)

    def __setattr__(self, k, v):
        self[k] = v


class FourierPotential:
    """A potential in the 'r' Fourier form: val (NumPy, loads first when
    loads > 1), data (the device tensor), N, mean() as Tensor.mean
    (objects.py:263-275: real part of the zero-frequency coefficient over
    prod(N))."""

    Fourier = True
    fft_form = 'r'

    def __init__(self, data, N):
        self.data = data
        self.N = tuple(N)

    @property
    def val(self):
        v = self.data.detach().cpu().numpy()
        return v[0] if v.shape[0] == 1 else v

    def mean(self):
        v = self.data.detach().cpu().numpy()
        m = v[(slice(None),) + (0,) * len(self.N)].real / float(np.prod(self.N))
        return float(m[0]) if m.size == 1 else m


def _par(pars, key, default=None):
    if isinstance(pars, dict):
        return pars.get(key, default)
    return getattr(pars, key, default)


def get_preconditioner(N, pars):
    """P = 1/|2 pi xi| on the 'r' half spectrum of N, 1 at the mean
    (homogenisation.py:296-300), as a NumPy array."""
    N = np.asarray(N, dtype=np.int64)
    Y = np.asarray(_par(pars, 'Y', np.ones(N.size)), dtype=np.float64)
    xi = []
    for i, n in enumerate(N):
        z = np.fft.ifftshift(np.arange(np.trunc(-n / 2.), np.trunc(n / 2. + 0.5)))
        xi.append(z / Y[i])
    xi[-1] = xi[-1][:N[-1] // 2 + 1]
    grids = np.meshgrid(*xi, indexing='ij')
    k2 = sum((2 * np.pi * g) ** 2 for g in grids)
    k2[(0,) * N.size] = 1.
    return 1. / k2 ** 0.5


def _coef(A):
    return A.data if hasattr(A, 'data') else torch.as_tensor(np.asarray(A))


def _solve(plan, pars, N):
    solver = _par(pars, 'solver', {}) or {}
    tol = float(solver.get('tol', 1e-6))
    maxiter = int(solver.get('maxiter', 1000))
    PB = plan.potential_rhs()
    t0 = time.perf_counter()
    iPU, info = plan.potential_cg(PB, tol=tol, maxiter=maxiter)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    P = torch.as_tensor(get_preconditioner(N, pars), device=iPU.device).to(iPU.dtype)
    Fu = FourierPotential(P * iPU, N)
    if plan.nloads == 1:
        info = {k: (v[0] if isinstance(v, list) else v) for k, v in info.items()}
    return iPU, Fu, info, elapsed


def _ah(plan, X):
    AH = plan.energy(X, add_macro=True)
    return float(AH[0, 0]) if plan.nloads == 1 else AH


def homog_GaNi_full_potential(Agani, Aga, pars, loads=1):
    N = tuple(int(n) for n in Agani.N)
    d = len(N)
    Y = np.asarray(_par(pars, 'Y', np.ones(d)), dtype=np.float64)
    prec = _par(pars, 'precision', 'f64') or 'f64'
    plan = GalerkinPlan(N, Y, physics='scalar', nloads=loads, precision=prec)
    plan.set_coefficient(_coef(Agani))
    iPU, Fu, info, elapsed = _solve(plan, pars, N)
    if Aga is None:
        AH = _ah(plan, plan.potential_field(iPU))
    else:
        Nbar = tuple(int(n) for n in Aga.N)
        post = GalerkinPlan(Nbar, Y, physics='scalar', nloads=loads, band=N, precision=prec)
        post.set_coefficient(_coef(Aga))
        AH = _ah(post, post.potential_field(iPU))
    return Struct(AH=AH, Fu=Fu, info=info, time=elapsed, pars=pars)


def homog_Ga_full_potential(Aga, pars, loads=1):
    Nbar = tuple(int(n) for n in Aga.N)
    N = tuple((n + 1) // 2 for n in Nbar)
    d = len(N)
    Y = np.asarray(_par(pars, 'Y', np.ones(d)), dtype=np.float64)
    prec = _par(pars, 'precision', 'f64') or 'f64'
    plan = GalerkinPlan(Nbar, Y, physics='scalar', nloads=loads, band=N, precision=prec)
    plan.set_coefficient(_coef(Aga))
    iPU, Fu, info, elapsed = _solve(plan, pars, N)
    X = plan.potential_field(iPU)
    return Struct(AH=_ah(plan, X), e=X, Fu=Fu, info=info, time=elapsed)
