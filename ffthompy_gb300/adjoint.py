"""Differentiable homogenised coefficients (torch.autograd).

homogenized_matrix(a) solves the scalar GaNi cell problems for an isotropic
coefficient a(x) on the GPU (batched CG over the d unit loads) and returns
A_H = [<a u_i, u_j>] as a torch tensor whose backward pass gives
dF/da(x) = sum_ij dF/dA_H[i, j] * u_i(x) . u_j(x) / M.  The corrector fields
are stationary at the solution (Galerkin orthogonality), so the gradient
needs no adjoint solve, only the stored solution (one kernel,
fhp_energy_gradient).  The reference has no derivatives; its assembly_matrix
(ffthompy/postprocess.py:53-70) is the forward map.
"""
import numpy as np
import torch

from . import _lib
from .engine import GalerkinPlan


class _HomogenizedISO(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, plan, tol, maxiter):
        plan.set_coefficient_packed(a.detach().reshape((1,) + plan.N), _lib.FHP_COEF_ISO)
        B = plan.rhs_macro(1)
        X, info = plan.cg(B, tol=tol, maxiter=maxiter)
        AH = plan.energy(X)
        ctx.plan = plan
        ctx.X = X
        ctx.info = info
        return torch.as_tensor(AH, dtype=torch.float64, device=a.device)

    @staticmethod
    def backward(ctx, gAH):
        W = gAH.detach().to('cpu', torch.float64).numpy()
        g = ctx.plan.energy_gradient(ctx.X, W)
        return g.reshape(ctx.plan.N), None, None, None


def homogenized_matrix(a, Y=None, tol=1e-10, maxiter=1000, precision='f64', plan=None):
    """A_H (d x d) of the scalar GaNi problem with isotropic coefficient a
    (torch float64 tensor of the grid shape, on the GPU), differentiable with
    respect to a.  tol is the reference's absolute CG tolerance on
    sqrt(<R, R>); the gradient is exact for the converged fields, with an
    error of first order in tol.  A plan for the grid may be passed for reuse."""
    N = tuple(int(n) for n in a.shape)
    if plan is None:
        Y = np.ones(len(N)) if Y is None else np.asarray(Y, dtype=np.float64)
        plan = GalerkinPlan(N, Y, physics='scalar', precision=precision)
    return _HomogenizedISO.apply(a, plan, float(tol), int(maxiter))
