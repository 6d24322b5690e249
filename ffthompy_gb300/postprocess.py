"""Homogenised matrices and their guaranteed bounds, mirroring
ffthompy/postprocess.py.

postprocess (postprocess.py:6-51) evaluates A_H for every postprocess kind:
'GaNi' on the solve grid, 'Ga' with the exact-integration coefficient on the
double grid 2N-1 (the solution is trigonometrically interpolated there first,
postprocess.py:60-66) - the upper bound from the primal problem and, through
inv(A_H), the lower bound from the dual problem (postprocess.py:43-46).
Energies A_H[i,j] = <A (X_i+E_i), X_j+E_j> are accumulated in FP64 by one GPU
kernel over all load pairs (fhp_energy_matrix).
"""
import time

import numpy as np

from .engine import GalerkinPlan
from .tensors.objects import Tensor


class Solutions:
    """The L zero-mean correctors of one primal/dual solve, kept on the GPU.

    Indexing gives the reference's solution Tensors X_l + E_l
    (add_macro2minimizer, postprocess.py:73-86).
    """

    def __init__(self, plan, X, Y):
        self.plan = plan
        self.X = X          # (L, dv) + N, zero-mean fluctuations
        self.Y = Y
        self.N = plan.N

    def __len__(self):
        return self.plan.nloads

    def __getitem__(self, l):
        v = self.X[l].clone()
        v[l] += 1.0
        return Tensor(name='X+E', val=v, order=1, Y=self.Y)

    def tolist(self):
        return [self[l] for l in range(len(self))]


def assembly_matrix(A, solutions):
    """A_H from a coefficient Tensor A and a Solutions batch (postprocess.py:53-70)."""
    plan = solutions.plan
    if tuple(A.N) != tuple(plan.N):
        tgt = GalerkinPlan(A.N, plan.Y, physics=plan.physics, nloads=plan.nloads,
                           precision=plan.precision)
        X = plan.interpolate_to(tgt, solutions.X)
        tgt.set_coefficient(A.data)
        return tgt.energy(X, add_macro=True)
    plan_e = plan
    if getattr(plan, '_coef_tensor', None) is not A:
        plan_e = GalerkinPlan(plan.N, plan.Y, physics=plan.physics, nloads=plan.nloads,
                              band=plan.band, scale=plan.scale, precision=plan.precision)
        plan_e.set_coefficient(A.data)
    return plan_e.energy(solutions.X, add_macro=True)


def postprocess(pb, A, mat, solutions, results, primaldual):
    t0 = time.time()
    matrices = {}
    N = np.asarray(pb.solve['N'], dtype=np.int64)
    for pp in pb.postprocess:
        Ap = A
        if pp['kind'] in ('GaNi', 'gani'):
            order_name = Nname = ''
            if A.name != 'A_GaNi':
                Ap = mat.get_A_GaNi(N, primaldual)
        elif pp['kind'] in ('Ga', 'ga'):
            order_name = Nname = ''
            if 'order' in pp:
                Npp = tuple(2 * N - 1)
                if pp['order'] is None:
                    Ap = mat.get_A_Ga(Nbar=Npp, primaldual=primaldual, order=pp['order'])
                else:
                    order_name = '_o' + str(pp['order'])
                    Nname = '_P%d' % np.mean(pp['P'])
                    Ap = mat.get_A_Ga(Nbar=Npp, primaldual=primaldual, order=pp['order'],
                                      P=pp['P'])
        else:
            raise ValueError('postprocess kind %s' % pp['kind'])
        name = 'AH_%s%s%s_%s' % (pp['kind'], order_name, Nname, primaldual)
        AH = assembly_matrix(Ap, solutions)
        matrices[name] = AH if primaldual == 'primal' else np.linalg.inv(AH)
    pb.output.update({'sol_' + primaldual: solutions.tolist(),
                      'res_' + primaldual: results,
                      'mat_' + primaldual: matrices})
    pb.output.setdefault('time', {})['postprocess_' + primaldual] = time.time() - t0


def add_macro2minimizer(X, E):
    """postprocess.py:73-86."""
    if np.allclose(X.mean(), E):
        return X
    if np.allclose(X.mean(), np.zeros_like(E)):
        EN = X.zeros_like(name='EN')
        EN.set_mean(E)
        return X + EN
    raise ValueError('Field is neither zero-mean nor E-mean.')
