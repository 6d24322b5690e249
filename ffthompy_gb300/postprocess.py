"""Homogenised matrices and their guaranteed bounds, mirroring
ffthompy/postprocess.py.

postprocess (postprocess.py:6-51) evaluates A_H for every postprocess kind:
'GaNi' on the solve grid, 'Ga' with the exact-integration coefficient on the
double grid 2N-1 (the solution is trigonometrically interpolated there first,
postprocess.py:60-66) - the upper bound from the primal problem and, through
inv(A_H), the lower bound from the dual problem (postprocess.py:43-46).
Energies A_H[i,j] = <A (X_i+E_i), X_j+E_j> are accumulated in FP64 by one GPU
kernel over all load pairs (fhp_energy_matrix).

The Ga coefficient is sampled on nice_size(2N-1) (factors 2, 3, 5, 7) instead
of 2N-1 itself: the same trigonometric polynomial (its frequencies lie in the
2N-1 band), and the energy with band-limited solutions is exact on any grid
of at least 2N-1 points per axis, so A_H is the reference's; a 2N-1 with a
large prime factor (253 = 11 x 23) would otherwise take Bluestein lines.
"""
import time

import numpy as np

from .engine import interpolate_fields, nice_size, shared_plan
from .tensors.objects import Tensor


class Solutions:
    """The L zero-mean correctors of one primal/dual solve, kept on the GPU.

    Indexing gives the reference's solution Tensors X_l + E_l on the
    reference's solution grid out_grid (N for GaNi, 2N-1 for Ga; band-mode
    fields are interpolated there on access) (add_macro2minimizer,
    postprocess.py:73-86).
    """

    def __init__(self, plan, X, Y, out_grid=None):
        self.plan = plan
        self.X = X          # (L, dv) + plan.N, zero-mean fluctuations
        self.Y = Y
        self.N = plan.N
        self.out_grid = tuple(out_grid) if out_grid is not None else plan.N

    def __len__(self):
        return self.plan.nloads

    def fields(self):
        if self.out_grid == tuple(self.N):
            return self.X
        return interpolate_fields(self.X, self.N, self.out_grid)

    def tolist(self):
        X = self.fields()
        out = []
        for l in range(len(self)):
            v = X[l].clone()
            v[l] += 1.0
            out.append(Tensor(name='X+E', val=v, order=1, Y=self.Y))
        return out

    def __getitem__(self, l):
        return self.tolist()[l]


def assembly_matrix(A, solutions):
    """A_H from a coefficient Tensor A and a Solutions batch (postprocess.py:53-70).

    The energy <A (X_i+E_i), X_j+E_j> on A's grid is exact for band-limited
    solutions: on the solve grid by a direct sum, on a finer grid (the Ga
    bounds) through a band plan whose integration grid is A's grid.
    """
    plan = solutions.plan
    G = tuple(int(n) for n in A.N)
    N = tuple(plan.N)
    if getattr(plan, '_coef_tensor', None) is A:
        return plan.energy(solutions.X, add_macro=True)
    if G == N and plan.integ is None:
        plan_e = shared_plan(N, plan.Y, physics=plan.physics, nloads=plan.nloads,
                             band=plan.band, scale=plan.scale, precision=plan.precision)
    elif all(g >= 2 * n - 1 for g, n in zip(G, N)):
        plan_e = shared_plan(N, plan.Y, physics=plan.physics, nloads=plan.nloads, integ=G,
                             precision=plan.precision)
    elif G == N:
        plan_e = shared_plan(N, plan.Y, physics=plan.physics, nloads=plan.nloads,
                             precision=plan.precision)
    else:
        raise NotImplementedError('energy of solutions on %s with a coefficient on %s'
                                  % (N, G))
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
                G = tuple(nice_size(int(n)) for n in Npp)
                if not all(g >= 2 * n - 1 for g, n in zip(G, solutions.plan.N)):
                    G = Npp     # solutions on the double grid (full-grid Ga solve)
                if pp['order'] is None:
                    Ap = mat.get_A_Ga(Nbar=Npp, primaldual=primaldual, order=pp['order'],
                                      grid=G)
                else:
                    order_name = '_o' + str(pp['order'])
                    Nname = '_P%d' % np.mean(pp['P'])
                    Ap = mat.get_A_Ga(Nbar=Npp, primaldual=primaldual, order=pp['order'],
                                      P=pp['P'], grid=G)
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
