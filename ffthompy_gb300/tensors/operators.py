"""DFT and Operator, mirroring ffthompy/tensors/operators.py:14-225.

Operator(mat=[[FiN, hG, FN]]) is the Green projection in real space and
Operator(mat=[[GN, A]]) the homogenisation operator FiGFA = G o A
(ffthompy/applications.py:33-58).  Both compositions are recognised and run
as one fused CUDA call (fhp_apply); there is no NumPy evaluation path.
"""
import numpy as np

from ..projections import GreenProjection
from .objects import Tensor


class DFT:
    """Forward / inverse DFT factor (operators.py:14-106); only a marker here."""

    def __init__(self, inverse=False, N=None, fft_form='r', **kwargs):
        self.__dict__.update(kwargs)
        self.name = kwargs.get('name', 'iDFT' if inverse else 'DFT')
        self.N = np.array(N, dtype=np.int32)
        self.inverse = inverse
        self.fft_form = fft_form

    def __call__(self, x):
        raise NotImplementedError('Fourier transforms run inside the fused GPU operator; '
                                  'compose DFTs with a projection in an Operator')

    def transpose(self):
        return DFT(inverse=not self.inverse, N=self.N, fft_form=self.fft_form, name=self.name)


class Operator:
    """Sum of products of callables; [[FiN, hG, FN]] and [[GN, A]] are fused."""

    def __init__(self, name='Operator', mat_rev=None, mat=None, operand=None):
        self.name = name
        if mat is None and mat_rev is not None:
            mat = [list(reversed(s)) for s in mat_rev]
        if mat is None:
            raise ValueError('Operator needs mat')
        self.mat = mat
        self.mat_rev = [list(reversed(s)) for s in mat]
        self.no_summands = len(mat)
        self.kind = None
        self.projection = None
        self.coef = None
        self._plan = None
        if len(mat) == 1:
            s = mat[0]
            if (len(s) == 3 and isinstance(s[0], DFT) and s[0].inverse and
                    isinstance(s[1], GreenProjection) and isinstance(s[2], DFT) and
                    not s[2].inverse):
                if tuple(s[0].N) != s[1].N or tuple(s[2].N) != s[1].N:
                    raise ValueError('DFT and projection grids differ')
                self.kind = 'projection'
                self.projection = s[1]
            elif (len(s) == 2 and isinstance(s[0], Operator) and s[0].kind == 'projection' and
                  isinstance(s[1], Tensor)):
                if tuple(s[1].N) != s[0].projection.N:
                    raise ValueError('coefficient and projection grids differ')
                self.kind = 'GA'
                self.projection = s[0].projection
                self.coef = s[1]
        self.N = self.projection.N if self.projection is not None else None

    def plan(self, nloads=1, precision='f64'):
        """The CUDA plan behind a fused operator (built on first use)."""
        from ..engine import GalerkinPlan
        if self._plan is None:
            G = self.projection
            self._plan = GalerkinPlan(G.N, G.Y, physics=G.physics, nloads=nloads, band=G.band,
                                      scale=G.scale, precision=precision)
            if self.kind == 'GA':
                A = self.coef
                if A.origin != 0:
                    raise ValueError('coefficient must have origin 0 (call .shift())')
                self._plan.set_coefficient(A.val)
            else:
                dv = self._plan.dv
                eye = np.zeros((dv, dv) + G.N)
                for i in range(dv):
                    eye[i, i] = 1.
                self._plan.set_coefficient(eye)
        return self._plan

    def __call__(self, x):
        if self.kind is None:
            res = None
            for summand in self.mat_rev:
                prod = x
                for m in summand:
                    prod = m(prod)
                res = prod if res is None else prod + res
            res.name = '{0}({1})'.format(self.name[:6], x.name[:10])
            return res
        plan = self.plan()
        y = plan.apply(x.data.reshape((1,) + tuple(x.data.shape)), proj=self.projection.proj)
        return x.copy(name='{0}({1})'.format(self.name[:6], x.name[:10]), val=y[0])

    def __repr__(self):
        return 'Class : Operator\n    name : %s\n    kind : %s\n' % (self.name, self.kind)

    def transpose(self):
        if self.kind == 'projection':
            return self  # the Green projections are symmetric
        raise NotImplementedError('transpose of a fused G o A operator')
