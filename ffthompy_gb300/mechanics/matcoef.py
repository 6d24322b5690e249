"""Isotropic elastic tensors and Mandel / Voigt matrices (host utilities).

Mirrors ffthompy/mechanics/matcoef.py: ElasticTensor(bulk, mu, stiffness,
plane) (matcoef.py:4-72) with .val (3x3x3x3), .mandel and .voigt, and the
conversions create_mandel (152-208) / create_voigt (279-332).  Mandel order in
3D: 0,1,2 normal, 3 <-> (1,2), 4 <-> (0,2), 5 <-> (0,1); plane problems keep
rows/columns (0, 1, 5).
"""
import numpy as np

_PAIRS3 = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
_PAIRS2 = [(0, 0), (1, 1), (0, 1)]


def _pairs(dim):
    return _PAIRS3 if dim == 3 else _PAIRS2


class ElasticTensor:
    def __init__(self, bulk=None, mu=None, stiffness=True, plane=None):
        if plane not in (None, 'strain', 'stress'):
            raise ValueError('This type of plane (%s) is not supported.' % str(plane))
        self.stiffness = stiffness
        self.val_type = 'stiffness' if stiffness else 'compliance'
        self.plane = plane
        self.dim = 3 if plane is None else 2
        self.sym = self.get_sym(self.dim)
        self.bulk = float(bulk)
        self.mu = float(mu)
        I = np.eye(3)
        vol = np.einsum('ij,kl->ijkl', I, I) / 3.
        idsym = 0.5 * (np.einsum('ik,jl->ijkl', I, I) + np.einsum('il,jk->ijkl', I, I))
        dev = idsym - vol
        if stiffness:
            self.val = 3. * self.bulk * vol + 2. * self.mu * dev
        else:
            self.val = 1. / (3 * self.bulk) * vol + 1. / (2 * self.mu) * dev
        self.mandel = self.create_mandel(self.val)
        self.voigt = self.create_voigt(self.val)
        if plane is not None:
            self.val = self.val[:2, :2, :2, :2]
            keep = [0, 1, 5]
            if (stiffness and plane == 'strain') or (not stiffness and plane == 'stress'):
                self.mandel = self.mandel[np.ix_(keep, keep)]
                self.voigt = self.voigt[np.ix_(keep, keep)]
            else:
                inv = np.linalg.inv
                self.mandel = inv(inv(self.mandel)[np.ix_(keep, keep)])
                self.voigt = inv(inv(self.voigt)[np.ix_(keep, keep)])

    @staticmethod
    def get_sym(dim):
        return dim * (dim + 1) // 2

    @staticmethod
    def create_mandel(mat):
        """(d,d,d,d) tensor -> (D,D) Mandel matrix, or (d,d) -> (D,) vector."""
        dim = mat.shape[0]
        P = _pairs(dim)
        w = [1. if a == b else 2 ** .5 for a, b in P]
        if mat.ndim >= 4:
            return np.array([[w[I] * w[J] * mat[P[I][0], P[I][1], P[J][0], P[J][1]]
                              for J in range(len(P))] for I in range(len(P))])
        return np.array([w[I] * mat[P[I][0], P[I][1]] for I in range(len(P))])

    @staticmethod
    def create_voigt(mat):
        """(d,d,d,d) tensor -> (D,D) Voigt stiffness matrix (no weights)."""
        dim = mat.shape[0]
        P = _pairs(dim)
        return np.array([[mat[P[I][0], P[I][1], P[J][0], P[J][1]] for J in range(len(P))]
                         for I in range(len(P))])

    @staticmethod
    def mandel_to_voigt(C):
        """Convert a Mandel stiffness matrix (or a field of them) to Voigt."""
        D = C.shape[0]
        dim = 3 if D == 6 else 2
        w = np.array([1. if a == b else 2 ** .5 for a, b in _pairs(dim)])
        shp = (D, D) + (1,) * (C.ndim - 2)
        return C / (w[:, None] * w[None, :]).reshape(shp)

    def __repr__(self):
        ss = 'Class: %s\n' % self.__class__.__name__
        ss += '    stiffness = %s (%s)\n' % (self.stiffness, self.val_type)
        ss += '    dim = %d' % self.dim + ('\n' if self.plane is None else ' (plane %s)\n' % self.plane)
        ss += '    bulk = %s\n    mu = %s\n' % (self.bulk, self.mu)
        return ss
