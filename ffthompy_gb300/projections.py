"""Green projections in Fourier space, mirroring ffthompy/projections.py.

scalar(N, Y) (projections.py:9-112) returns the mean, curl-free (G1) and
divergence-free (G2) projections; elasticity(N, Y) (projections.py:114-267)
returns G0, G1h, G1s, G2h, G2s in Mandel notation.  Here they are
descriptors: the CUDA library evaluates G(xi) on the fly inside the FFT
projection pass instead of storing (d,d)+N arrays.  enlarge(M) moves a
projection to the Ga grid M = 2N-1 with the reference's scale
prod(M)/prod(N) (Tensor.enlarge, ffthompy/tensors/objects.py:428-467).
"""
import numpy as np


class GreenProjection:
    Fourier = True
    fft_form = 'r'

    def __init__(self, physics, which, N, Y, band=None, scale=1.0, name=None):
        self.physics = physics
        self.which = which          # 'G0' | 'G1' | 'G2' | 'G1h' | 'G1s' | 'G2h' | 'G2s'
        self.N = tuple(int(n) for n in N)
        self.band = tuple(int(n) for n in (band if band is not None else N))
        self.Y = np.asarray(Y, dtype=np.float64)
        self.scale = float(scale)
        self.name = name or 'h' + which
        self.dim = len(self.N)
        self.order = 2
        self.multype = 21

    @property
    def proj(self):
        """1 for the compatible projection G1, 2 for the equilibrated G2."""
        if self.which == 'G1':
            return 1
        if self.which == 'G2':
            return 2
        raise NotImplementedError('projection %s is not applied on its own; use G1 = G1h+G1s '
                                  'or G2 = G2h+G2s' % self.which)

    def enlarge(self, M):
        M = tuple(int(m) for m in np.atleast_1d(M))
        if M == self.N:
            return self
        s = float(np.prod(M, dtype=np.float64) / np.prod(self.N, dtype=np.float64))
        return GreenProjection(self.physics, self.which, M, self.Y, self.band,
                               self.scale * s, self.name)

    def __add__(self, other):
        pair = {frozenset(('G1h', 'G1s')): 'G1', frozenset(('G2h', 'G2s')): 'G2'}
        key = frozenset((self.which, other.which))
        if key not in pair or self.N != other.N or self.scale != other.scale:
            raise NotImplementedError('sum of projections %s + %s' % (self.which, other.which))
        return GreenProjection(self.physics, pair[key], self.N, self.Y, self.band, self.scale,
                               'h' + pair[key])

    @property
    def val(self):
        raise NotImplementedError('the Green operator is evaluated on the fly on the GPU')

    def __repr__(self):
        return 'GreenProjection(%s, %s, N=%s, band=%s, scale=%g)' % (
            self.physics, self.which, self.N, self.band, self.scale)


def scalar(N, Y, NyqNul=True, tensor=True, fft_form='r'):
    if not NyqNul:
        raise NotImplementedError('only the Nyquist-free projections (NyqNul=True)')
    N = tuple(int(n) for n in np.atleast_1d(N))
    return tuple(GreenProjection('scalar', w, N, Y) for w in ('G0', 'G1', 'G2'))


def elasticity(N, Y, NyqNul=True, tensor=True, fft_form='r'):
    if not NyqNul:
        raise NotImplementedError('only the Nyquist-free projections (NyqNul=True)')
    N = tuple(int(n) for n in np.atleast_1d(N))
    return tuple(GreenProjection('elasticity', w, N, Y)
                 for w in ('G0', 'G1h', 'G1s', 'G2h', 'G2s'))
