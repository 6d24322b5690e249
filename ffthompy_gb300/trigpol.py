"""Grids of trigonometric polynomials (host utilities).

Mirrors ffthompy/trigpol.py: Grid.get_ZNl / get_xil / get_coordinates
(trigpol.py:9-71), get_Nodd (216-218), mean_index (220-224) and the centred
spectrum crop/pad helpers enlarge / decrease (162-214).
"""
import numpy as np

fft_form_default = 'r'


def _ints(n, centered):
    z = np.arange(-(int(n) // 2), (int(n) + 1) // 2, dtype=np.int64)
    return z if centered else np.fft.ifftshift(z)


class Grid:
    @staticmethod
    def get_ZNl(N, fft_form=fft_form_default):
        """Integer frequencies per axis; centred for 'c', FFT order otherwise."""
        N = np.atleast_1d(np.asarray(N, dtype=np.int64))
        return [_ints(n, fft_form == 'c') for n in N]

    @staticmethod
    def get_xil(N, Y, fft_form=fft_form_default):
        out = [z / Y[i] for i, z in enumerate(Grid.get_ZNl(N, 'c'))]
        if fft_form in ('r', 0):
            out = [np.fft.ifftshift(x) for x in out]
            if fft_form == 'r':
                out[-1] = out[-1][:int(N[-1]) // 2 + 1]
        return out

    @staticmethod
    def get_coordinates(N, Y):
        """Nodes Y_i * k_i / N_i, centred origin, shape (d,) + N."""
        return np.stack(np.meshgrid(*Grid.get_axes(N, Y), indexing='ij'))

    @staticmethod
    def get_axes(N, Y):
        """The per-axis node coordinates of get_coordinates."""
        N = np.asarray(N, dtype=np.int64)
        return [Y[i] * _ints(N[i], True) / N[i] for i in range(N.size)]


def get_Nodd(N):
    N = np.asarray(N, dtype=np.int64)
    return N - ((N + 1) % 2)


def mean_index(N, fft_form=fft_form_default):
    N = np.asarray(N, dtype=np.int64)
    if fft_form in (0, 'r'):
        return tuple(np.zeros_like(N))
    return tuple(N // 2)


def decrease(xN, M):
    """Central crop of a centred spectrum to shape M."""
    M = np.asarray(M, dtype=np.int64)
    N = np.asarray(xN.shape, dtype=np.int64)
    ibeg = (N - M + (M % 2)) // 2
    return xN[tuple(slice(b, b + m) for b, m in zip(ibeg, M))]


def enlarge(xN, M):
    """Zero padding of a centred spectrum to shape M (odd sizes)."""
    M = np.asarray(M, dtype=np.int64)
    N = np.asarray(xN.shape, dtype=np.int64)
    if np.all(M == N):
        return xN
    ibeg = -((N - M) // 2)  # ceil((M-N)/2)
    out = np.zeros(tuple(M), dtype=xN.dtype)
    out[tuple(slice(b, b + n) for b, n in zip(ibeg, N))] = xN
    return out
