"""Seeded synthetic microstructures of the benchmark configurations.

The reference ships no generator for these geometries; they are defined by
their statistics and produce voxel images that feed both the GPU path and the
oracle as 'fun' materials (the pattern of examples/scalar/from_file.py:23-41):

* spheres  - scalar 3D: radius r, centres uniform in the unit cell, added until
  the union volume fraction on the voxel grid reaches vf (periodic, overlap
  allowed); phases 1 / contrast.
* fibres   - elasticity 3D: n parallel cylinders along x3 of radius r, centres
  uniform with periodic centre distance > min_dist; isotropic phases given by
  (E, nu) -> (K, mu).
* grf      - 2D thresholded Gaussian random field (squared-exponential
  covariance of correlation length ell, phase 1 above the q-quantile).
* exp_grf  - a(x) = exp(g(x)), g a Gaussian random field (mean 0, std 1).

Voxel centres are the reference's grid nodes Y*k/N, k centred
(ffthompy/trigpol.py:56-71).
"""
import numpy as np

from .mechanics.matcoef import ElasticTensor
from .trigpol import Grid


def _nodes(N, Y):
    return Grid.get_coordinates(N, Y)


def spheres_indicator(N, radius=0.08, vf=0.3, seed=0, Y=None):
    """Boolean (N0,N1,N2) image of a periodic union of spheres."""
    N = tuple(int(n) for n in N)
    Y = np.ones(3) if Y is None else np.asarray(Y, dtype=np.float64)
    rng = np.random.default_rng(seed)
    img = np.zeros(N, dtype=bool)
    axes = [Y[i] * (np.arange(N[i]) - N[i] // 2) / N[i] for i in range(3)]
    h = [Y[i] / N[i] for i in range(3)]
    target = vf * img.size
    count = 0
    centres = []
    while count < target:
        c = (rng.random(3) - 0.5) * Y
        centres.append(c)
        idx, dist2 = [], []
        for i in range(3):
            lo = int(np.floor((c[i] - radius - axes[i][0]) / h[i])) - 1
            hi = int(np.ceil((c[i] + radius - axes[i][0]) / h[i])) + 1
            k = np.arange(lo, hi + 1)
            x = axes[i][0] + k * h[i]
            dx = x - c[i]
            dx -= Y[i] * np.round(dx / Y[i])
            idx.append(np.mod(k, N[i]))
            dist2.append(dx ** 2)
        d2 = dist2[0][:, None, None] + dist2[1][None, :, None] + dist2[2][None, None, :]
        inside = d2 < radius ** 2
        sub = img[np.ix_(*idx)]
        newly = inside & ~sub
        if newly.any():
            sub |= inside
            img[np.ix_(*idx)] = sub
            count = int(img.sum())
    return img, np.array(centres)


def spheres_coefficient(N, radius=0.08, vf=0.3, contrast=100., seed=0):
    """Isotropic scalar coefficient (3,3)+N with a = contrast in spheres, 1 outside."""
    img, _ = spheres_indicator(N, radius, vf, seed)
    a = np.where(img, float(contrast), 1.0)
    return np.einsum('ij,...->ij...', np.eye(3), a)


def fibres_indicator(N, n_fibres=8, radius=0.12, min_dist=0.24, seed=0, max_tries=100000):
    """Boolean image of parallel periodic cylinders along x3 (non-overlapping)."""
    N = tuple(int(n) for n in N)
    rng = np.random.default_rng(seed)
    centres = []
    tries = 0
    while len(centres) < n_fibres:
        tries += 1
        if tries > max_tries:
            raise RuntimeError('could not place %d fibres' % n_fibres)
        c = rng.random(2) - 0.5
        ok = True
        for q in centres:
            d = c - q
            d -= np.round(d)
            if np.hypot(*d) <= min_dist:
                ok = False
                break
        if ok:
            centres.append(c)
    x = _nodes(N[:2], np.ones(2))
    img2 = np.zeros(N[:2], dtype=bool)
    for c in centres:
        dx = x[0] - c[0]
        dy = x[1] - c[1]
        dx -= np.round(dx)
        dy -= np.round(dy)
        img2 |= dx ** 2 + dy ** 2 < radius ** 2
    return np.repeat(img2[:, :, None], N[2], axis=2), np.array(centres)


def youngs_to_bulk_shear(E, nu):
    return E / (3. * (1. - 2. * nu)), E / (2. * (1. + nu))


def fibres_coefficient(N, phases=((1., 0.3), (10., 0.2)), **kw):
    """Mandel 6x6 stiffness per voxel: matrix phase outside, fibre phase inside."""
    img, _ = fibres_indicator(N, **kw)
    Cm = ElasticTensor(*youngs_to_bulk_shear(*phases[0])).mandel
    Cf = ElasticTensor(*youngs_to_bulk_shear(*phases[1])).mandel
    return np.einsum('ij,...->ij...', Cm, ~img) + np.einsum('ij,...->ij...', Cf, img)


def gaussian_field(N, ell, seed=0):
    """Periodic stationary Gaussian field (mean 0, std 1), squared-exponential
    covariance exp(-|x|^2 / (2 ell^2)), by spectral filtering of white noise."""
    N = tuple(int(n) for n in N)
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(N)
    k2 = np.zeros(N)
    for i, n in enumerate(N):
        f = np.fft.fftfreq(n) * n
        k2 = k2 + (f ** 2).reshape([n if j == i else 1 for j in range(len(N))])
    # spectral density of the SE covariance ~ exp(-2 pi^2 ell^2 |k|^2)
    amp = np.exp(-np.pi ** 2 * ell ** 2 * k2)
    g = np.fft.ifftn(np.fft.fftn(w) * amp).real
    g -= g.mean()
    return g / g.std()


def grf_phase_coefficient(N, ell=0.1, quantile=0.4, contrast=10., seed=0):
    """2D isotropic coefficient: contrast where g > q-quantile, 1 elsewhere."""
    g = gaussian_field(N, ell, seed)
    a = np.where(g > np.quantile(g, quantile), float(contrast), 1.0)
    return np.einsum('ij,...->ij...', np.eye(len(N)), a)


def exp_grf_coefficient(N, ell=0.15, seed=0):
    g = gaussian_field(N, ell, seed)
    return np.einsum('ij,...->ij...', np.eye(len(N)), np.exp(g))


def fun_material(values, Y=None, order=0):
    """A 'fun' material dictionary returning the given nodal values."""
    values = np.asarray(values, dtype=np.float64)
    grid = values.shape[2:]
    Y = np.ones(len(grid)) if Y is None else np.asarray(Y, dtype=np.float64)

    def fun(coord, _v=values):
        return _v
    return {'fun': fun, 'Y': Y, 'order': order, 'P': np.array(grid)}
