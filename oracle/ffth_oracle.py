"""NumPy restatement of FFTHomPy's Fourier-Galerkin homogenisation (oracle).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py as the checker; the product package never imports it.

Every function cites the reference file:line whose algorithm it restates
(paths relative to the vondrejc/FFTHomPy repository).  Conventions:

* fields are real arrays of shape (d_v,) + N (component first, C order);
* the Fourier form is NumPy's r2c half spectrum over the last d axes
  (ffthompy/tensors/fft.py:39-43, ffthompy/trigpol.py:6 fft_form 'r');
* coefficients are arrays of shape (d_v, d_v) + N, applied by
  einsum('ij...,j...->i...') (ffthompy/tensors/objects.py:231-232);
* the inner product is the grid mean sum(x*y)/prod(N)
  (ffthompy/tensors/objects.py:634-635).
"""
import itertools

import numpy as np
import scipy.special as sps

__all__ = [
    'freq_ints', 'coordinates', 'projection_scalar', 'projection_elasticity',
    'green_operator', 'projection_elasticity_parts', 'apply_GA', 'scal', 'cg', 'get_inverse', 'Material',
    'project', 'assembly_matrix', 'solve_problem', 'mandel_isotropic',
    'bicg', 'cheby2term', 'grad_symbol', 'potential_preconditioner', 'scal_fourier', 'cg_fourier',
    'potential_operator', 'potential_rhs', 'potential_field', 'homog_potential',
]


# ----------------------------------------------------------------------------
# grids (ffthompy/trigpol.py)
# ----------------------------------------------------------------------------
def freq_ints(n, centered=False):
    """Integer frequencies of an n-point grid.

    trigpol.py:12-21 (Grid.get_ZNl): arange(fix(-n/2), fix(n/2+0.5)), either
    centred ('c') or ifftshift-ed (forms 0 and 'r').
    """
    z = np.arange(np.trunc(-n / 2.), np.trunc(n / 2. + 0.5)).astype(np.int64)
    return z if centered else np.fft.ifftshift(z)


def coordinates(N, Y):
    """Nodal coordinates, centred origin (trigpol.py:56-71)."""
    N = np.asarray(N, dtype=np.int64)
    d = N.size
    axes = [Y[i] * freq_ints(N[i], centered=True) / N[i] for i in range(d)]
    return np.stack(np.meshgrid(*axes, indexing='ij'))


def get_Nodd(N):
    """trigpol.py:216-218."""
    N = np.asarray(N, dtype=np.int64)
    return N - ((N + 1) % 2)


def _band_freqs(N, Ns, Y):
    """Frequencies xi of the solve grid Ns, masked to the band of grid N.

    Returns (xi list of broadcastable arrays on the full FFT grid Ns, band mask,
    zero-frequency mask).  The band is |k_i| <= (Nodd_i-1)/2, which is where
    projections.scalar/elasticity put nonzero entries after NyqNul zeroing
    (projections.py:37-42,102-105) and Tensor.enlarge zero padding
    (objects.py:428-467).
    """
    N = np.asarray(N)
    Ns = np.asarray(Ns)
    d = N.size
    h = (get_Nodd(N) - 1) // 2
    ks = [freq_ints(Ns[i]) for i in range(d)]
    shp = lambda i: tuple(Ns[i] if j == i else 1 for j in range(d))
    kk = [ks[i].reshape(shp(i)) for i in range(d)]
    band = np.ones(tuple(Ns), dtype=bool)
    for i in range(d):
        band &= (np.abs(kk[i]) <= h[i])
    xi = [kk[i] / Y[i] for i in range(d)]
    zero = np.zeros(tuple(Ns), dtype=bool)
    zero[(0,) * d] = True
    return xi, band, zero


def projection_scalar(N, Y, Ns=None):
    """Scalar Green projections (G1 curl-free, G2 div-free) on the full grid Ns.

    projections.py:9-112: G1 = xi xi^T/|xi|^2, G2 = I - G1, both zero at the
    mean frequency; computed on the odd-reduced grid and zero-padded.  With
    Ns = 2N-1 this is the band embedding of Tensor.enlarge (objects.py:428-467)
    WITHOUT its scale factor (see green_operator).
    Returns arrays (d, d) + Ns on NumPy's full (fftn) frequency layout.
    """
    N = np.asarray(N)
    Ns = N if Ns is None else np.asarray(Ns)
    d = N.size
    xi, band, zero = _band_freqs(N, Ns, Y)
    full = tuple(Ns)
    num = [[np.broadcast_to(xi[m] * xi[n], full) for n in range(d)] for m in range(d)]
    denom = sum(num[m][m] for m in range(d)).copy()
    denom[zero] = 1.
    G1 = np.zeros((d, d) + full)
    G2 = np.zeros((d, d) + full)
    for m in range(d):
        for n in range(m, d):
            G1[m, n] = num[m][n] / denom
            G2[m, n] = (m == n) - G1[m, n]
            G2[m, n][zero] = 0.
            G1[n, m] = G1[m, n]
            G2[n, m] = G2[m, n]
    G1 *= band
    G2 *= band
    return G1, G2


def projection_elasticity_parts(N, Y, Ns=None):
    """Mandel strain/stress projection parts [G1h, G1s, G2h, G2s].

    projections.py:114-267, restated term by term (S, G1h, W, Lamh, IS0); the
    Mandel shear order is 3<->(1,2), 4<->(0,2), 5<->(0,1) for d=3 and
    2<->(0,1) for d=2 (projections.py:196-229).
    Returns four arrays (D, D) + Ns, full fftn layout, band-masked, unscaled.
    """
    N = np.asarray(N)
    Ns = N if Ns is None else np.asarray(Ns)
    d = N.size
    D = d * (d + 1) // 2
    xi, band, zero = _band_freqs(N, Ns, Y)
    full = tuple(Ns)
    one = np.ones(full)
    num = [[xi[m] * xi[n] * one for n in range(d)] for m in range(d)]
    norm2 = sum(num[m][m] for m in range(d))
    norm4 = norm2 ** 2
    norm2 = norm2.copy()
    norm2[zero] = 1.
    norm4[zero] = 1.
    z = lambda: np.zeros((D, D) + full)
    G1h, S, W, Lamh, IS0 = z(), z(), z(), z(), z()
    r2 = 2 ** .5
    for m in range(d):
        S[m, m] = 2 * num[m][m] / norm2
        for n in range(d):
            G1h[m, n] = num[m][m] * num[n][n] / norm4
            Lamh[m, n] = one / d
            Lamh[m, n][zero] = 0.
    for m in range(D):
        IS0[m, m] = one
        IS0[m, m][zero] = 0.
    if d == 2:
        S[0, 2] = r2 * num[0][1] / norm2
        S[1, 2] = r2 * num[0][1] / norm2
        S[2, 2] = one
        S[2, 2][zero] = 0.
        G1h[0, 2] = r2 * num[0][0] * num[0][1] / norm4
        G1h[1, 2] = r2 * num[0][1] * num[1][1] / norm4
        G1h[2, 2] = 2 * num[0][0] * num[1][1] / norm4
        for m in range(d):
            for n in range(d):
                W[m, n] = num[m][m] / norm2
            W[2, m] = r2 * num[0][1] / norm2
    else:
        for m in range(d):
            S[m + 3, m + 3] = 1 - num[m][m] / norm2
            S[m + 3, m + 3][zero] = 0.
        for m in range(d):
            for n in range(m + 1, d):
                S[m + 3, n + 3] = num[m][n] / norm2
                G1h[m + 3, n + 3] = num[m][m] * num[n][n] / norm4
        for m in range(d):
            for n in range(d):
                ind = [i for i in range(d) if i != n]
                S[m, n + 3] = (m != n) * r2 * num[ind[0]][ind[1]] / norm2
                G1h[m, n + 3] = r2 * num[m][m] * num[ind[0]][ind[1]] / norm4
                W[m, n] = num[m][m] / norm2
                W[n + 3, m] = r2 * num[ind[0]][ind[1]] / norm2
        for m in range(d):
            for n in range(d):
                im = [i for i in range(d) if i != m]
                jn = [i for i in range(d) if i != n]
                G1h[m + 3, n + 3] = 2 * num[im[0]][im[1]] * num[jn[0]][jn[1]] / norm4
    for n in range(D):
        for m in range(n + 1, D):
            S[m, n] = S[n, m]
            G1h[m, n] = G1h[n, m]
    G1s = S - 2 * G1h
    WT = np.swapaxes(W, 0, 1)
    G2h = 1. / (d - 1) * (d * Lamh + G1h - W - WT)
    G2s = IS0 - G1h - G1s - G2h
    return [G1h * band, G1s * band, G2h * band, G2s * band]


def projection_elasticity(N, Y, Ns=None):
    """G1 = G1h + G1s and G2 = G2h + G2s of projection_elasticity_parts."""
    G1h, G1s, G2h, G2s = projection_elasticity_parts(N, Y, Ns)
    return G1h + G1s, G2h + G2s


def _as_r_form(G, N, physics):
    """Rounding of the 0 -> 'r' form conversion of projections.scalar/elasticity.

    set_fft_form('r') multiplies by prod(N) (objects.py:164-165); the builders
    then divide by prod(N) (scalar, projections.py:107-110) or multiply by its
    reciprocal (elasticity, projections.py:262-265).  Restated so that the
    oracle's multiplier carries the same roundoff as the reference's.
    """
    pN = float(np.prod(N))
    G = G * pN
    return G / pN if physics == 'scalar' else (1. / pN) * G


def _enlarge_scale(G, N, M):
    """Scale of Tensor.enlarge 'r' -> 'c' -> 'r' (objects.py:154,160,437-467)."""
    return (1. / float(np.prod(N)) * G) * float(np.prod(M))


def green_operator(physics, N, Y, kind, proj):
    """Half-spectrum Green multiplier used by FiGFA (applications.py:24-37).

    kind 'GaNi': solve grid N.  kind 'Ga': solve grid 2N-1 and the multiplier
    is scaled by prod(2N-1)/prod(N): Tensor.enlarge converts 'r'->'c' with
    1/prod(N) (objects.py:154) and back 'c'->'r' with prod(M) (objects.py:160).
    Elasticity multipliers are the sums G1h+G1s / G2h+G2s formed after these
    conversions (applications.py:113-122).  Returns (G_half, Ns).
    """
    N = np.asarray(N, dtype=np.int64)
    Ns = N if kind == 'GaNi' else 2 * N - 1
    if physics == 'scalar':
        G1, G2 = projection_scalar(N, Y, Ns)
        parts = [G1 if proj == 1 else G2]
    else:
        parts = projection_elasticity_parts(N, Y, Ns)[2 * (proj - 1):2 * proj]
    out = 0.
    for G in parts:
        G = _as_r_form(G, N, physics)
        if kind == 'Ga':
            G = _enlarge_scale(G, N, Ns)
        out = G + out
    return np.ascontiguousarray(out[..., :Ns[-1] // 2 + 1]), Ns


# ----------------------------------------------------------------------------
# operator and solver
# ----------------------------------------------------------------------------
def apply_GA(G_half, A, x):
    """FiGFA(x) = iF( G . F( A . x ) )  (applications.py:58, operators.py:136-144).

    A . x: einsum 'ij...,j...->i...' (objects.py:231-232); F: unnormalised rfftn
    (fft.py:39-40); G.xhat: einsum in Fourier space; iF: irfftn (fft.py:42-43).
    """
    N = x.shape[1:]
    axes = tuple(range(1, 1 + len(N)))
    q = np.einsum('ij...,j...->i...', A, x)
    qh = np.fft.rfftn(q, s=N, axes=axes)
    qh = np.einsum('ij...,j...->i...', G_half, qh)
    return np.fft.irfftn(qh, s=N, axes=axes)


def scal(x, y):
    """Grid-mean L2 product (objects.py:634-635)."""
    return float(np.sum(x * y) / np.prod(x.shape[1:]))


def cg(Afun, B, x0, tol=1e-6, maxiter=1000, callback=None):
    """Conjugate gradients with the absolute residual test (solver.py:80-139).

    Returns (x, {'kit', 'norm_res', 'res_log'}).  With callback given, it is
    called with x0 first (solver.py:17-18) and with each iterate
    (solver.py:135-136), as linear_solver does.
    """
    if callback is not None:
        callback(x0)
    x = x0
    R = B - Afun(x0)
    P = R
    rr = scal(R, R)
    kit = 0
    norm_res = np.double(rr) ** 0.5
    log = [norm_res]
    while norm_res > tol and kit < maxiter:
        kit += 1
        AP = Afun(P)
        alp = float(rr / scal(P, AP))
        x = x + alp * P
        R = R - alp * AP
        rrnext = scal(R, R)
        bet = rrnext / rr
        rr = rrnext
        P = R + bet * P
        norm_res = np.double(rr) ** 0.5
        log.append(norm_res)
        if callback is not None:
            callback(x)
    if kit == 0:
        norm_res = 0
    return x, {'kit': kit, 'norm_res': norm_res, 'res_log': log}


def bicg(Afun, ATfun, B, x0, tol=1e-6, maxiter=1000):
    """BiConjugate gradients (solver.py:142-204): shadow residual Rs with
    ATfun, rr = <R, Rs>, stop on sqrt(rr) <= tol (absolute)."""
    x = x0
    R = B - Afun(x0)
    Rs = R
    rr = scal(R, Rs)
    P, Ps = R, Rs
    kit = 0
    norm_res = rr ** 0.5
    log = [norm_res]
    while norm_res > tol and kit < maxiter:
        kit += 1
        AP = Afun(P)
        alp = rr / scal(AP, Ps)
        x = x + alp * P
        R = R - alp * AP
        Rs = Rs - alp * ATfun(Ps)
        rrnext = scal(R, Rs)
        bet = rrnext / rr
        rr = rrnext
        P = R + bet * P
        Ps = Rs + bet * Ps
        norm_res = rr ** 0.5
        log.append(norm_res)
    if kit == 0:
        norm_res = 0
    return x, {'kit': kit, 'norm_res': norm_res, 'res_log': log}


def cheby2term(Afun, B, x0, eigrange, tol=1e-6, maxit=1e7):
    """Chebyshev two-term iteration (solver.py:206-285) on the eigenvalue
    interval eigrange; norm_res is |r| / |r0| in the grid-mean norm."""
    kit = 0
    bnrm2 = scal(B, B) ** 0.5
    Ib = 1.0 / bnrm2
    x = x0
    r = B - Afun(x)
    r0 = np.double(scal(r, r)) ** 0.5
    norm_res = Ib * r0
    if norm_res < tol:
        return x, {'kit': kit, 'norm_res': norm_res}
    d = (eigrange[1] + eigrange[0]) / 2.0
    c = (eigrange[1] - eigrange[0]) / 2.0
    v = 0 * x0
    w = 0.
    while norm_res > tol and kit < maxit:
        kit += 1
        x_prev = x
        if kit == 1:
            p = 0
            w = 1 / d
        elif kit == 2:
            p = -(1 / 2) * (c / d) * (c / d)
            w = 1 / (d - c * c / 2 / d)
        else:
            p = -(c * c / 4) * w * w
            w = 1 / (d - c * c * w / 4)
        v = r - p * v
        x = x_prev + w * v
        r = B - Afun(x)
        norm_res = (1.0 / r0) * scal(r, r) ** 0.5
    if kit == 0:
        norm_res = 0
    return x, {'kit': kit, 'norm_res': norm_res}


def get_inverse(A):
    """Per-voxel Gauss-Jordan inverse without pivoting (trigpol.py:120-159)."""
    B = np.array(A, dtype=np.float64, copy=True)
    d = A.shape[0]
    N = A.shape[2:]
    inv = [[np.full(N, float(m == n)) for n in range(d)] for m in range(d)]
    Bl = [[B[m, n] for n in range(d)] for m in range(d)]
    for m in range(d):
        piv = Bl[m][m].copy()
        Bl[m][m] = np.ones(N)
        for n in range(m + 1, d):
            Bl[m][n] = Bl[m][n] / piv
        for n in range(d):
            inv[m][n] = inv[m][n] / piv
        for k in range(m + 1, d):
            f = Bl[k][m].copy()
            for l in range(d):
                Bl[k][l] = Bl[k][l] - Bl[m][l] * f
                inv[k][l] = inv[k][l] - inv[m][l] * f
    for m in range(d - 1, -1, -1):
        for k in range(m - 1, -1, -1):
            f = Bl[k][m].copy()
            for l in range(d):
                Bl[k][l] = Bl[k][l] - Bl[m][l] * f
                inv[k][l] = inv[k][l] - inv[m][l] * f
    return np.array(inv)


# ----------------------------------------------------------------------------
# materials (ffthompy/materials.py)
# ----------------------------------------------------------------------------
_CUBE = ('cube', 'square')
_BALL = ('ball', 'circle')
_PYRAMID = ('bilinear_pyramid', 'pyramid')


def _cfftnc(x, N):
    """fft.py:4-9 (centred real and Fourier FFT, normalised by 1/prod(N))."""
    ax = tuple(range(x.ndim - len(N), x.ndim))
    return np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(x, ax), s=tuple(N), axes=ax), ax) \
        / np.prod(N)


def _icfftnc(X, N):
    """fft.py:11-16."""
    ax = tuple(range(X.ndim - len(N), X.ndim))
    return np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(X, ax), s=tuple(N), axes=ax),
                           ax).real * np.prod(N)


def _decrease(x, M):
    """trigpol.py:191-214: central crop of a centred spectrum."""
    M = np.asarray(M)
    N = np.asarray(x.shape)
    ibeg = np.trunc((N - M + (M % 2)) / 2).astype(int)
    iend = np.trunc((N + M + (M % 2)) / 2).astype(int)
    return x[tuple(slice(b, e) for b, e in zip(ibeg, iend))]


def _sep_product(N, factors):
    """Outer product over axes of 1D arrays factors[i] (length N[i])."""
    out = np.ones(tuple(N))
    d = len(N)
    for i, f in enumerate(factors):
        out = out * f.reshape(tuple(N[i] if j == i else 1 for j in range(d)))
    return out


def weights_con(h, Nbar, Y):
    """materials.py:333-359: sinc weights of a box of sides h."""
    Nbar = np.asarray(Nbar)
    d = Nbar.size
    return _sep_product(Nbar, [h[i] * np.sinc(h[i] * freq_ints(Nbar[i], True) / Y[i])
                               for i in range(d)]) / np.prod(Y)


def weights_lin(h, Nbar, Y):
    """materials.py:362-389: squared-sinc weights of a bilinear pyramid."""
    Nbar = np.asarray(Nbar)
    d = Nbar.size
    return _sep_product(Nbar, [h[i] * np.sinc(h[i] * freq_ints(Nbar[i], True) / Y[i]) ** 2
                               for i in range(d)]) / np.prod(Y)


def weights_circ(r, Nbar, Y):
    """materials.py:392-425: disc transform r^2 J1(2 pi r|xi|)/(r|xi|) (any d)."""
    Nbar = np.asarray(Nbar)
    d = Nbar.size
    circ = np.zeros(tuple(Nbar))
    for m in range(d):
        f = (freq_ints(Nbar[m], True) / Y[m]) ** 2
        circ = circ + f.reshape(tuple(Nbar[m] if j == m else 1 for j in range(d)))
    circ = circ ** 0.5
    ind = tuple(Nbar // 2)
    circ[ind] = 1.
    W = r ** 2 * sps.jv(1, 2 * np.pi * circ * r) / (circ * r)
    W[ind] = np.pi * r ** 2
    return W / np.prod(Y)


def _shift_inclusion(N, h, Y):
    """materials.py:317-330 (phase factor; uses the ifftshift-ed frequencies)."""
    N = np.asarray(N)
    d = N.size
    return _sep_product(N, [np.exp(-2 * np.pi * 1j * (h[i] * freq_ints(N[i]) / Y[i]))
                            for i in range(d)]).astype(np.complex128)


class Material:
    """Coefficient fields on a grid (materials.py:15-301).

    conf is the reference's material dictionary: either {'fun', 'Y', ...} or
    {'inclusions', 'positions', 'params', 'vals', 'Y', 'order', 'P'}.
    Returned coefficients are arrays (d_v, d_v) + N with origin 0 (after the
    Tensor.shift of materials.py:112-113,123, i.e. ifftshift).
    """

    def __init__(self, conf):
        self.conf = dict(conf)
        self.Y = np.asarray(conf['Y'], dtype=np.float64)
        if 'inclusions' in self.conf:
            pos = list(self.conf['positions'])
            for ii, incl in enumerate(self.conf['inclusions']):
                if incl in ('all', 'otherwise'):
                    continue
                pos[ii] = np.asarray(pos[ii]) % self.Y      # materials.py:47
            self.conf['positions'] = pos
        elif 'fun' not in self.conf:
            raise NotImplementedError('Improper material definition!')

    # materials.py:212-301 (periodic images of each inclusion on the nodes)
    def topologies(self, coord):
        incs, params, poss = self.conf['inclusions'], self.conf['params'], self.conf['positions']
        d = coord.shape[0]
        grid = coord.shape[1:]
        images = list(itertools.product((-1, 0, 1), repeat=d))
        topos = []
        for ii, kind in enumerate(incs):
            if kind in _CUBE:
                p = np.asarray(params[ii], dtype=np.float64)
                x0 = np.asarray(poss[ii], dtype=np.float64)
                t = np.zeros(grid)
                for im in images:
                    loc = np.ones(grid)
                    for dd in range(d):
                        u = coord[dd] - x0[dd] + self.Y[dd] * im[dd]
                        loc = loc * (u > -p[dd] / 2) * (u <= p[dd] / 2)
                    t += loc
            elif kind in _BALL:
                x0 = np.asarray(poss[ii], dtype=np.float64)
                t = np.zeros(grid)
                for im in images:
                    r2 = sum((coord[dd] - x0[dd] - self.Y[dd] * im[dd]) ** 2 for dd in range(d))
                    t += (r2 ** 0.5 < params[ii] / 2)
            elif kind in _PYRAMID:
                p = np.asarray(params[ii], dtype=np.float64)
                x0 = np.asarray(poss[ii], dtype=np.float64)
                t = np.zeros(grid)
                for im in images:
                    loc = np.ones(grid)
                    for dd in range(d):     # materials.py:283 shifts by 2*Y*image
                        u = coord[dd] - x0[dd] + 2 * self.Y[dd] * im[dd]
                        loc = loc * np.maximum(1 - np.abs(u) / (p[dd] / 2.), 0.)
                    t += loc
            elif kind == 'otherwise':
                t = np.ones(grid)
                for prev in topos:
                    t = t - prev
                if not (t >= 0).all():
                    raise NotImplementedError('Overlapping inclusions!')
            elif kind == 'all':
                t = np.ones(grid)
            else:
                raise NotImplementedError('Inclusion (%s) is not implemented.' % kind)
            topos.append(t)
        return topos

    def evaluate(self, coord):
        """materials.py:171-210 (values on the nodes, centred origin)."""
        if 'fun' in self.conf:
            return np.asarray(self.conf['fun'](coord), dtype=np.float64)
        vals = self.conf['vals']
        A = np.zeros(np.shape(vals[0]) + coord.shape[1:])
        for v, t in zip(vals, self.topologies(coord)):
            A += np.multiply.outer(np.asarray(v, dtype=np.float64), t)
        return A

    def _shift(self, A):
        return np.fft.ifftshift(A, axes=tuple(range(2, A.ndim)))

    def get_A_GaNi(self, N, primaldual='primal'):
        """materials.py:115-123."""
        A = self.evaluate(coordinates(N, self.Y))
        if primaldual == 'dual':
            A = get_inverse(A)
        return self._shift(A)

    def shape_functions(self, Nbar):
        """materials.py:125-169 (characteristic functions, exact integration)."""
        Nbar = np.asarray(Nbar)
        chars = []
        SS = None
        for ii, incl in enumerate(self.conf['inclusions']):
            pos = self.conf['positions'][ii]
            if isinstance(pos, np.ndarray):
                SS = _shift_inclusion(Nbar, pos, self.Y)
            p = self.conf['params'][ii]
            if incl in _CUBE:
                chars.append(_icfftnc(SS * weights_con(p, Nbar, self.Y), Nbar))
            elif incl in _BALL:
                r = p / 2
                W = np.zeros(tuple(Nbar)) if r == 0 else weights_circ(r, Nbar, self.Y)
                chars.append(_icfftnc(SS * W, Nbar))
            elif incl in _PYRAMID:
                chars.append(_icfftnc(SS * weights_lin(np.asarray(p) / 2., Nbar, self.Y), Nbar))
            elif incl == 'all':
                chars.append(np.ones(tuple(Nbar)))
            elif incl == 'otherwise':
                c = np.ones(tuple(Nbar))
                for prev in chars:
                    c = c - prev
                chars.append(c)
            else:
                raise NotImplementedError('The inclusion (%s) is not supported!' % incl)
        return chars

    def get_A_Ga(self, Nbar, primaldual='primal', order=-1, P=None):
        """materials.py:54-113 (inclusion-based or grid-based composite)."""
        Nbar = np.asarray(Nbar, dtype=np.int64)
        if order == -1:
            if 'order' not in self.conf:
                raise ValueError('The material order is undefined!')
            order = self.conf['order']
        elif order not in (None, 'exact', 0, 1):
            raise ValueError('Wrong material order (%s)!' % str(order))
        if order in (None, 'exact'):
            chars = self.shape_functions(Nbar)
            vals = self.conf['vals']
            val = np.zeros(np.shape(vals[0]) + tuple(Nbar))
            for v, c in zip(vals, chars):
                v = np.asarray(v, dtype=np.float64)
                if primaldual == 'dual':
                    v = np.linalg.inv(v)
                val += np.multiply.outer(v, c)
        else:
            if P is None and 'P' in self.conf:
                P = self.conf['P']
            P = np.asarray(P, dtype=np.int64)
            vals = self.evaluate(coordinates(P, self.Y))
            if primaldual == 'dual':
                vals = get_inverse(vals)
            h = self.Y / P
            Wraw = weights_con(h, Nbar, self.Y) if order in (0, 'constant') \
                else weights_lin(h, Nbar, self.Y)
            val = np.zeros(vals.shape[:2] + tuple(Nbar))
            for m, n in itertools.product(range(vals.shape[0]), range(vals.shape[1])):
                hAM0 = np.prod(P) * _cfftnc(vals[m, n], P)
                if np.allclose(P, Nbar):
                    hAM = hAM0
                elif np.all(P >= Nbar):
                    hAM = _decrease(hAM0, Nbar)
                elif np.all(P < Nbar):
                    factor = np.ceil(Nbar.astype(np.float64) / 2 / P).astype(int)
                    hAM = _decrease(np.tile(hAM0, 2 * factor + 1), Nbar)
                else:
                    raise NotImplementedError('grid combination N=%s P=%s' % (Nbar, P))
                val[m, n] = _icfftnc(Wraw * hAM, Nbar).real
        return self._shift(val)


# ----------------------------------------------------------------------------
# postprocessing (ffthompy/postprocess.py, objects.py:428-511)
# ----------------------------------------------------------------------------
def project(x, M):
    """Trigonometric interpolation of a real field (d_v,)+N to grid M.

    Tensor.project (objects.py:488-511) = rfftn, Tensor.enlarge in centred
    form with the even-N Nyquist split 0.5*X[-N/2] / 0.5*conj (objects.py:
    441-453), centred zero padding, irfftn on M.
    """
    N = np.asarray(x.shape[1:])
    M = np.asarray(M)
    if np.all(N == M):
        return x
    d = N.size
    ax = tuple(range(1, d + 1))
    X = np.fft.fftshift(np.fft.fftn(x, axes=ax), axes=ax) / np.prod(N)
    for i, a in enumerate(ax):
        if N[i] % 2 == 0:
            n0 = np.take(X, [0], axis=a)
            rest = np.take(X, np.arange(1, X.shape[a]), axis=a)
            n2 = n0.copy()
            for j, b in enumerate(ax):
                if b == a:
                    continue
                if n2.shape[b] % 2 == 0:
                    n20 = np.take(n2, [0], axis=b)
                    n2c = np.take(n2, np.arange(1, n2.shape[b]), axis=b)
                    n2 = np.concatenate((n20, np.flip(n2c, axis=b)), axis=b)
                else:
                    n2 = np.flip(n2, axis=b)
            X = np.concatenate((0.5 * n0, rest, 0.5 * n2.conj()), axis=a)
    Nc = np.asarray(X.shape[1:], dtype=np.float64)
    ibeg = np.ceil((M - Nc) / 2).astype(int)
    iend = np.ceil((M + Nc) / 2).astype(int)
    Y = np.zeros((x.shape[0],) + tuple(M), dtype=np.complex128)
    Y[(slice(None),) + tuple(slice(b, e) for b, e in zip(ibeg, iend))] = X
    Y = np.fft.ifftshift(Y, axes=ax)
    return np.fft.ifftn(Y, axes=ax).real * np.prod(M)


def assembly_matrix(A, solutions):
    """A_H[i,j] = <A sol_i, sol_j> (postprocess.py:53-70)."""
    Nbar = A.shape[2:]
    sols = [project(s, Nbar) for s in solutions]
    L = len(sols)
    AH = np.zeros((L, L))
    for i, j in itertools.product(range(L), repeat=2):
        AH[i, j] = scal(np.einsum('ij...,j...->i...', A, sols[i]), sols[j])
    return AH


def mandel_isotropic(bulk, mu, dim=3):
    """Mandel matrix of an isotropic stiffness (mechanics/matcoef.py:4-72,152-208).

    C = 3K * vol + 2mu * dev; in Mandel notation this is
    K*11^T (normal block, d=3) + 2mu*(I - 11^T/3); plane strain (d=2) keeps
    rows/cols (0, 1, 5) of the 3D matrix (matcoef.py:74-97).
    """
    I6 = np.eye(6)
    J = np.zeros((6, 6))
    J[:3, :3] = 1. / 3
    C = 3. * bulk * J + 2. * mu * (I6 - J)
    if dim == 2:
        idx = [0, 1, 5]
        C = C[np.ix_(idx, idx)]
    return C


# ----------------------------------------------------------------------------
# the application driver (ffthompy/applications.py:11-176)
# ----------------------------------------------------------------------------
def solve_problem(problem, as_shipped=False, verbose=False):
    """Run one problem definition through the restated pipeline.

    problem: dict with keys physics, material, solve {kind, N, primaldual},
    solver {tol, maxiter}, postprocess (list).  Mirrors applications.scalar /
    applications.elasticity and postprocess.postprocess.  as_shipped=True adds
    the reference's per-iteration CallBack residual matvec
    (solver_pp.py:13-24, installed at applications.py:71-72).
    Returns dict with mat_<pd>, sol_<pd>, res_<pd> (kit, norm_res).
    """
    physics = problem['physics']
    mconf = problem['material']
    Y = np.asarray(mconf['Y'], dtype=np.float64)
    d = Y.size
    N = np.asarray(problem['solve']['N'], dtype=np.int64)
    kind = problem['solve']['kind']
    L = d if physics == 'scalar' else d * (d + 1) // 2
    tol = problem['solver'].get('tol', 1e-6)
    maxiter = problem['solver'].get('maxiter', 1e3)
    out = {}
    for pd in problem['solve']['primaldual']:
        G, Ns = green_operator(physics, N, Y, kind, 1 if pd == 'primal' else 2)
        mat = Material(mconf)
        if kind == 'GaNi':
            A = mat.get_A_GaNi(N, pd)
            A_name = 'A_GaNi'
        else:
            A = mat.get_A_Ga(Ns, pd)
            A_name = 'A_Ga'
        Afun = lambda v: apply_GA(G, A, v)
        sols, res = [], []
        for iL in range(L):
            EN = np.zeros((L,) + tuple(Ns))
            EN[iL] = 1.
            B = Afun(-EN)
            x0 = np.zeros_like(EN)
            cb = None
            if as_shipped:
                cb = lambda v: float(np.sqrt(scal(B - Afun(v), B - Afun(v))))
            X, info = cg(Afun, B, x0, tol=tol, maxiter=maxiter, callback=cb)
            sols.append(X + EN)
            res.append(info)
        mats = {}
        for pp in problem['postprocess']:
            Ap = A
            if pp['kind'] in ('GaNi', 'gani'):
                order_name, Nname = '', ''
                if A_name != 'A_GaNi' or pd == 'dual':
                    Ap = mat.get_A_GaNi(N, pd)
            elif pp['kind'] in ('Ga', 'ga'):
                order_name, Nname = '', ''
                if 'order' in pp:
                    Npp = 2 * N - 1
                    if pp['order'] is None:
                        Ap = mat.get_A_Ga(Npp, pd, order=None)
                    else:
                        order_name = '_o' + str(pp['order'])
                        Nname = '_P%d' % np.mean(pp['P'])
                        Ap = mat.get_A_Ga(Npp, pd, order=pp['order'], P=pp['P'])
            else:
                raise ValueError(pp['kind'])
            name = 'AH_%s%s%s_%s' % (pp['kind'], order_name, Nname, pd)
            AH = assembly_matrix(Ap, sols)
            mats[name] = AH if pd == 'primal' else np.linalg.inv(AH)
        out['mat_' + pd] = mats
        out['sol_' + pd] = sols
        out['res_' + pd] = res
    return out


# ----------------------------------------------------------------------------
# potential formulation (ffthompy/tensorsLowRank/homogenisation.py:41-127)
# ----------------------------------------------------------------------------
# The unknown is the scalar potential u in the 'r' Fourier form of the N grid
# (unnormalised half spectrum); the CG iterates are such spectra and the
# inner product is the 'r' branch of scalar_product.
def grad_symbol(N, Y):
    """2 pi i xi on the 'r' half spectrum of grid N: grad_tensor
    (tensors/operators.py:371-386) with frequencies Grid.get_xil (trigpol.py:
    27-40; even N: the Nyquist index carries -N/2, also on the last axis)."""
    N = np.asarray(N, dtype=np.int64)
    Y = np.asarray(Y, dtype=np.float64)
    d = N.size
    xi = [freq_ints(int(n)) / Y[i] for i, n in enumerate(N)]
    xi[-1] = xi[-1][:N[-1] // 2 + 1]
    shape = tuple(len(x) for x in xi)
    out = np.zeros((d,) + shape, dtype=np.complex128)
    for i in range(d):
        sh = [1] * d
        sh[i] = shape[i]
        out[i] = np.broadcast_to(xi[i].reshape(sh), shape)
    return out * 2 * np.pi * 1j


def potential_preconditioner(N, Y):
    """P = 1/|2 pi xi| with 1 at the mean index (homogenisation.py:296-300)."""
    h = grad_symbol(N, Y)
    k2 = np.einsum('i...,i...', h, np.conj(h)).real
    k2[(0,) * len(N)] = 1.
    return 1. / k2 ** 0.5


def scal_fourier(x, y, N):
    """scalar_product of two 'r' form Fourier tensors (objects.py:618-631)."""
    M2 = float(np.prod(N)) ** 2
    if N[-1] % 2 == 1:
        s = (np.sum(y[..., 0] * np.conj(x[..., 0])).real +
             2 * np.sum(y[..., 1:] * np.conj(x[..., 1:])).real)
    else:
        s = (np.sum(y[..., 0] * np.conj(x[..., 0])).real +
             np.sum(y[..., -1] * np.conj(x[..., -1])).real +
             2 * np.sum(y[..., 1:-1] * np.conj(x[..., 1:-1])).real)
    return float(s / M2)


def cg_fourier(Afun, B, x0, N, tol=1e-6, maxiter=1000):
    """CG (solver.py:80-139) with the 'r' Fourier inner product (get_scal picks
    X*Y = scalar_product for Tensors, solver.py:287-298)."""
    x = x0
    R = B - Afun(x0)
    P = R
    rr = scal_fourier(R, R, N)
    kit = 0
    norm_res = np.double(rr) ** 0.5
    log = [norm_res]
    while norm_res > tol and kit < maxiter:
        kit += 1
        AP = Afun(P)
        alp = float(rr / scal_fourier(P, AP, N))
        x = x + alp * P
        R = R - alp * AP
        rrnext = scal_fourier(R, R, N)
        bet = rrnext / rr
        rr = rrnext
        P = R + bet * P
        norm_res = np.double(rr) ** 0.5
        log.append(norm_res)
    if kit == 0:
        norm_res = 0
    return x, {'kit': kit, 'norm_res': norm_res, 'res_log': log}


def _r_axes(d, lead):
    return tuple(range(lead, lead + d))


def _enlarge_r(X, N, M):
    """Tensor.enlarge of 'r' Fourier tensors (objects.py:428-467) for odd N:
    centred zero padding with the 'r' <-> 'c' scalings 1/prod(N), prod(M).
    For odd N the spectra here are Hermitian (rfftn of real fields), so the
    padding equals the trigonometric interpolation of the real field."""
    d = len(N)
    ax = _r_axes(d, X.ndim - d)
    x = np.fft.irfftn(X, s=tuple(N), axes=ax)
    return np.fft.rfftn(project(x.reshape((-1,) + tuple(N)), M).reshape(
        X.shape[:X.ndim - d] + tuple(M)), axes=ax)


def _decrease_r(X, M, N):
    """Tensor.decrease / project to a smaller grid (objects.py:469-511 with
    trigpol.py:191-214) for odd N and M: the centred band of N, scaled by
    prod(N)/prod(M)."""
    d = len(N)
    lead = X.shape[:X.ndim - d]
    ax = _r_axes(d, len(lead))
    full = np.fft.fftn(np.fft.irfftn(X, s=tuple(M), axes=ax), axes=ax)
    idx = np.ix_(*[np.fft.ifftshift(np.arange(-(n // 2), n // 2 + 1)) % m
                   for n, m in zip(N, M)])
    out = full[(Ellipsis,) + idx] * (float(np.prod(N)) / float(np.prod(M)))
    return out[..., :N[-1] // 2 + 1]


def _grad(X, N, Y):
    return grad_symbol(N, Y) * X[None]


def _div(X, N, Y):
    return np.einsum('i...,i...->...', grad_symbol(N, Y), X)


def potential_operator(A, N, Y, Nbar=None):
    """PDFAFGPfun (homogenisation.py:61-67, 97-103) as a function of the
    preconditioned potential: P (-div F(A iF(grad(P x)))), with the Ga
    enlargement to Nbar and projection back to N when Nbar is given."""
    N = tuple(int(n) for n in N)
    P = potential_preconditioner(N, Y)
    d = len(N)
    Ns = N if Nbar is None else tuple(int(n) for n in Nbar)
    ax = _r_axes(d, 1)

    def afun(x):
        g = _grad(P * x, N, Y)
        if Nbar is not None:
            g = _enlarge_r(g, N, Ns)
        e = np.fft.irfftn(g, s=Ns, axes=ax)
        q = np.einsum('ij...,j...->i...', A, e)
        Q = np.fft.rfftn(q, s=Ns, axes=ax)
        if Nbar is not None:
            Q = _decrease_r(Q, Ns, N)
        return P * (-_div(Q, N, Y))
    return afun


def potential_rhs(A, N, Y, load=0, Nbar=None):
    """P * B with B = div(F(A E)) (decreased to N for Ga), homogenisation.py:
    58, 95 (E = e_load)."""
    N = tuple(int(n) for n in N)
    d = len(N)
    Ns = N if Nbar is None else tuple(int(n) for n in Nbar)
    E = np.zeros((d,) + Ns)
    E[load] = 1.
    Q = np.fft.rfftn(np.einsum('ij...,j...->i...', A, E), s=Ns, axes=_r_axes(d, 1))
    if Nbar is not None:
        Q = _decrease_r(Q, Ns, N)
    return potential_preconditioner(N, Y) * _div(Q, N, Y)


def potential_field(x, N, Y, Ns=None):
    """X = iF(grad(P x)) on N, or iF2(grad(P x).project(Ns)) on the larger grid
    Ns (homogenisation.py:74-77, 117-124)."""
    N = tuple(int(n) for n in N)
    d = len(N)
    g = _grad(potential_preconditioner(N, Y) * x, N, Y)
    if Ns is None or tuple(Ns) == N:
        return np.fft.irfftn(g, s=N, axes=_r_axes(d, 1))
    Ns = tuple(int(n) for n in Ns)
    return np.fft.irfftn(_enlarge_r(g, N, Ns), s=Ns, axes=_r_axes(d, 1))


def homog_potential(A, N, Y, tol, maxiter, Nbar=None, A_post=None, load=0):
    """homog_GaNi_full_potential (homogenisation.py:83-127; Nbar None, A the
    GaNi coefficient on N, A_post the optional Ga coefficient on 2N-1) and
    homog_Ga_full_potential (homogenisation.py:41-81; A the Ga coefficient on
    Nbar).  Returns dict AH, iPU (CG solution), Fu = P iPU, info."""
    N = tuple(int(n) for n in N)
    afun = potential_operator(A, N, Y, Nbar)
    PB = potential_rhs(A, N, Y, load, Nbar)
    x0 = np.zeros_like(PB)
    iPU, info = cg_fourier(afun, PB, x0, N, tol=tol, maxiter=maxiter)
    Fu = potential_preconditioner(N, Y) * iPU
    if Nbar is not None:
        Ap, Ns = A, tuple(int(n) for n in Nbar)
    elif A_post is not None:
        Ap, Ns = A_post, tuple(int(n) for n in A_post.shape[2:])
    else:
        Ap, Ns = A, N
    X = potential_field(iPU, N, Y, Ns)
    X[load] += 1.
    AH = scal(np.einsum('ij...,j...->i...', Ap, X), X)
    return {'AH': AH, 'iPU': iPU, 'Fu': Fu, 'info': info}
