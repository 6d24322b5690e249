"""Material coefficients on grids, mirroring ffthompy/materials.py.

Material(conf) accepts the reference's material dictionaries: either a
function {'fun': f(coord) -> (d_v, d_v) + grid, 'Y', 'order', 'P'} or
inclusions {'inclusions', 'positions', 'params', 'vals', 'Y', 'order', 'P'}.

* get_A_GaNi(N, primaldual): nodal values (materials.py:115-123, 171-301);
* get_A_Ga(Nbar, primaldual, order, P): exact-integration coefficient on the
  double grid, inclusion based (order None: sinc / squared-sinc / disc
  transforms, materials.py:66-75, 125-169, 333-425) or grid based (order 0 /
  1: Fourier coefficients of a P-voxel image weighted by the cell shape
  function, materials.py:77-110).

Coefficient assembly runs once per problem. On a GPU the grid-based Ga
coefficient (fhp_ga_grid_coefficient), the dual inverse
(fhp_coefficient_inverse), the Ga characteristic function of balls
(fhp_ball_characteristic), their GaNi topologies (fhp_ball_topology) and the
sum over inclusions of the exact-integration coefficient
(fhp_outer_accumulate) run in the CUDA library. Boxes and pyramids use separable host transforms; the
rest runs on the host (NumPy). The result is a Tensor with origin 0 on the
GPU.
"""
import itertools

import numpy as np
import scipy.special as sps

from .tensors.objects import Tensor
from .trigpol import Grid, decrease

inclusion_keys = {'ball': ['ball', 'circle'],
                  'cube': ['cube', 'square'],
                  'pyramid': ['bilinear_pyramid', 'pyramid']}


def _outer_axes(N, vecs):
    """prod_i vecs[i] broadcast along axis i of a grid of shape N."""
    out = np.ones(tuple(N))
    d = len(N)
    for i, v in enumerate(vecs):
        out = out * v.reshape([N[i] if j == i else 1 for j in range(d)])
    return out


def _centered_fft(x, shape):
    """Centred, 1/prod(N)-normalised DFT of a real grid image (fft.py:4-9)."""
    ax = tuple(range(x.ndim - len(shape), x.ndim))
    X = np.fft.fftn(np.fft.ifftshift(x, axes=ax), s=tuple(shape), axes=ax)
    return np.fft.fftshift(X, axes=ax) / np.prod(shape)


def _centered_ifft_real(X, shape):
    """Real part of the centred inverse DFT times prod(N) (fft.py:11-16)."""
    ax = tuple(range(X.ndim - len(shape), X.ndim))
    x = np.fft.ifftn(np.fft.ifftshift(X, axes=ax), s=tuple(shape), axes=ax)
    return np.fft.fftshift(x, axes=ax).real * np.prod(shape)


def get_weights_con(h, Nbar, Y):
    """Box of sides h: prod_i h_i sinc(h_i k_i / Y_i) / |Y| (materials.py:333-359)."""
    Nbar = np.asarray(Nbar, dtype=np.int64)
    Z = Grid.get_ZNl(Nbar, fft_form='c')
    return _outer_axes(Nbar, [h[i] * np.sinc(h[i] * Z[i] / Y[i]) for i in range(Nbar.size)]) \
        / np.prod(Y)


def get_weights_lin(h, Nbar, Y):
    """Bilinear pyramid of half-support h: squared sincs (materials.py:362-389)."""
    Nbar = np.asarray(Nbar, dtype=np.int64)
    Z = Grid.get_ZNl(Nbar, fft_form='c')
    return _outer_axes(Nbar, [h[i] * np.sinc(h[i] * Z[i] / Y[i]) ** 2
                              for i in range(Nbar.size)]) / np.prod(Y)


def get_weights_circ(r, Nbar, Y):
    """Disc of radius r: r^2 J1(2 pi r |xi|) / (r |xi|) (materials.py:392-425).

    The reference uses this planar formula in any dimension; kept as is.
    """
    Nbar = np.asarray(Nbar, dtype=np.int64)
    Z = Grid.get_ZNl(Nbar, fft_form='c')
    d = Nbar.size
    rad2 = np.zeros(tuple(Nbar))
    for m in range(d):
        rad2 = rad2 + ((Z[m] / Y[m]) ** 2).reshape([Nbar[m] if j == m else 1 for j in range(d)])
    rad = np.sqrt(rad2)
    c = tuple(Nbar // 2)
    rad[c] = 1.
    W = r ** 2 * sps.jv(1, 2 * np.pi * rad * r) / (rad * r)
    W[c] = np.pi * r ** 2
    return W / np.prod(Y)


def _centered_ifft_real_separable(vecs, shape):
    """_centered_ifft_real of the outer product of per-axis spectra vecs[i]:
    the d-dimensional transform of a separable product is the product of the
    1D transforms, so the cost is O(d N) transforms and one outer product
    (the real part is formed from the complex partial products)."""
    cs = [np.fft.fftshift(np.fft.ifft(np.fft.ifftshift(X))) * int(n)
          for X, n in zip(vecs, shape)]
    t = cs[0]
    for c in cs[1:-1]:
        t = np.multiply.outer(t, c)
    if len(cs) == 1:
        return t.real.copy()
    last = cs[-1]
    return np.multiply.outer(t.real, last.real) - np.multiply.outer(t.imag, last.imag)


def _separable_char(kind, h, pos, N, Y):
    """Characteristic function of a box ('cube') or bilinear pyramid on grid N
    from its separable spectrum: per axis the phase of get_shift_inclusion
    (integer frequencies in FFT order, as the reference pairs them) times the
    centred 1D weight of get_weights_con / get_weights_lin; 1/|Y| once.
    Equals _centered_ifft_real(SS * W, N) up to roundoff."""
    N = np.asarray(N, dtype=np.int64)
    Zr = Grid.get_ZNl(N)
    Zc = Grid.get_ZNl(N, fft_form='c')
    vecs = []
    for i in range(N.size):
        if kind == 'cube':
            w = h[i] * np.sinc(h[i] * Zc[i] / Y[i])
        else:
            w = h[i] * np.sinc(h[i] * Zc[i] / Y[i]) ** 2
        ph = np.ones(N[i], dtype=np.complex128) if pos is None else \
            np.exp(-2j * np.pi * pos[i] * Zr[i] / Y[i])
        vecs.append(ph * w)
    vecs[0] = vecs[0] / np.prod(Y)
    return _centered_ifft_real_separable(vecs, N)


def get_shift_inclusion(N, h, Y):
    """Phase factor of an inclusion at position h (materials.py:317-330)."""
    N = np.asarray(N, dtype=np.int64)
    Z = Grid.get_ZNl(N)
    return _outer_axes(N, [np.exp(-2j * np.pi * h[i] * Z[i] / Y[i])
                           for i in range(N.size)]).astype(np.complex128)


def get_inverse(A):
    """Per-voxel inverse of (d, d) + N values, Gauss-Jordan without pivoting
    (ffthompy/trigpol.py:120-159), vectorised over the grid."""
    d = A.shape[0]
    B = np.array(A, dtype=np.float64, copy=True)
    inv = np.zeros_like(B)
    for m in range(d):
        inv[m, m] = 1.
    for m in range(d):
        piv = B[m, m].copy()
        B[m, m] = 1.
        B[m, m + 1:] = B[m, m + 1:] / piv
        inv[m] = inv[m] / piv
        for k in range(m + 1, d):
            f = B[k, m].copy()
            B[k] = B[k] - B[m] * f
            inv[k] = inv[k] - inv[m] * f
    for m in range(d - 1, -1, -1):
        for k in range(m - 1, -1, -1):
            f = B[k, m].copy()
            B[k] = B[k] - B[m] * f
            inv[k] = inv[k] - inv[m] * f
    return inv


def ga_axis_tables(P, Nbar, h, Y, order, target=None):
    """Per-axis source indices and weights of the grid-based Ga coefficient.

    For target frequency q of the Nbar grid (FFT order), src gives the FFT-order
    index of the P-grid DFT coefficient that the reference's tile + central
    crop of the centred spectrum places there (materials.py:94-106), and w the
    1D cell-shape weight h sinc(h q / Y) (order 0) or h sinc^2 (order 1)
    (materials.py:333-389).  The 1/|Y| factor is folded into axis 0.
    target (>= Nbar, odd Nbar) re-indexes the tables onto a larger grid with
    zero weight outside the Nbar band: the same trigonometric polynomial.
    """
    P = np.asarray(P, dtype=np.int64)
    Nbar = np.asarray(Nbar, dtype=np.int64)
    if np.all(P == Nbar):
        mode = 'same'
    elif np.all(P >= Nbar):
        mode = 'crop'
    elif np.all(P < Nbar):
        mode = 'tile'
    else:
        raise NotImplementedError('This combination of double N (%s) and P (%s)' % (Nbar, P))
    srcs, ws = [], []
    for i in range(Nbar.size):
        p_, n_ = int(P[i]), int(Nbar[i])
        cidx = np.arange(p_)
        if mode == 'same':
            sel = cidx
        elif mode == 'crop':
            sel = decrease(cidx, [n_])
        else:
            f = int(np.ceil(n_ / 2. / p_))
            sel = decrease(np.tile(cidx, 2 * f + 1), [n_])
        tpos = (np.arange(n_) - n_ // 2) % n_
        src = np.empty(n_, dtype=np.int32)
        src[tpos] = (sel - p_ // 2) % p_
        Z = Grid.get_ZNl([n_], fft_form='c')[0]
        wc = h[i] * np.sinc(h[i] * Z / Y[i])
        if order in (1, 'bilinear'):
            wc = h[i] * np.sinc(h[i] * Z / Y[i]) ** 2
        w = np.empty(n_)
        w[tpos] = wc
        srcs.append(src)
        ws.append(w)
    ws[0] = ws[0] / np.prod(Y)
    if target is not None:
        target = np.asarray(target, dtype=np.int64)
        for i in range(Nbar.size):
            n_, t_ = int(Nbar[i]), int(target[i])
            hb = (n_ - 1) // 2
            q = np.fft.fftfreq(t_, 1. / t_).astype(np.int64)
            inb = np.abs(q) <= hb
            s2 = np.zeros(t_, dtype=np.int32)
            w2 = np.zeros(t_)
            s2[inb] = srcs[i][q[inb] % n_]
            w2[inb] = ws[i][q[inb] % n_]
            srcs[i], ws[i] = s2, w2
    return np.concatenate(srcs).astype(np.int32), np.concatenate(ws)


def _ball_char_gpu(r, pos, N, Y):
    """get_shape_functions' ball characteristic function on the GPU
    (fhp_ball_characteristic), centred like _centered_ifft_real(SS * W, N).
    The tables pair what the reference pairs position by position: the
    weight of centred frequency i - N/2 (get_weights_circ, materials.py:
    392-425) with the phase of get_shift_inclusion at the same array position,
    whose frequencies are in FFT order (materials.py:317-330)."""
    from .engine import ball_characteristic
    N = np.asarray(N, dtype=np.int64)
    Y = np.asarray(Y, dtype=np.float64)
    h = np.asarray(pos, dtype=np.float64)
    Zc = Grid.get_ZNl(N, fft_form='c')
    Zf = Grid.get_ZNl(N)
    sq = [(Zc[i] / Y[i]) ** 2 for i in range(N.size)]
    ph = [np.exp(-2j * np.pi * h[i] * Zf[i] / Y[i]) for i in range(N.size)]
    out = ball_characteristic(N, r, float(np.prod(Y)), sq, ph)
    return np.fft.fftshift(out.cpu().numpy())


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def ga_grid_coefficient_gpu(vals, P, Nbar, Y, order, target=None):
    """Grid-based Ga coefficient on the GPU (fhp_ga_grid_coefficient).

    vals: (dv, dv) + P nodal values, a NumPy array with the centred origin or a
    CUDA tensor with origin 0 (as coefficient_inverse(..., shift=True) returns
    it).  Distinct component fields are transformed once; returns a torch
    tensor (dv, dv) + grid, origin 0, grid = Nbar or the larger target grid
    (same trigonometric polynomial).
    """
    grid = Nbar if target is None else np.asarray(target, dtype=np.int64)
    import ctypes
    import torch
    from . import _lib
    lib = _lib.load()
    dv = vals.shape[0]
    d = len(P)
    on_device = not isinstance(vals, np.ndarray)
    same = torch.equal if on_device else np.array_equal
    comps, where = [], {}
    for m in range(dv):
        for n in range(dv):
            v = vals[m, n]
            if not bool(v.any()):
                continue
            for k, c in enumerate(comps):
                if same(c, v):
                    where[(m, n)] = k
                    break
            else:
                where[(m, n)] = len(comps)
                comps.append(v)
    out = torch.zeros((dv, dv) + tuple(int(n) for n in grid), dtype=torch.float64, device='cuda')
    if not comps:
        return out
    src, w = ga_axis_tables(P, Nbar, np.asarray(Y, dtype=np.float64) / np.asarray(P), Y, order,
                            target=target)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k0 in range(0, len(comps), 6):
        chunk = comps[k0:k0 + 6]
        if on_device:
            dimg = torch.stack(chunk).contiguous()
        else:
            img = np.stack([np.fft.ifftshift(c) for c in chunk])
            dimg = torch.from_numpy(np.ascontiguousarray(img)).to('cuda')
        dout = torch.empty((len(chunk),) + tuple(int(n) for n in grid), dtype=torch.float64,
                           device='cuda')
        hp, ho = ctypes.c_void_p(), ctypes.c_void_p()
        np_ = (ctypes.c_int * d)(*[int(x) for x in P])
        no_ = (ctypes.c_int * d)(*[int(x) for x in grid])
        _lib.check(lib.fhp_fft_plan_create(ctypes.byref(hp), d, np_, len(chunk), _lib.FHP_F64),
                   'fhp_fft_plan_create')
        try:
            _lib.check(lib.fhp_fft_plan_create(ctypes.byref(ho), d, no_, len(chunk),
                                               _lib.FHP_F64), 'fhp_fft_plan_create')
            try:
                _lib.check(lib.fhp_ga_grid_coefficient(
                    hp, ho, ctypes.c_void_p(dimg.data_ptr()),
                    src.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                    w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                    ctypes.c_void_p(dout.data_ptr()), stream), 'fhp_ga_grid_coefficient')
            finally:
                lib.fhp_plan_destroy(ho)
        finally:
            lib.fhp_plan_destroy(hp)
        for (m, n), k in where.items():
            if k0 <= k < k0 + len(chunk):
                out[m, n] = dout[k - k0]
    return out


class Material:
    def __init__(self, material_conf):
        self.conf = material_conf
        if 'Y' not in self.conf:
            raise ValueError('The definition of PUC size (Y) is missing!')
        self.Y = np.asarray(material_conf['Y'], dtype=np.float64)
        if 'fun' in self.conf:
            return
        if 'inclusions' not in self.conf:
            raise NotImplementedError('Improper material definition!')
        n_incl = len(self.conf['inclusions'])
        for key in ('inclusions', 'positions', 'params', 'vals'):
            if key in self.conf and len(self.conf[key]) != n_incl:
                raise ValueError('Improper no. of values in material for (%s)!' % key)
        for ii, incl in enumerate(self.conf['inclusions']):
            if incl in ('all', 'otherwise'):
                continue
            param = self.conf['params'][ii]
            if np.any(np.greater(param, self.Y)):
                raise ValueError('Improper parameters of inclusion!')
            self.conf['positions'][ii] = np.asarray(self.conf['positions'][ii]) % self.Y

    # -- nodal evaluation -------------------------------------------------------
    def get_topologies(self, coord):
        """Characteristic functions at the nodes, summed over the 3^d periodic
        images of each inclusion (materials.py:212-301).  coord are the
        tensor-product nodes of Grid.get_coordinates."""
        incs = self.conf['inclusions']
        params, poss = self.conf['params'], self.conf['positions']
        d = coord.shape[0]
        grid = coord.shape[1:]
        images = list(itertools.product((-1, 0, 1), repeat=d))
        # boxes and pyramids are products over the axes, so their sum over the
        # 3^d periodic images is the product of per-axis sums over 3 images
        axes = [coord[a][(0,) * a + (slice(None),) + (0,) * (d - a - 1)] for a in range(d)]

        def outer(vs):
            t = vs[0]
            for v in vs[1:]:
                t = np.multiply.outer(t, v)
            return t.reshape(grid)
        topos = []
        for ii, kind in enumerate(incs):
            if kind in inclusion_keys['cube']:
                p = np.asarray(params[ii], dtype=np.float64)
                x0 = np.asarray(poss[ii], dtype=np.float64)
                vs = []
                for a in range(d):
                    va = np.zeros(grid[a])
                    for im in (-1, 0, 1):
                        u = axes[a] - x0[a] + self.Y[a] * im
                        va += (u > -p[a] / 2) & (u <= p[a] / 2)
                    vs.append(va)
                t = outer(vs)
            elif kind in inclusion_keys['ball'] and _gpu_available() and d in (2, 3):
                from .engine import ball_topology
                t = ball_topology(axes, np.asarray(poss[ii], dtype=np.float64), self.Y,
                                  params[ii] / 2).cpu().numpy()
            elif kind in inclusion_keys['ball']:
                x0 = np.asarray(poss[ii], dtype=np.float64)
                t = np.zeros(grid)
                for im in images:
                    r2 = np.zeros(grid)
                    for a in range(d):
                        r2 += (coord[a] - x0[a] - self.Y[a] * im[a]) ** 2
                    t += np.sqrt(r2) < params[ii] / 2
            elif kind in inclusion_keys['pyramid']:
                p = np.asarray(params[ii], dtype=np.float64)
                x0 = np.asarray(poss[ii], dtype=np.float64)
                vs = []
                for a in range(d):  # the reference shifts pyramids by 2*Y per image
                    va = np.zeros(grid[a])
                    for im in (-1, 0, 1):
                        u = axes[a] - x0[a] + 2 * self.Y[a] * im
                        va += np.maximum(1 - np.abs(u) / (p[a] / 2.), 0.)
                    vs.append(va)
                t = outer(vs)
            elif kind == 'otherwise':
                t = np.ones(grid) - sum(topos) if topos else np.ones(grid)
                if not (t >= 0).all():
                    raise NotImplementedError('Overlapping inclusions!')
            elif kind == 'all':
                t = np.ones(grid)
            else:
                raise NotImplementedError('Inclusion (%s) is not implemented.' % kind)
            topos.append(t)
        return topos

    def evaluate(self, coord):
        """Coefficient values (d_v, d_v) + grid at the nodes, centred origin."""
        if 'fun' in self.conf:
            return np.asarray(self.conf['fun'](coord), dtype=np.float64)
        vals = self.conf['vals']
        A = np.zeros(np.shape(vals[0]) + coord.shape[1:])
        for v, t in zip(vals, self.get_topologies(coord)):
            A += np.multiply.outer(np.asarray(v, dtype=np.float64), t)
        return A

    @staticmethod
    def _origin0(val, name):
        val = np.fft.ifftshift(val, axes=tuple(range(2, val.ndim)))
        return Tensor(name=name, val=val, order=2, multype=21, origin=0)

    def get_A_GaNi(self, N, primaldual='primal'):
        A = self.evaluate(Grid.get_coordinates(N, self.Y))
        name = 'A_GaNi'
        if primaldual == 'dual':
            name = 'inv(A_GaNi)'
            if _gpu_available():
                from .engine import coefficient_inverse
                out = Tensor(name=name, val=coefficient_inverse(A, shift=True), order=2,
                             multype=21, origin=0)
                out.Y = self.Y
                return out
            A = get_inverse(A)
        out = self._origin0(A, name)
        out.Y = self.Y
        return out

    def get_shape_functions(self, N2):
        N2 = np.asarray(N2, dtype=np.int64)
        incs = self.conf['inclusions']
        params, poss = self.conf['params'], self.conf['positions']
        chars = []
        SS = None
        shift_pos = None   # the phase of the last inclusion with a position (as SS)
        for ii, incl in enumerate(incs):
            if isinstance(poss[ii], np.ndarray):
                shift_pos = np.asarray(poss[ii], dtype=np.float64)
                SS = None
            if incl in inclusion_keys['cube']:
                # separable spectrum: 1D transforms and an outer product
                chars.append(_separable_char('cube', np.asarray(params[ii], dtype=np.float64),
                                             shift_pos, N2, self.Y))
            elif incl in inclusion_keys['ball']:
                r = params[ii] / 2
                if r != 0 and _gpu_available() and np.all(N2 % 2 == 1) and N2.size in (2, 3):
                    chars.append(_ball_char_gpu(r, shift_pos, N2, self.Y))
                    continue
                if SS is None:
                    SS = get_shift_inclusion(N2, shift_pos, self.Y)
                W = np.zeros(tuple(N2)) if r == 0 else get_weights_circ(r, N2, self.Y)
                chars.append(_centered_ifft_real(SS * W, N2))
            elif incl in inclusion_keys['pyramid']:
                chars.append(_separable_char('pyramid', np.asarray(params[ii], dtype=np.float64) / 2.,
                                             shift_pos, N2, self.Y))
            elif incl == 'all':
                chars.append(np.ones(tuple(N2)))
            elif incl == 'otherwise':
                chars.append(np.ones(tuple(N2)) - sum(chars) if chars else np.ones(tuple(N2)))
            else:
                raise NotImplementedError('The inclusion (%s) is not supported!' % incl)
        return chars

    def _get_A_Ga_on(self, Nbar, primaldual, order, P, grid):
        grid = tuple(int(g) for g in grid)
        if order == -1:
            order = self.conf.get('order', -1)
        if order in (0, 1, 'constant', 'bilinear') and _gpu_available() and \
                np.all(Nbar % 2 == 1):
            if P is None and 'P' in self.conf:
                P = self.conf['P']
            P = np.asarray(P, dtype=np.int64)
            vals = self.evaluate(Grid.get_coordinates(P, self.Y))
            if primaldual == 'dual':
                from .engine import coefficient_inverse
                vals = coefficient_inverse(vals, shift=True)
            out = Tensor(name='A_Ga_o{0}_P{1}'.format(order, np.array(P).max()),
                         val=ga_grid_coefficient_gpu(vals, P, Nbar, self.Y, order, target=grid),
                         order=2, multype=21, origin=0)
            out.Y = self.Y
            return out
        from .engine import interpolate_fields
        A = self.get_A_Ga(Nbar, primaldual, order=order, P=P)
        out = A.copy(val=interpolate_fields(A.data, tuple(int(n) for n in Nbar), grid))
        out.Y = self.Y
        return out

    def get_A_Ga(self, Nbar, primaldual='primal', order=-1, P=None, grid=None):
        """grid (optional, >= Nbar): return the same coefficient (the same
        trigonometric polynomial) sampled on a larger integration grid."""
        Nbar = np.asarray(Nbar, dtype=np.int64)
        if grid is not None and tuple(int(g) for g in grid) != tuple(Nbar):
            return self._get_A_Ga_on(Nbar, primaldual, order, P, grid)
        if order == -1:
            if 'order' not in self.conf:
                raise ValueError('The material order is undefined!')
            order = self.conf['order']
        elif order not in (None, 'exact', 0, 1):
            raise ValueError('Wrong material order (%s)!' % str(order))
        if order in (None, 'exact'):
            chars = self.get_shape_functions(Nbar)
            vals = self.conf['vals']
            if _gpu_available():
                # each characteristic function moved to origin 0 and uploaded
                # once; the sum over inclusions runs on the GPU
                # (fhp_outer_accumulate), bit-identical to the host sum
                import torch
                from .engine import outer_accumulate
                shape = tuple(np.shape(vals[0]))
                val_d = torch.zeros(shape + tuple(int(n) for n in Nbar), dtype=torch.float64,
                                    device='cuda')
                flat = val_d.view(int(np.prod(shape)), -1)
                for v, c in zip(vals, chars):
                    v = np.asarray(v, dtype=np.float64)
                    if primaldual == 'dual':
                        v = np.linalg.inv(v)
                    c0 = torch.from_numpy(np.ascontiguousarray(np.fft.ifftshift(c))).to('cuda')
                    outer_accumulate(flat, v, c0)
                out = Tensor(name='A_Ga', val=val_d, order=2, multype=21, origin=0)
                out.Y = self.Y
                return out
            val = np.zeros(np.shape(vals[0]) + tuple(Nbar))
            for v, c in zip(vals, chars):
                v = np.asarray(v, dtype=np.float64)
                if primaldual == 'dual':
                    v = np.linalg.inv(v)
                val += np.multiply.outer(v, c)
            name = 'A_Ga'
        else:
            if P is None and 'P' in self.conf:
                P = self.conf['P']
            P = np.asarray(P, dtype=np.int64)
            vals = self.evaluate(Grid.get_coordinates(P, self.Y))
            name = 'A_Ga_o{0}_P{1}'.format(order, np.array(P).max())
            if _gpu_available() and np.all(Nbar % 2 == 1) and Nbar.size == P.size:
                if primaldual == 'dual':
                    from .engine import coefficient_inverse
                    vals = coefficient_inverse(vals, shift=True)
                out = Tensor(name=name, val=ga_grid_coefficient_gpu(vals, P, Nbar, self.Y, order),
                             order=2, multype=21, origin=0)
                out.Y = self.Y
                return out
            if primaldual == 'dual':
                vals = get_inverse(vals)
            h = self.Y / P
            W = get_weights_con(h, Nbar, self.Y) if order in (0, 'constant') \
                else get_weights_lin(h, Nbar, self.Y)
            val = np.zeros(vals.shape[:2] + tuple(Nbar))
            for m, n in itertools.product(range(vals.shape[0]), range(vals.shape[1])):
                hA = np.prod(P) * _centered_fft(vals[m, n], P)
                if np.all(P == Nbar):
                    hAN = hA
                elif np.all(P >= Nbar):
                    hAN = decrease(hA, Nbar)
                elif np.all(P < Nbar):
                    reps = 2 * np.ceil(Nbar / 2. / P).astype(np.int64) + 1
                    hAN = decrease(np.tile(hA, reps), Nbar)
                else:
                    raise NotImplementedError('This combination of double N (%s) and P (%s)'
                                              % (Nbar, P))
                val[m, n] = _centered_ifft_real(W * hAN, Nbar)
            name = 'A_Ga_o{0}_P{1}'.format(order, np.array(P).max())
        out = self._origin0(val, name)
        out.Y = self.Y
        return out
