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

Coefficient assembly runs once per problem, on the GPU (it needs CUDA, as
the solve does; there is no host fallback).  Topologies and characteristic
functions are built at origin 0 on the device: boxes and pyramids from
their per-axis factors (fhp_separable_char; the per-axis factors are 1D
sums and 1D transforms formed on the host), balls by fhp_ball_topology /
fhp_ball_characteristic; sums over inclusions (fhp_outer_accumulate), the
dual inverse (fhp_coefficient_inverse) and the grid-based Ga coefficient
(fhp_ga_grid_coefficient) run in the CUDA library.  Results are
bit-identical to the NumPy evaluation of the reference's expressions except
the transforms (ball characteristic functions, grid-based Ga), which agree to
roundoff.  A 'fun' material's values come from the user's host function and
are uploaded.  The result is a Tensor with origin 0 on the GPU.
"""
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


def _separable_axis_values(kind, h, pos, N, Y):
    """Per-axis factors of the characteristic function of a box ('cube') or
    bilinear pyramid on grid N (centred order, complex): per axis the phase
    of get_shift_inclusion (integer frequencies in FFT order, as the
    reference pairs them) times the centred 1D weight of get_weights_con /
    get_weights_lin, 1/|Y| on axis 0, transformed by the centred 1D inverse
    DFT.  The d-dimensional function is the real part of their product
    (the transform of a separable spectrum is the product of the 1D
    transforms), as the reference's centred inverse DFT of SS * W forms it."""
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
    return [np.fft.fftshift(np.fft.ifft(np.fft.ifftshift(X))) * int(n)
            for X, n in zip(vecs, N)]


def _separable_dev(N, vecs):
    """Product of per-axis factors on the GPU (fhp_separable_char), origin 0:
    real tables give prod_a v_a[x_a], complex ones the real part of the
    product, each as NumPy's outer products round them."""
    from .engine import separable_char
    N = np.asarray(N, dtype=np.int64)
    if N.size not in (2, 3):
        raise NotImplementedError('grids of 2 or 3 dimensions')
    vecs = [np.asarray(v)[_o0(n)] for v, n in zip(vecs, N)]
    if np.iscomplexobj(vecs[0]):
        return separable_char(N, [v.real for v in vecs], [v.imag for v in vecs])
    return separable_char(N, vecs, None)


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


def _o0(n):
    """Gather indices of np.fft.ifftshift on an axis of n points: the
    origin-0 array's entry j is the centred array's entry _o0(n)[j]."""
    return np.fft.ifftshift(np.arange(int(n)))


def _ball_char_dev(r, pos, N, Y):
    """Ga characteristic function of a ball on the GPU
    (fhp_ball_characteristic), origin 0.  The tables pair what the reference
    pairs position by position: the weight of centred frequency i - N/2
    (get_weights_circ, materials.py:392-425) with the phase of
    get_shift_inclusion at the same array position, whose frequencies are in
    FFT order (materials.py:317-330)."""
    from .engine import ball_characteristic
    N = np.asarray(N, dtype=np.int64)
    Y = np.asarray(Y, dtype=np.float64)
    h = np.asarray(pos, dtype=np.float64)
    Zc = Grid.get_ZNl(N, fft_form='c')
    Zf = Grid.get_ZNl(N)
    sq = [(Zc[i] / Y[i]) ** 2 for i in range(N.size)]
    ph = [np.exp(-2j * np.pi * h[i] * Zf[i] / Y[i]) for i in range(N.size)]
    return ball_characteristic(N, r, float(np.prod(Y)), sq, ph)


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
    @staticmethod
    def _grid_axes(coord):
        """Per-axis node coordinates of tensor-product nodes (Grid.get_coordinates)."""
        d = coord.shape[0]
        return [np.asarray(coord[a][(0,) * a + (slice(None),) + (0,) * (d - a - 1)],
                           dtype=np.float64) for a in range(d)]

    def _topologies_dev(self, axes, origin0=True):
        """Characteristic functions at the nodes (per-axis coordinates axes,
        centred order), summed over the 3^d periodic images of each inclusion
        (materials.py:212-301), on the GPU; origin0 returns them ifftshift-ed.
        Boxes and pyramids are products over the axes, so their sum over the
        images is the product of per-axis sums over 3 images."""
        import torch
        from .engine import ball_topology, outer_accumulate, require_cuda
        require_cuda()
        incs = self.conf['inclusions']
        params, poss = self.conf['params'], self.conf['positions']
        d = len(axes)
        grid = tuple(len(a) for a in axes)
        perm = [_o0(n) if origin0 else np.arange(n) for n in grid]
        topos = []
        for ii, kind in enumerate(incs):
            if kind in inclusion_keys['cube'] or kind in inclusion_keys['pyramid']:
                p = np.asarray(params[ii], dtype=np.float64)
                x0 = np.asarray(poss[ii], dtype=np.float64)
                cube = kind in inclusion_keys['cube']
                vs = []
                for a in range(d):
                    va = np.zeros(grid[a])
                    for im in (-1, 0, 1):
                        if cube:
                            u = axes[a] - x0[a] + self.Y[a] * im
                            va += (u > -p[a] / 2) & (u <= p[a] / 2)
                        else:  # the reference shifts pyramids by 2*Y per image
                            u = axes[a] - x0[a] + 2 * self.Y[a] * im
                            va += np.maximum(1 - np.abs(u) / (p[a] / 2.), 0.)
                    vs.append(va[perm[a]])
                from .engine import separable_char
                t = separable_char(grid, vs, None)
            elif kind in inclusion_keys['ball']:
                t = ball_topology([ax[pm] for ax, pm in zip(axes, perm)],
                                  np.asarray(poss[ii], dtype=np.float64), self.Y, params[ii] / 2)
            elif kind == 'otherwise':
                # np.ones(grid) - sum(topos), with Python's left-to-right sum
                t = torch.ones(grid, dtype=torch.float64, device='cuda')
                if topos:
                    acc = torch.zeros(grid, dtype=torch.float64, device='cuda')
                    for prev in topos:
                        outer_accumulate(acc.view(1, -1), [1.], prev)
                    outer_accumulate(t.view(1, -1), [-1.], acc)
                if bool((t < 0).any()):
                    raise NotImplementedError('Overlapping inclusions!')
            elif kind == 'all':
                t = torch.ones(grid, dtype=torch.float64, device='cuda')
            else:
                raise NotImplementedError('Inclusion (%s) is not implemented.' % kind)
            topos.append(t.contiguous())
        return topos

    def _nodal_dev(self, axes, origin0=True):
        """Nodal coefficient (d_v, d_v) + grid of an inclusion material on the
        GPU: sum over inclusions of vals (x) topology, as evaluate."""
        import torch
        from .engine import outer_accumulate
        vals = self.conf['vals']
        shape = tuple(np.shape(vals[0]))
        grid = tuple(len(a) for a in axes)
        A = torch.zeros(shape + grid, dtype=torch.float64, device='cuda')
        flat = A.view(int(np.prod(shape)), -1)
        for v, t in zip(vals, self._topologies_dev(axes, origin0)):
            outer_accumulate(flat, np.asarray(v, dtype=np.float64), t)
        return A

    def get_topologies(self, coord):
        """Characteristic functions at the nodes coord (tensor-product nodes of
        Grid.get_coordinates), centred, as host arrays (materials.py:212-301);
        computed on the GPU."""
        return [t.cpu().numpy() for t in self._topologies_dev(self._grid_axes(coord), False)]

    def evaluate(self, coord):
        """Coefficient values (d_v, d_v) + grid at the nodes, centred origin
        (host array; inclusion materials are evaluated on the GPU)."""
        if 'fun' in self.conf:
            return np.asarray(self.conf['fun'](coord), dtype=np.float64)
        return self._nodal_dev(self._grid_axes(coord), False).cpu().numpy()

    def _nodal_origin0(self, N):
        """Nodal values on grid N with origin 0 as a CUDA tensor, and whether
        they are already shifted (inclusions: built shifted on the GPU; 'fun':
        the user's host values, centred)."""
        if 'fun' in self.conf:
            return self.evaluate(Grid.get_coordinates(N, self.Y)), False
        return self._nodal_dev(Grid.get_axes(N, self.Y), True), True

    @staticmethod
    def _origin0(val, name):
        val = np.fft.ifftshift(val, axes=tuple(range(2, val.ndim)))
        return Tensor(name=name, val=val, order=2, multype=21, origin=0)

    def get_A_GaNi(self, N, primaldual='primal'):
        from .engine import coefficient_inverse, require_cuda
        require_cuda()
        N = np.asarray(N, dtype=np.int64)
        A, shifted = self._nodal_origin0(N)
        name = 'A_GaNi'
        if primaldual == 'dual':
            name = 'inv(A_GaNi)'
            out = Tensor(name=name, val=coefficient_inverse(A, shift=not shifted), order=2,
                         multype=21, origin=0)
        elif shifted:
            out = Tensor(name=name, val=A, order=2, multype=21, origin=0)
        else:
            out = self._origin0(A, name)
        out.Y = self.Y
        return out

    def _shape_functions_dev(self, N2, origin0=True):
        """Ga characteristic functions of the inclusions on grid N2
        (materials.py:125-169) as CUDA tensors (origin 0, or centred)."""
        import torch
        from .engine import outer_accumulate, require_cuda
        require_cuda()
        N2 = np.asarray(N2, dtype=np.int64)
        incs = self.conf['inclusions']
        params, poss = self.conf['params'], self.conf['positions']
        grid = tuple(int(n) for n in N2)
        chars = []
        shift_pos = None   # the position of the last inclusion that has one
        for ii, incl in enumerate(incs):
            if isinstance(poss[ii], np.ndarray):
                shift_pos = np.asarray(poss[ii], dtype=np.float64)
            if incl in inclusion_keys['cube'] or incl in inclusion_keys['pyramid']:
                cube = incl in inclusion_keys['cube']
                h = np.asarray(params[ii], dtype=np.float64) / (1. if cube else 2.)
                vecs = _separable_axis_values('cube' if cube else 'pyramid', h, shift_pos, N2,
                                              self.Y)
                c = _separable_dev(N2, vecs)
            elif incl in inclusion_keys['ball']:
                r = params[ii] / 2
                if r == 0:
                    c = torch.zeros(grid, dtype=torch.float64, device='cuda')
                elif np.all(N2 % 2 == 1) and N2.size in (2, 3):
                    c = _ball_char_dev(r, shift_pos, N2, self.Y)
                else:
                    raise NotImplementedError('ball inclusions need an odd grid of 2 or 3 '
                                              'dimensions (exact integration grids 2N-1 are)')
            elif incl == 'all':
                c = torch.ones(grid, dtype=torch.float64, device='cuda')
            elif incl == 'otherwise':
                c = torch.ones(grid, dtype=torch.float64, device='cuda')
                if chars:
                    acc = torch.zeros(grid, dtype=torch.float64, device='cuda')
                    for prev in chars:
                        outer_accumulate(acc.view(1, -1), [1.], prev)
                    outer_accumulate(c.view(1, -1), [-1.], acc)
            else:
                raise NotImplementedError('The inclusion (%s) is not supported!' % incl)
            chars.append(c.contiguous())
        if not origin0:
            # the centred order of the public get_shape_functions
            chars = [torch.fft.fftshift(c) for c in chars]
        return chars

    def get_shape_functions(self, N2):
        """Characteristic functions on grid N2, centred (host arrays), as the
        reference returns them (materials.py:125-169); computed on the GPU."""
        return [c.cpu().numpy() for c in self._shape_functions_dev(N2, origin0=False)]

    def _get_A_Ga_on(self, Nbar, primaldual, order, P, grid):
        grid = tuple(int(g) for g in grid)
        if order == -1:
            order = self.conf.get('order', -1)
        if order in (0, 1, 'constant', 'bilinear') and np.all(Nbar % 2 == 1):
            if P is None and 'P' in self.conf:
                P = self.conf['P']
            P = np.asarray(P, dtype=np.int64)
            vals = self._grid_image(P, primaldual)
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

    def _grid_image(self, P, primaldual):
        """The P-voxel image of a grid-based Ga coefficient for
        ga_grid_coefficient_gpu: origin-0 CUDA values (inverted per voxel for
        the dual), or the centred host values of a 'fun' material's primal."""
        from .engine import coefficient_inverse
        vals, shifted = self._nodal_origin0(P)
        if primaldual == 'dual':
            return coefficient_inverse(vals, shift=not shifted)
        return vals

    def get_A_Ga(self, Nbar, primaldual='primal', order=-1, P=None, grid=None):
        """grid (optional, >= Nbar): return the same coefficient (the same
        trigonometric polynomial) sampled on a larger integration grid."""
        from .engine import require_cuda
        require_cuda()
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
            # each characteristic function at origin 0 on the GPU; the sum over
            # inclusions runs there too (fhp_outer_accumulate), bit-identical
            # to the host sum of the same functions
            import torch
            from .engine import outer_accumulate
            chars = self._shape_functions_dev(Nbar)
            vals = self.conf['vals']
            shape = tuple(np.shape(vals[0]))
            val_d = torch.zeros(shape + tuple(int(n) for n in Nbar), dtype=torch.float64,
                                device='cuda')
            flat = val_d.view(int(np.prod(shape)), -1)
            for v, c in zip(vals, chars):
                v = np.asarray(v, dtype=np.float64)
                if primaldual == 'dual':
                    v = np.linalg.inv(v)
                outer_accumulate(flat, v, c)
            out = Tensor(name='A_Ga', val=val_d, order=2, multype=21, origin=0)
            out.Y = self.Y
            return out
        if P is None and 'P' in self.conf:
            P = self.conf['P']
        P = np.asarray(P, dtype=np.int64)
        if not (np.all(Nbar % 2 == 1) and Nbar.size == P.size):
            raise NotImplementedError('grid-based Ga coefficients need an odd double grid '
                                      '(2N-1 is) of the image dimension')
        name = 'A_Ga_o{0}_P{1}'.format(order, np.array(P).max())
        out = Tensor(name=name, val=ga_grid_coefficient_gpu(self._grid_image(P, primaldual), P,
                                                            Nbar, self.Y, order),
                     order=2, multype=21, origin=0)
        out.Y = self.Y
        return out

