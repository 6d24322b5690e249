"""Tensor of trigonometric-polynomial values, mirroring ffthompy.tensors.Tensor.

Mirrors ffthompy/tensors/objects.py:92-636 for the parts the homogenisation
path uses: construction from (val, order) or (shape, N), value semantics of
+, -, scalar * (objects.py:194-218), the multiplication types 'scal'
(grid-mean inner product, 618-636), 21 ('ij...,j...->i...') and 42,
mean / set_mean / add_mean (263-300), norm (253-261), zeros_like / copy,
inv (per-voxel inverse, 247-251) and shift (169-186).

Values live on the GPU (a torch tensor in .data) when a CUDA device is
present; .val returns a NumPy copy on the host, as the reference's .val is a
NumPy array.  Real-space tensors only: the Fourier-space factors of the
operator are handled inside the CUDA library.
"""
import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _to_device(v, dtype=None):
    if isinstance(v, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(v))
    else:
        t = v
    if torch.cuda.is_available():
        t = t.to('cuda')
    if dtype is not None:
        t = t.to(dtype)
    return t.contiguous()


class Tensor:
    keys = ('name', 'val', 'order', 'Y', 'N', 'multype', 'Fourier', 'fft_form', 'origin')

    def __init__(self, name='', val=None, order=None, shape=None, N=None, Y=None,
                 multype='scal', Fourier=False, fft_form='r', origin=0):
        if Fourier:
            raise NotImplementedError('Fourier-space Tensors are internal to the CUDA '
                                      'library; use real-space Tensors')
        self.name = name
        self.Fourier = False
        self.fft_form = fft_form
        self.origin = origin
        self.multype = multype
        if val is not None:
            self.order = int(order)
            self.data = _to_device(val)
            self.shape = tuple(self.data.shape[:self.order])
            self.N = tuple(int(n) for n in self.data.shape[self.order:])
        elif shape is not None and N is not None:
            self.N = tuple(int(n) for n in np.atleast_1d(N))
            self.shape = tuple(int(s) for s in shape)
            self.order = len(self.shape)
            self.data = _to_device(np.zeros(self.shape + self.N))
        else:
            raise ValueError('Initialization of Tensor.')
        self.dim = len(self.N)
        self.Y = np.ones(self.dim) if Y is None else np.asarray(Y, dtype=np.float64)

    # pickling (Problem.postprocessing saves Tensors, as the reference does,
    # ffthompy/problem.py:98-126): the values travel as a host NumPy array
    # and return to the GPU on loading when one is present
    def __getstate__(self):
        st = {k: v for k, v in self.__dict__.items() if k != 'data'}
        st['val_host'] = self.data.detach().cpu().numpy()
        return st

    def __setstate__(self, st):
        st = dict(st)
        v = st.pop('val_host')
        self.__dict__.update(st)
        self.data = _to_device(v)

    # -- values -----------------------------------------------------------------
    @property
    def val(self):
        return self.data.detach().cpu().numpy()

    @val.setter
    def val(self, v):
        self.data = _to_device(v)

    def pN(self):
        return int(np.prod(self.N))

    @property
    def axes(self):
        return tuple(range(self.order, self.order + self.dim))

    def copy(self, **kw):
        args = dict(name=self.name, order=self.order, Y=self.Y, multype=self.multype,
                    fft_form=self.fft_form, origin=self.origin)
        data = kw.pop('val', None)
        args.update(kw)
        out = Tensor.__new__(Tensor)
        out.name = args['name']
        out.Fourier = False
        out.fft_form = args['fft_form']
        out.origin = args['origin']
        out.multype = args['multype']
        out.order = int(args['order'])
        out.data = self.data.clone() if data is None else _to_device(data)
        out.shape = tuple(out.data.shape[:out.order])
        out.N = tuple(int(n) for n in out.data.shape[out.order:])
        out.dim = len(out.N)
        out.Y = np.asarray(args['Y'], dtype=np.float64)
        return out

    def zeros_like(self, name=None):
        return self.copy(name=name or 'zeros({})'.format(self.name[:10]),
                         val=torch.zeros_like(self.data))

    def empty_like(self, name=None):
        return self.copy(name=name or 'empty({})'.format(self.name[:10]),
                         val=torch.empty_like(self.data))

    # -- arithmetic (value semantics, objects.py:194-218) -------------------------
    def __neg__(self):
        return self.copy(name='-' + self.name[:10], val=-self.data)

    def __add__(self, x):
        if isinstance(x, Tensor):
            assert self.data.shape == x.data.shape
            return self.copy(name='({0}+{1})'.format(self.name[:10], x.name[:10]),
                             val=self.data + x.data)
        if isinstance(x, (np.ndarray, float, int)):
            return self.copy(val=self.data + _to_device(np.asarray(x), self.data.dtype))
        raise ValueError('Tensor.__add__')

    def __sub__(self, x):
        return self.__add__(-x)

    def __rmul__(self, x):
        if np.size(x) == 1:
            return self.copy(val=float(x) * self.data)
        raise ValueError()

    def __call__(self, *args, **kwargs):
        return self.__mul__(*args, **kwargs)

    def __mul__(self, Y, multype=None):
        multype = self.multype if multype is None else multype
        if not isinstance(Y, Tensor):
            return float(Y) * self
        if multype in ('scal', 'scalar'):
            return scalar_product(self, Y)
        if multype in (21, '21'):
            return einsum('ij...,j...->i...', self, Y)
        if multype in (42, '42'):
            return einsum('ijkl...,kl...->ij...', self, Y)
        if multype in (0, 'elementwise', 'hadamard'):
            return einsum('...,...->...', self, Y)
        return einsum(multype, self, Y)

    # -- means (objects.py:263-300) ---------------------------------------------
    def mean(self):
        m = self.data.reshape(self.shape + (-1,)).mean(dim=-1)
        return m.detach().cpu().numpy().astype(np.float64)

    def add_mean(self, mean):
        mean = np.asarray(mean, dtype=np.float64)
        assert self.shape == mean.shape
        self.data = self.data + _to_device(mean, self.data.dtype).reshape(
            self.shape + (1,) * self.dim)
        return self

    def set_mean(self, mean):
        mean = np.asarray(mean, dtype=np.float64)
        assert self.shape == mean.shape
        self.add_mean(-self.mean())
        return self.add_mean(mean)

    def norm(self, ntype='L2', componentwise=False):
        if componentwise:
            out = np.empty(self.shape)
            for ind in np.ndindex(*self.shape):
                t = Tensor(name='aux', val=self.data[ind], order=0)
                out[ind] = t.norm(ntype)
            return out
        if ntype in ('L2', 2):
            return scalar_product(self, self) ** 0.5
        if ntype == 1:
            return float(self.data.abs().sum())
        if ntype == 'inf':
            return float(self.data.abs().max())
        raise NotImplementedError('This type ({}) of norm is not implemented!'.format(ntype))

    def inv(self):
        """Per-voxel matrix inverse (objects.py:247-251): the reference's
        Gauss-Jordan elimination (trigpol.py:120-159) in the CUDA library."""
        assert self.order == 2 and self.shape[0] == self.shape[1]
        from ..engine import coefficient_inverse
        return self.copy(name='inv({})'.format(self.name), val=coefficient_inverse(self.data))

    def shift(self, origin=None):
        """Move the origin between centred ('c') and 0 (objects.py:169-186)."""
        if origin == self.origin:
            return self
        if origin is not None:
            raise ValueError()
        if self.origin in (0,):
            self.data = torch.fft.fftshift(self.data, dim=self.axes)
            self.origin = 'c'
        else:
            self.data = torch.fft.ifftshift(self.data, dim=self.axes)
            self.origin = 0
        return self

    def __eq__(self, Y, full=True, tol=1e-13):
        ok = isinstance(Y, Tensor) and tuple(self.data.squeeze().shape) == tuple(Y.data.squeeze().shape)
        res = float((self.data.squeeze() - Y.data.squeeze()).norm()) if ok else np.inf
        b = res < tol
        return (b, res) if full else b

    __hash__ = object.__hash__

    def __repr__(self):
        return 'Class : Tensor\n    name = {}\n    shape = {}\n    N = {}\n    origin = {}\n'.format(
            self.name, self.shape, self.N, self.origin)


def einsum(op, x, y):
    assert tuple(x.N) == tuple(y.N)
    val = torch.einsum(op, x.data, y.data)
    order = val.dim() - len(x.N)
    return y.copy(name='{0}({1})'.format(x.name, y.name), val=val, order=order)


def scalar_product(y, x):
    """sum(y*x)/prod(N) in FP64 (objects.py:618-636, real-space branch)."""
    assert isinstance(x, Tensor) and tuple(y.data.shape) == tuple(x.data.shape)
    return float((y.data.double() * x.data.double()).sum()) / float(np.prod(y.N))
