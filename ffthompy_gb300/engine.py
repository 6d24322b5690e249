"""Python handle of one C-ABI plan (GPU Fourier-Galerkin operator + CG).

Device memory for fields is allocated with torch (plumbing only); all
arithmetic on the hot path runs in the library's own CUDA kernels.
"""
import collections
import ctypes
import threading

import numpy as np

from . import _lib

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard requirement on GPU hosts
    torch = None


def require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError('ffthompy_gb300 needs a CUDA GPU; no CPU fallback exists')


def coef_kind_of(A):
    """Classify a coefficient array (dv, dv) + grid: ISO, SYM or FULL."""
    dv = A.shape[0]
    off = np.ones((dv, dv), dtype=bool)
    np.fill_diagonal(off, False)
    diag = np.stack([A[i, i] for i in range(dv)])
    if not np.any(A[off]) and np.all(diag == diag[0:1]):
        return _lib.FHP_COEF_ISO
    if all(np.array_equal(A[i, j], A[j, i]) for i in range(dv) for j in range(i + 1, dv)):
        return _lib.FHP_COEF_SYM
    return _lib.FHP_COEF_FULL


def pack_coefficient(A, kind):
    """Component-major float64 values for fhp_set_coefficient."""
    dv = A.shape[0]
    if kind == _lib.FHP_COEF_ISO:
        return np.ascontiguousarray(A[0, 0][None], dtype=np.float64)
    if kind == _lib.FHP_COEF_SYM:
        comps = [A[i, j] for i in range(dv) for j in range(i, dv)]
        return np.ascontiguousarray(np.stack(comps), dtype=np.float64)
    return np.ascontiguousarray(A.reshape((dv * dv,) + A.shape[2:]), dtype=np.float64)


def coef_kind_of_torch(A):
    dv = A.shape[0]
    offdiag = any(bool(A[i, j].any()) for i in range(dv) for j in range(dv) if i != j)
    if not offdiag and all(bool(torch.equal(A[i, i], A[0, 0])) for i in range(1, dv)):
        return _lib.FHP_COEF_ISO
    if all(bool(torch.equal(A[i, j], A[j, i])) for i in range(dv) for j in range(i + 1, dv)):
        return _lib.FHP_COEF_SYM
    return _lib.FHP_COEF_FULL


def pack_coefficient_torch(A, kind):
    dv = A.shape[0]
    if kind == _lib.FHP_COEF_ISO:
        return A[0, 0][None].contiguous()
    if kind == _lib.FHP_COEF_SYM:
        return torch.stack([A[i, j] for i in range(dv) for j in range(i, dv)]).contiguous()
    return A.reshape((dv * dv,) + tuple(A.shape[2:])).contiguous()


def nice_size(n):
    """Smallest m >= n whose prime factors are all in {2, 3, 5, 7}."""
    m = int(n)
    while True:
        r = m
        for p in (2, 3, 5, 7):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


class GalerkinPlan:
    """G o A on one solve grid for a batch of load cases.

    N: solve grid; band: grid whose band carries the Green projection
    (GaNi: band = N; Ga on the full double grid: N = 2*band - 1); scale: Ga
    scale prod(N)/prod(band) by default; physics 'scalar' | 'elasticity';
    precision 'f64' | 'f32' | 'mixed' (FP64 fields, FP32 inner CG with FP64
    iterative refinement).
    integ: band representation of Ga - fields on N, coefficient on the
    integration grid integ >= 2N-1, projection scale prod(2N-1)/prod(N).
    band_cg (band plans): 'spectral' keeps the CG iterates as half spectra of
    N (no transform of the N grid inside an iteration), 'real' as real fields.
    integ_kernel (band plans): 'register' runs the integration pass with
    lines held in registers where that kernel applies (TMA row loads for the
    full band), 'register_cpasync' the same lines with per-lane cp.async
    loads, 'shared' with the shared-memory line cores.
    ncells (GaNi / full-grid Ga): cells of the same grid solved together
    (fhp_plan_create_cells): fields (cells, loads, dv) + N, packed
    coefficients (cells, c) + N, per-load results cell-major, A_H
    (cells, L, L); each load of each cell keeps its own CG state.
    """

    def __init__(self, N, Y, physics='scalar', nloads=None, band=None, scale=None,
                 precision='f64', integ=None, band_cg='spectral', integ_kernel='register',
                 ncells=1):
        require_cuda()
        self.ncells = int(ncells)
        if self.ncells < 1:
            raise ValueError('ncells must be >= 1')
        if self.ncells > 1 and integ is not None:
            raise ValueError('band plans hold one cell')
        self.lib = _lib.load()
        self.N = tuple(int(n) for n in N)
        self.dim = len(self.N)
        self.band = tuple(int(n) for n in (band if band is not None else N))
        self.integ = tuple(int(n) for n in integ) if integ is not None else None
        self.Y = np.asarray(Y, dtype=np.float64)
        self.physics = physics
        self.dv = self.dim if physics == 'scalar' else self.dim * (self.dim + 1) // 2
        self.nloads = int(nloads if nloads is not None else self.dv)
        if scale is None:
            if self.integ is not None:
                scale = float(np.prod([2 * n - 1 for n in self.N], dtype=np.float64)
                              / np.prod(self.N, dtype=np.float64))
            else:
                scale = float(np.prod(self.N, dtype=np.float64)
                              / np.prod(self.band, dtype=np.float64))
        self.scale = float(scale)
        self.precision = precision
        if precision not in ('f64', 'f32', 'mixed'):
            raise ValueError('precision must be f64, f32 or mixed')
        self.dtype = torch.float32 if precision == 'f32' else torch.float64
        self.device = torch.device('cuda', torch.cuda.current_device())
        n = (ctypes.c_int * self.dim)(*self.N)
        nb = (ctypes.c_int * self.dim)(*self.band)
        y = (ctypes.c_double * self.dim)(*self.Y)
        h = ctypes.c_void_p()
        phys = _lib.FHP_SCALAR if physics == 'scalar' else _lib.FHP_ELASTICITY
        prec = {'f64': _lib.FHP_F64, 'f32': _lib.FHP_F32, 'mixed': _lib.FHP_MIXED}[precision]
        if self.integ is not None:
            ni = (ctypes.c_int * self.dim)(*self.integ)
            _lib.check(self.lib.fhp_plan_create_band(ctypes.byref(h), self.dim, n, ni, y, phys,
                                                     self.nloads, self.scale, prec),
                       'fhp_plan_create_band')
        elif self.ncells > 1:
            _lib.check(self.lib.fhp_plan_create_cells(ctypes.byref(h), self.dim, n, nb, y, phys,
                                                      self.nloads, self.scale, prec,
                                                      self.ncells), 'fhp_plan_create_cells')
        else:
            _lib.check(self.lib.fhp_plan_create(ctypes.byref(h), self.dim, n, nb, y, phys,
                                                self.nloads, self.scale, prec),
                       'fhp_plan_create')
        self.handle = h
        self.coef_kind = None
        if band_cg not in ('spectral', 'real'):
            raise ValueError("band_cg must be 'spectral' or 'real'")
        self.band_cg = band_cg
        _lib.check(self.lib.fhp_plan_set_band_cg(h, 1 if band_cg == 'spectral' else 0),
                   'fhp_plan_set_band_cg')
        kinds = {'register': 1, 'register_cpasync': 2, 'shared': 0}
        if integ_kernel not in kinds:
            raise ValueError("integ_kernel must be 'register', 'register_cpasync' or 'shared'")
        self.integ_kernel = integ_kernel
        _lib.check(self.lib.fhp_plan_set_integration_kernel(h, kinds[integ_kernel]),
                   'fhp_plan_set_integration_kernel')

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            self.lib.fhp_plan_destroy(h)
            self.handle = None

    # -- helpers ---------------------------------------------------------------
    @property
    def field_shape(self):
        """(loads, dv) + N; (cells, loads, dv) + N for a plan of several cells."""
        lead = (self.ncells,) if self.ncells > 1 else ()
        return lead + (self.nloads, self.dv) + self.N

    @property
    def _lk(self):
        # per-load results: every load of every cell, cell-major
        return self.nloads * self.ncells

    @property
    def coef_grid(self):
        return self.integ if self.integ is not None else self.N

    def empty(self):
        return torch.empty(self.field_shape, dtype=self.dtype, device=self.device)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _dev(self, x):
        if not isinstance(x, torch.Tensor):
            x = torch.as_tensor(np.asarray(x))
        x = x.to(device=self.device, dtype=self.dtype).contiguous()
        if tuple(x.shape) != self.field_shape:
            x = x.reshape(self.field_shape)
        return x

    @staticmethod
    def _ptr(x):
        return ctypes.c_void_p(x.data_ptr())

    def launches(self):
        return int(self.lib.fhp_plan_launches(self.handle))

    def profile(self, enable=True):
        """Start (reset) or stop per-kernel CUDA-event timing."""
        _lib.check(self.lib.fhp_profile_enable(self.handle, int(bool(enable))), 'profile')

    def profile_read(self, max_kinds=32):
        """{kernel: {'launches', 'ms', 'bytes_per_launch'}} of the recorded passes."""
        names = ctypes.create_string_buffer(64 * max_kinds)
        la = (ctypes.c_longlong * max_kinds)()
        ms = (ctypes.c_double * max_kinds)()
        by = (ctypes.c_double * max_kinds)()
        nk = ctypes.c_int()
        _lib.check(self.lib.fhp_profile_read(self.handle, max_kinds, names, la, ms, by,
                                             ctypes.byref(nk)), 'profile_read')
        out = {}
        for i in range(min(nk.value, max_kinds)):
            nm = names.raw[64 * i:64 * (i + 1)].split(b'\0')[0].decode()
            out[nm] = {'launches': int(la[i]), 'ms': float(ms[i]),
                       'bytes_per_launch': float(by[i])}
        return out

    # -- API -------------------------------------------------------------------
    def set_coefficient(self, A, kind=None):
        """A: (dv, dv) + N coefficient (numpy, or torch on the GPU), origin 0.
        Plans of several cells take packed values (set_coefficient_packed)."""
        if self.ncells > 1:
            raise ValueError('a plan of several cells takes set_coefficient_packed')
        shape = (self.dv, self.dv) + self.coef_grid
        if tuple(A.shape) != shape:
            raise ValueError('coefficient shape %s, expected %s' % (tuple(A.shape), shape))
        if isinstance(A, torch.Tensor) and A.is_cuda:
            A = A.detach().to(self.device, torch.float64)
            kind = coef_kind_of_torch(A) if kind is None else kind
            vals = pack_coefficient_torch(A, kind)
            _lib.check(self.lib.fhp_set_coefficient(self.handle, kind, self._ptr(vals), 1,
                                                    self._stream()), 'fhp_set_coefficient')
        else:
            if isinstance(A, torch.Tensor):
                A = A.detach().cpu().numpy()
            A = np.asarray(A, dtype=np.float64)
            kind = coef_kind_of(A) if kind is None else kind
            vals = pack_coefficient(A, kind)
            _lib.check(self.lib.fhp_set_coefficient(self.handle, kind, vals.ctypes.data_as(
                ctypes.c_void_p), 0, self._stream()), 'fhp_set_coefficient')
        torch.cuda.current_stream(self.device).synchronize()
        self.coef_kind = kind

    def set_coefficient_packed(self, vals, kind):
        """vals: packed (c,) + coefficient grid float64 (numpy, or torch on the
        GPU) of kind FHP_COEF_ISO / SYM / FULL (c = 1, dv(dv+1)/2, dv*dv)."""
        c = {_lib.FHP_COEF_ISO: 1, _lib.FHP_COEF_SYM: self.dv * (self.dv + 1) // 2,
             _lib.FHP_COEF_FULL: self.dv * self.dv}[kind]
        shape = ((self.ncells,) if self.ncells > 1 else ()) + (c,) + self.coef_grid
        if tuple(vals.shape) != shape:
            vals = vals.reshape(shape)
        if isinstance(vals, torch.Tensor) and vals.is_cuda:
            vals = vals.detach().to(self.device, torch.float64).contiguous()
            _lib.check(self.lib.fhp_set_coefficient(self.handle, kind, self._ptr(vals), 1,
                                                    self._stream()), 'fhp_set_coefficient')
        else:
            if isinstance(vals, torch.Tensor):
                vals = vals.detach().cpu().numpy()
            vals = np.ascontiguousarray(vals, dtype=np.float64)
            _lib.check(self.lib.fhp_set_coefficient(self.handle, kind, vals.ctypes.data_as(
                ctypes.c_void_p), 0, self._stream()), 'fhp_set_coefficient')
        torch.cuda.current_stream(self.device).synchronize()
        self.coef_kind = kind

    def apply(self, x, proj=1):
        x = self._dev(x)
        y = self.empty()
        _lib.check(self.lib.fhp_apply(self.handle, proj, self._ptr(x), self._ptr(y),
                                      self._stream()), 'fhp_apply')
        return y

    def rhs_macro(self, proj=1):
        b = self.empty()
        _lib.check(self.lib.fhp_rhs_macro(self.handle, proj, self._ptr(b), self._stream()),
                   'fhp_rhs_macro')
        return b

    def cg(self, b, x0=None, tol=1e-6, maxiter=1000, proj=1, log_rows=None):
        """Batched CG; returns (x, info) with per-load kit / norm_res / res_log
        (every load of every cell, cell-major, for a plan of several cells)."""
        b = self._dev(b)
        x0p = ctypes.c_void_p(None)
        if x0 is not None:
            x0 = self._dev(x0)
            x0p = self._ptr(x0)
        x = self.empty()
        L = self._lk
        kit = (ctypes.c_int * L)()
        nres = (ctypes.c_double * L)()
        stat = (ctypes.c_int * L)()
        maxiter = int(maxiter)
        rows = int(log_rows if log_rows is not None else min(maxiter + 1, 100001))
        log = np.zeros((rows, L))
        st = self.lib.fhp_cg_solve(self.handle, proj, self._ptr(b), x0p, float(tol), maxiter,
                                   self._ptr(x), kit, nres, stat,
                                   log.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), rows,
                                   self._stream())
        _lib.check(st, 'fhp_cg_solve')
        kits = list(kit)
        info = {'kit': kits, 'norm_res': list(nres), 'status': list(stat),
                'res_log': [log[:k + 1, l].copy() for l, k in enumerate(kits)]}
        return x, info

    def solve_other(self, kind, b, x0=None, tol=1e-6, maxiter=1000, proj=1, p0=0., p1=0.):
        """Richardson ('richardson', p0 = omega), two-term Chebyshev
        ('chebyshev', eigenvalues in [p0, p1]) or BiCG ('bicg') on the GPU,
        all loads at once (fhp_richardson_solve / fhp_chebyshev_solve /
        fhp_bicg_solve).  Returns (x, info) with per-load kit / norm_res /
        status."""
        b = self._dev(b)
        x0p = ctypes.c_void_p(None)
        if x0 is not None:
            x0 = self._dev(x0)
            x0p = self._ptr(x0)
        x = self.empty()
        L = self.nloads
        kit = (ctypes.c_int * L)()
        nres = (ctypes.c_double * L)()
        stat = (ctypes.c_int * L)()
        args = (kit, nres, stat, self._stream())
        if kind == 'richardson':
            st = self.lib.fhp_richardson_solve(self.handle, proj, self._ptr(b), x0p, float(p0),
                                               float(tol), int(maxiter), self._ptr(x), *args)
        elif kind == 'chebyshev':
            st = self.lib.fhp_chebyshev_solve(self.handle, proj, self._ptr(b), x0p, float(p0),
                                              float(p1), float(tol), int(maxiter), self._ptr(x),
                                              *args)
        elif kind == 'bicg':
            st = self.lib.fhp_bicg_solve(self.handle, proj, self._ptr(b), x0p, float(tol),
                                         int(maxiter), self._ptr(x), *args)
        else:
            raise ValueError('unknown solver %s' % kind)
        _lib.check(st, 'fhp_%s_solve' % kind)
        return x, {'kit': list(kit), 'norm_res': list(nres), 'status': list(stat)}

    def autotune(self):
        """Time candidate launch shapes of the operator on this plan and keep
        the fastest (fhp_plan_autotune; cached per plan geometry).  Returns
        (choice triple, ms per operator application)."""
        ch = (ctypes.c_int * 3)()
        ms = ctypes.c_float()
        _lib.check(self.lib.fhp_plan_autotune(self.handle, ch, ctypes.byref(ms), self._stream()),
                   'fhp_plan_autotune')
        return tuple(ch), float(ms.value)

    def energy(self, X, add_macro=True):
        """A_H[i, j] = <A u_i, u_j> over the solve grid (u = X + E if add_macro);
        (cells, L, L) for a plan of several cells."""
        X = self._dev(X)
        L = self.nloads
        AH = np.zeros(((self.ncells,) if self.ncells > 1 else ()) + (L, L))
        _lib.check(self.lib.fhp_energy_matrix(self.handle, self._ptr(X), int(bool(add_macro)),
                                              AH.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                              self._stream()), 'fhp_energy_matrix')
        return AH

    def energy_gradient(self, X, W, add_macro=True):
        """d(sum_ij W_ij A_H[i, j]) / dA_c(v) for the stored coefficient
        components c of this plan's kind: a float64 torch tensor (c,) + N."""
        X = self._dev(X)
        L = self.nloads
        W = np.ascontiguousarray(np.broadcast_to(np.asarray(W, dtype=np.float64), (L, L)))
        c = {_lib.FHP_COEF_ISO: 1, _lib.FHP_COEF_SYM: self.dv * (self.dv + 1) // 2,
             _lib.FHP_COEF_FULL: self.dv * self.dv}[self.coef_kind]
        grad = torch.empty((c,) + self.N, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.fhp_energy_gradient(
            self.handle, self._ptr(X), int(bool(add_macro)),
            W.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self._ptr(grad),
            self._stream()), 'fhp_energy_gradient')
        return grad

    def interpolate(self, x, grid):
        """Trigonometric interpolation of this plan's fields onto grid (>= N)."""
        grid = tuple(int(n) for n in grid)
        if grid == self.N:
            return self._dev(x)
        return interpolate_fields(self._dev(x), self.N, grid)

    def interpolate_to(self, other, x):
        """Trigonometric interpolation of fields x onto other's grid."""
        x = self._dev(x)
        y = other.empty()
        _lib.check(self.lib.fhp_fourier_interp(self.handle, other.handle, self._ptr(x),
                                               self._ptr(y), self._stream()),
                   'fhp_fourier_interp')
        return y

    # -- potential formulation (tensorsLowRank/homogenisation.py:41-127) -------
    @property
    def potential_shape(self):
        """(loads,) + the 'r' half-spectrum shape of the band grid N."""
        return (self.nloads,) + self.band[:-1] + (self.band[-1] // 2 + 1,)

    def _cdev(self, x):
        cdt = torch.complex64 if self.precision == 'f32' else torch.complex128
        if not isinstance(x, torch.Tensor):
            x = torch.as_tensor(np.asarray(x))
        x = x.to(device=self.device, dtype=cdt).contiguous()
        if tuple(x.shape) != self.potential_shape:
            x = x.reshape(self.potential_shape)
        return x

    def _cempty(self):
        cdt = torch.complex64 if self.precision == 'f32' else torch.complex128
        return torch.empty(self.potential_shape, dtype=cdt, device=self.device)

    def potential_rhs(self):
        """P B per load, B_l = div(decrease_N F(A E_l)) (homogenisation.py:58, 95)."""
        b = self._cempty()
        _lib.check(self.lib.fhp_potential_rhs(self.handle, self._ptr(b), self._stream()),
                   'fhp_potential_rhs')
        return b

    def potential_apply(self, x):
        """PDFAFGPfun(x) per load (homogenisation.py:50-65, 88-101)."""
        x = self._cdev(x)
        y = self._cempty()
        _lib.check(self.lib.fhp_potential_apply(self.handle, self._ptr(x), self._ptr(y),
                                                self._stream()), 'fhp_potential_apply')
        return y

    def potential_cg(self, b, tol=1e-6, maxiter=1000, log_rows=None):
        """CG from 0 with the 'r' Fourier inner product; returns (iPU, info)."""
        b = self._cdev(b)
        x = self._cempty()
        L = self.nloads
        kit = (ctypes.c_int * L)()
        nres = (ctypes.c_double * L)()
        stat = (ctypes.c_int * L)()
        maxiter = int(maxiter)
        rows = int(log_rows if log_rows is not None else min(maxiter + 1, 100001))
        log = np.zeros((rows, L))
        _lib.check(self.lib.fhp_potential_cg(self.handle, self._ptr(b), float(tol), maxiter,
                                             self._ptr(x), kit, nres, stat,
                                             log.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             rows, self._stream()), 'fhp_potential_cg')
        kits = list(kit)
        return x, {'kit': kits, 'norm_res': list(nres), 'status': list(stat),
                   'res_log': [log[:k + 1, l].copy() for l, k in enumerate(kits)]}

    def potential_field(self, x):
        """X = iF(enlarge(grad(P x))) as this plan's fields (loads, dim) + N."""
        x = self._cdev(x)
        X = self.empty()
        _lib.check(self.lib.fhp_potential_field(self.handle, self._ptr(x), self._ptr(X),
                                                self._stream()), 'fhp_potential_field')
        return X

    def homogenize_host(self, A=None, proj=1, tol=1e-6, maxiter=1000, return_solution=False,
                        packed=None, kind=None):
        """End to end with host buffers: coefficient in, A_H out (fhp_homogenize_host).

        A: (dv, dv) + N host coefficient, or packed: host values already in the
        layout of kind (e.g. a(x) for FHP_COEF_ISO, shape (1,) + N or N).
        """
        if packed is not None:
            if kind is None:
                raise ValueError('packed values need their kind')
            vals = np.ascontiguousarray(packed, dtype=np.float64)
        else:
            A = np.asarray(A, dtype=np.float64)
            kind = coef_kind_of(A)
            vals = pack_coefficient(A, kind)
        L = self.nloads
        AH = np.zeros(((self.ncells,) if self.ncells > 1 else ()) + (L, L))
        kit = (ctypes.c_int * self._lk)()
        nres = (ctypes.c_double * self._lk)()
        xh = None
        xp = ctypes.c_void_p(None)
        if return_solution:
            xh = np.zeros(self.field_shape, dtype=np.float32 if self.precision == 'f32'
                          else np.float64)
            xp = xh.ctypes.data_as(ctypes.c_void_p)
        st = self.lib.fhp_homogenize_host(self.handle, proj, kind,
                                          vals.ctypes.data_as(ctypes.c_void_p), float(tol),
                                          int(maxiter),
                                          AH.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          kit, nres, xp, self._stream())
        _lib.check(st, 'fhp_homogenize_host')
        self.coef_kind = kind
        return AH, list(kit), list(nres), xh


# Plans of small grids reused across calls of the drop-in API (creation
# allocates and uploads line tables: a latency-bound problem would pay it on
# every call); least recently used first out
_PLAN_CACHE = collections.OrderedDict()
_PLAN_CACHE_LOCK = threading.Lock()
_PLAN_CACHE_SIZE = 4
_PLAN_CACHE_MAX_POINTS = 1 << 21


def shared_plan(N, Y, **kw):
    """GalerkinPlan(N, Y, **kw) from a small process-wide cache when its grids
    are small (at most 2^21 points), else a new plan.  A cached plan is the
    caller's until its next request of the same geometry; one thread at a
    time (the Problem / applications path)."""
    N = tuple(int(n) for n in N)
    integ = kw.get('integ')
    pts = max(int(np.prod(N)), int(np.prod(integ)) if integ is not None else 0)
    if pts > _PLAN_CACHE_MAX_POINTS:
        return GalerkinPlan(N, Y, **kw)
    norm = tuple(sorted((k, tuple(v) if isinstance(v, (list, tuple, np.ndarray)) else v)
                        for k, v in kw.items()))
    key = (torch.cuda.current_device(), N, tuple(np.asarray(Y, dtype=np.float64).tolist()), norm)
    with _PLAN_CACHE_LOCK:
        plan = _PLAN_CACHE.get(key)
        if plan is not None:
            _PLAN_CACHE.move_to_end(key)
            return plan
    plan = GalerkinPlan(N, Y, **kw)
    with _PLAN_CACHE_LOCK:
        _PLAN_CACHE[key] = plan
        while len(_PLAN_CACHE) > _PLAN_CACHE_SIZE:
            _PLAN_CACHE.popitem(last=False)
    return plan


def homogenize_host_many(plan, packed, kind, proj=1, tol=1e-6, maxiter=1000):
    """fhp_homogenize_host_many: A_H of several host coefficients (packed
    values of `kind`, each (cells, c) + grid or (c,) + grid) on one plan, the
    next upload overlapping the current solve (pinned host arrays overlap).
    Returns (AH list, kit list, norm_res list) per coefficient."""
    require_cuda()
    vals = [np.ascontiguousarray(v, dtype=np.float64) for v in packed]
    n = len(vals)
    lead = (plan.ncells,) if plan.ncells > 1 else ()
    L = plan.nloads
    AH = np.zeros((n,) + lead + (L, L))
    kit = (ctypes.c_int * (n * plan._lk))()
    nres = (ctypes.c_double * (n * plan._lk))()
    ptrs = (ctypes.c_void_p * n)(*[v.ctypes.data for v in vals])
    st = plan.lib.fhp_homogenize_host_many(plan.handle, int(proj), int(kind), n, ptrs,
                                           float(tol), int(maxiter),
                                           AH.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           kit, nres, plan._stream())
    _lib.check(st, 'fhp_homogenize_host_many')
    plan.coef_kind = kind
    k = plan._lk
    return ([AH[i] for i in range(n)], [list(kit[i * k:(i + 1) * k]) for i in range(n)],
            [list(nres[i * k:(i + 1) * k]) for i in range(n)])


def cg_many(plans, bs, tol=1e-6, maxiter=1000, proj=1):
    """CG on several plans at once (fhp_cg_solve_many): plan i solves its own
    loads from bs[i], zero start, with its own scalars and stopping tests; all
    plans advance together, one CUDA graph per iteration.  Returns
    [(x_i, info_i)] with info as GalerkinPlan.cg (without residual logs)."""
    require_cuda()
    plans = list(plans)
    if not plans:
        return []
    lib = plans[0].lib
    n = len(plans)
    bs = [p._dev(b) for p, b in zip(plans, bs)]
    xs = [p.empty() for p in plans]
    hs = (ctypes.c_void_p * n)(*[p.handle.value for p in plans])
    bp = (ctypes.c_void_p * n)(*[b.data_ptr() for b in bs])
    xp = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
    tot = sum(p._lk for p in plans)
    kit = (ctypes.c_int * tot)()
    nres = (ctypes.c_double * tot)()
    stat = (ctypes.c_int * tot)()
    st = lib.fhp_cg_solve_many(n, hs, int(proj), bp, float(tol), int(maxiter), xp, kit, nres,
                               stat, plans[0]._stream())
    _lib.check(st, 'fhp_cg_solve_many')
    out, off = [], 0
    for p, x in zip(plans, xs):
        L = p._lk
        out.append((x, {'kit': list(kit[off:off + L]), 'norm_res': list(nres[off:off + L]),
                        'status': list(stat[off:off + L])}))
        off += L
    return out


def _fft_plan(grid, ncomp, precision):
    lib = _lib.load()
    h = ctypes.c_void_p()
    n = (ctypes.c_int * len(grid))(*grid)
    prec = _lib.FHP_F32 if precision == torch.float32 else _lib.FHP_F64
    _lib.check(lib.fhp_fft_plan_create(ctypes.byref(h), len(grid), n, ncomp, prec),
               'fhp_fft_plan_create')
    return h


# FFT plans of small grids, kept for the process (creation uploads line
# tables and allocates; a latency-bound problem would pay it on every call);
# a plan is not re-entrant, so its use is serialised
_FFT_CACHE = collections.OrderedDict()
_FFT_CACHE_LOCK = threading.Lock()
_FFT_CACHE_MAX = 1 << 22     # grid points x components of a cached plan
_FFT_CACHE_SIZE = 16         # cached plan pairs (least recently used out)


def interpolate_fields(x, src, dst):
    """Trigonometric interpolation (Tensor.project, objects.py:488-511) of the
    fields x[..., src] onto grid dst >= src on the GPU (fhp_fourier_interp)."""
    lib = _lib.load()
    src = tuple(int(n) for n in src)
    dst = tuple(int(n) for n in dst)
    lead = tuple(x.shape[:x.dim() - len(src)])
    ncomp = int(np.prod(lead)) if lead else 1
    xs = x.reshape((ncomp,) + src).contiguous()
    out = torch.empty((ncomp,) + dst, dtype=x.dtype, device=x.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    for k0 in range(0, ncomp, 6):
        k1 = min(ncomp, k0 + 6)
        args = (ctypes.c_void_p(xs[k0:k1].data_ptr()), ctypes.c_void_p(out[k0:k1].data_ptr()),
                stream)
        if int(np.prod(dst)) * (k1 - k0) <= _FFT_CACHE_MAX:
            key = (x.device.index, src, dst, k1 - k0, x.dtype)
            with _FFT_CACHE_LOCK:
                if key not in _FFT_CACHE:
                    _FFT_CACHE[key] = (_fft_plan(src, k1 - k0, x.dtype),
                                       _fft_plan(dst, k1 - k0, x.dtype))
                    while len(_FFT_CACHE) > _FFT_CACHE_SIZE:
                        for h in _FFT_CACHE.popitem(last=False)[1]:
                            lib.fhp_plan_destroy(h)
                _FFT_CACHE.move_to_end(key)
                hs, hd = _FFT_CACHE[key]
                _lib.check(lib.fhp_fourier_interp(hs, hd, *args), 'fhp_fourier_interp')
            continue
        hs = _fft_plan(src, k1 - k0, x.dtype)
        try:
            hd = _fft_plan(dst, k1 - k0, x.dtype)
            try:
                _lib.check(lib.fhp_fourier_interp(hs, hd, *args), 'fhp_fourier_interp')
            finally:
                lib.fhp_plan_destroy(hd)
        finally:
            lib.fhp_plan_destroy(hs)
    return out.reshape(lead + dst)


def coefficient_inverse(A, shift=False):
    """Per-voxel inverse of a (d, d) + grid coefficient on the GPU
    (fhp_coefficient_inverse): the reference's Gauss-Jordan elimination
    without pivoting (trigpol.py:120-159, Tensor.inv objects.py:247-251),
    bit-identical to it for finite input.  A: NumPy array or torch tensor;
    shift=True also moves a centred origin to 0 (the ifftshift of
    Material.get_A_GaNi, materials.py:115-123).  Returns a float64 CUDA tensor.
    """
    require_cuda()
    lib = _lib.load()
    if isinstance(A, np.ndarray):
        A = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float64))
    A = A.to('cuda' if not A.is_cuda else A.device, torch.float64).contiguous()
    d = int(A.shape[0])
    if A.dim() < 3 or A.shape[1] != d:
        raise NotImplementedError('Non-square matrix!')
    grid = tuple(int(n) for n in A.shape[2:])
    out = torch.empty_like(A)
    n = (ctypes.c_int * len(grid))(*grid)
    stream = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    _lib.check(lib.fhp_coefficient_inverse(len(grid), n, d, ctypes.c_void_p(A.data_ptr()),
                                           ctypes.c_void_p(out.data_ptr()), int(bool(shift)),
                                           stream), 'fhp_coefficient_inverse')
    return out


def ball_characteristic(N, r, volume, sq, phase):
    """Ga characteristic function of a ball on the odd grid N, origin 0, on
    the GPU (fhp_ball_characteristic): the inverse transform of
    W(|xi|) prod_a phase_a.  sq, phase: per-axis host tables in centred
    position order (xi_a^2 and the complex phases), as the reference pairs
    them in Material.get_shape_functions (materials.py:125-169, 317-330,
    392-425).  Returns a float64 CUDA tensor of shape N."""
    require_cuda()
    lib = _lib.load()
    N = tuple(int(n) for n in N)
    h = _fft_plan(N, 1, torch.float64)
    out = torch.empty(N, dtype=torch.float64, device='cuda')
    sq = np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.float64) for s in sq]))
    ph = np.concatenate([np.asarray(p, dtype=np.complex128) for p in phase])
    ph = np.ascontiguousarray(ph.view(np.float64))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    try:
        _lib.check(lib.fhp_ball_characteristic(
            h, float(r), float(volume), sq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_void_p(out.data_ptr()),
            stream), 'fhp_ball_characteristic')
    finally:
        lib.fhp_plan_destroy(h)
    return out


def separable_char(N, re, im=None):
    """Product of per-axis factors on grid N on the GPU (fhp_separable_char):
    prod_a re_a[x_a], or with im the real part of prod_a (re_a + i im_a)[x_a],
    rounded as NumPy's outer products round them.  re, im: sequences of
    per-axis host vectors.  Returns a float64 CUDA tensor of shape N."""
    require_cuda()
    lib = _lib.load()
    N = tuple(int(n) for n in N)
    out = torch.empty(N, dtype=torch.float64, device='cuda')
    r = np.ascontiguousarray(np.concatenate([np.asarray(v, dtype=np.float64) for v in re]))
    dp = ctypes.POINTER(ctypes.c_double)
    ip = None
    if im is not None:
        i_ = np.ascontiguousarray(np.concatenate([np.asarray(v, dtype=np.float64) for v in im]))
        ip = i_.ctypes.data_as(dp)
    n = (ctypes.c_int * len(N))(*N)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.fhp_separable_char(len(N), n, r.ctypes.data_as(dp), ip,
                                      ctypes.c_void_p(out.data_ptr()), stream),
               'fhp_separable_char')
    return out


def ball_topology(axes, x0, Y, radius):
    """GaNi topology of a ball (fhp_ball_topology): at every node of the
    tensor grid with per-axis coordinates axes, the number of the 3^d periodic
    images within radius (materials.py:212-301), bit-identical to the NumPy
    evaluation.  Returns a float64 CUDA tensor."""
    require_cuda()
    lib = _lib.load()
    d = len(axes)
    N = tuple(int(len(a)) for a in axes)
    out = torch.empty(N, dtype=torch.float64, device='cuda')
    ax = np.ascontiguousarray(np.concatenate([np.asarray(a, dtype=np.float64) for a in axes]))
    x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.float64))
    Y = np.ascontiguousarray(np.asarray(Y, dtype=np.float64))
    n = (ctypes.c_int * d)(*N)
    dp = ctypes.POINTER(ctypes.c_double)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.fhp_ball_topology(d, n, ax.ctypes.data_as(dp), x0.ctypes.data_as(dp),
                                     Y.ctypes.data_as(dp), float(radius),
                                     ctypes.c_void_p(out.data_ptr()), stream),
               'fhp_ball_topology')
    return out


def outer_accumulate(out, v, c):
    """out[k] += v[k] * c over a (nv,) + grid CUDA float64 field, on the GPU
    (fhp_outer_accumulate): one inclusion's term of Material.get_A_Ga, order
    None (materials.py:66-75), bit-identical to val += np.multiply.outer(v, c).
    v: nv host values; c: CUDA float64 tensor of the grid's shape."""
    require_cuda()
    lib = _lib.load()
    v = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
    M = int(c.numel())
    if out.dtype != torch.float64 or c.dtype != torch.float64 or not out.is_contiguous() \
            or not c.is_contiguous() or out.numel() != v.size * M:
        raise ValueError('out must be a contiguous float64 field of len(v) x c.numel() values')
    stream = ctypes.c_void_p(torch.cuda.current_stream(out.device).cuda_stream)
    _lib.check(lib.fhp_outer_accumulate(int(v.size),
                                        v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        ctypes.c_void_p(c.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), M, stream),
               'fhp_outer_accumulate')
