"""fhp_homogenize_host_many (the next coefficient uploaded while the current
problem is solved) gives, per coefficient, exactly what fhp_homogenize_host
gives for it alone: GaNi FP64 / FP32 / mixed and a band (Ga) plan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _coefs(shape, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        a = 1. + 20. * (rng.random(shape) < 0.35)
        buf = torch.empty((1,) + shape, dtype=torch.float64, pin_memory=True).numpy()
        buf[0] = a
        out.append(buf)
    return out


@pytest.mark.parametrize('precision', ['f64', 'f32', 'mixed'])
def test_host_many_equals_single_calls(precision):
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.engine import GalerkinPlan, homogenize_host_many
    N = (33, 45)
    vals = _coefs(N, 4, seed=5)
    tol = 1e-5 if precision == 'f32' else 1e-9
    plan = GalerkinPlan(N, np.ones(2), precision=precision)
    AHs, kits, _ = homogenize_host_many(plan, vals, _lib.FHP_COEF_ISO, tol=tol, maxiter=800)
    ref = GalerkinPlan(N, np.ones(2), precision=precision)
    for v, AH, kit in zip(vals, AHs, kits):
        AH1, kit1, _, _ = ref.homogenize_host(packed=v, kind=_lib.FHP_COEF_ISO, tol=tol,
                                              maxiter=800)
        assert kit == kit1, (kit, kit1)
        assert np.array_equal(AH, AH1), (AH, AH1)


@pytest.mark.parametrize('N', [(15, 15, 15), (15, 16)])
@pytest.mark.parametrize('precision', ['f64', 'f32'])
def test_host_band_fused_equals_device_calls(N, precision):
    """Band plans run the host call's right-hand side, CG and energy with
    every vector in the spectral form (no real fields in between): the same
    iterations, A_H and solution as rhs_macro / cg / energy on device buffers
    (FP64 to roundoff; FP32 to its precision, iteration counts within 3 % or 1)."""
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.engine import GalerkinPlan, nice_size
    d = len(N)
    integ = tuple(nice_size(2 * n - 1) for n in N)
    v = _coefs(integ, 1, seed=11)[0]
    tol = 1e-9 if precision == 'f64' else 1e-4
    p1 = GalerkinPlan(N, np.ones(d), precision=precision, integ=integ)
    AH, kit, _, xh = p1.homogenize_host(packed=v, kind=_lib.FHP_COEF_ISO, tol=tol, maxiter=500,
                                        return_solution=True)
    p2 = GalerkinPlan(N, np.ones(d), precision=precision, integ=integ)
    p2.set_coefficient_packed(v, _lib.FHP_COEF_ISO)
    X, info = p2.cg(p2.rhs_macro(1), tol=tol, maxiter=500)
    AH2 = p2.energy(X)
    Xn = X.double().cpu().numpy()
    rel = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())
    if precision == 'f64':
        assert kit == info['kit'], (kit, info['kit'])
        assert rel(AH, AH2) < 1e-12, rel(AH, AH2)
        assert rel(xh, Xn) < 1e-10, rel(xh, Xn)
    else:
        assert all(abs(p - q) <= max(1, int(np.ceil(0.03 * q)))
                   for p, q in zip(kit, info['kit'])), (kit, info['kit'])
        assert rel(AH, AH2) < 1e-5, rel(AH, AH2)
        assert rel(xh, Xn) < 1e-2, rel(xh, Xn)


def test_host_many_band_plan():
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.engine import GalerkinPlan, homogenize_host_many, nice_size
    N = (15, 15, 15)
    integ = tuple(nice_size(2 * n - 1) for n in N)
    vals = _coefs(integ, 3, seed=9)
    plan = GalerkinPlan(N, np.ones(3), precision='f32', integ=integ)
    AHs, kits, _ = homogenize_host_many(plan, vals, _lib.FHP_COEF_ISO, tol=1e-4, maxiter=500)
    ref = GalerkinPlan(N, np.ones(3), precision='f32', integ=integ)
    for v, AH, kit in zip(vals, AHs, kits):
        AH1, kit1, _, _ = ref.homogenize_host(packed=v, kind=_lib.FHP_COEF_ISO, tol=1e-4,
                                              maxiter=500)
        assert kit == kit1
        assert np.abs(AH - AH1).max() <= 1e-12 * np.abs(AH1).max()
