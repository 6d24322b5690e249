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
