"""GPU parity of the potential formulation (fhp_potential_* through the C ABI)
against the reference's homog_GaNi_full_potential / homog_Ga_full_potential
(ffthompy/tensorsLowRank/homogenisation.py:41-127; fixtures
tests/golden/pot_*.npz) and against the oracle.

Tolerances: FP64 operator 1e-12 relative (max-norm); FP64 A_H 1e-10
relative with the reference's CG iteration count (+-1 where the reference
residual at the smaller count is already within 3 tol: the small even-N
cases run more CG iterations than they have unknowns, where residual
histories drift with roundoff); the potential Fu to
1e-7 of its max (CG tolerance 1e-8); FP32 A_H within 1e-5 of FP64.
"""
import numpy as np
import pytest

import golden_io
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

POT = golden_io.names('pot_')


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _relmax(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _tensor(A):
    from ffthompy_gb300.tensors.objects import Tensor
    return Tensor(name='A', val=A, order=2, multype=21)


@pytest.mark.parametrize('name', POT)
def test_potential_operator_matches_reference(name):
    from ffthompy_gb300.engine import GalerkinPlan
    meta, arr = golden_io.load(name)
    N = tuple(meta['N'])
    plan = GalerkinPlan(N, meta['Y'], physics='scalar', nloads=1)
    plan.set_coefficient(arr['A_gani'])
    y = plan.potential_apply(arr['x'][None])[0].cpu().numpy()
    assert _relmax(y, arr['y__gani']) < 1e-12
    if 'y__ga' in arr:
        Nbar = tuple(2 * n - 1 for n in N)
        pg = GalerkinPlan(Nbar, meta['Y'], physics='scalar', nloads=1, band=N)
        pg.set_coefficient(arr['A_ga'])
        y = pg.potential_apply(arr['x'][None])[0].cpu().numpy()
        assert _relmax(y, arr['y__ga']) < 1e-12


def _kit_ok(kit, ref_kit, A, N, tol, Nbar):
    if kit == ref_kit:
        return True
    if abs(kit - ref_kit) > 1:
        return False
    out = oracle.homog_potential(A, N, np.ones(len(N)), tol, max(kit, ref_kit), Nbar=Nbar)
    log = out['info']['res_log']
    r = log[min(kit, ref_kit)]
    return r <= 3 * tol


@pytest.mark.parametrize('name', POT)
def test_potential_solve_matches_reference(name):
    import ffthompy_gb300.tensorsLowRank.homogenisation as H
    meta, arr = golden_io.load(name)
    N = tuple(meta['N'])
    pars = H.Struct(Y=np.ones(len(N)), solver={'tol': meta['tol'], 'maxiter': meta['maxiter']})
    for key in meta['runs']:
        if key == 'gani':
            r = H.homog_GaNi_full_potential(_tensor(arr['A_gani']), None, pars)
            A, Nbar = arr['A_gani'], None
        elif key == 'gani_ga':
            r = H.homog_GaNi_full_potential(_tensor(arr['A_gani']), _tensor(arr['A_ga']), pars)
            A, Nbar = arr['A_gani'], None
        else:
            r = H.homog_Ga_full_potential(_tensor(arr['A_ga']), pars)
            A, Nbar = arr['A_ga'], tuple(2 * n - 1 for n in N)
        ref_ah = float(arr['AH__' + key])
        assert abs(r.AH - ref_ah) <= 1e-10 * abs(ref_ah), (key, r.AH, ref_ah)
        assert _kit_ok(r.info['kit'], int(arr['kit__' + key]), A, N, meta['tol'], Nbar), (
            key, r.info['kit'], int(arr['kit__' + key]))
        assert r.info['status'] == 0
        assert _relmax(r.Fu.val, arr['Fu__' + key]) < 1e-7, key
        assert abs(r.Fu.mean()) < 1e-12


def test_potential_all_loads_and_gradient_formulation():
    """loads = d: A_H is symmetric, its (0,0) entry is the single-load value,
    and it equals the A_H of the gradient (Green projection) formulation on
    the same discretisation (GaNi and Ga), to the CG tolerance."""
    import ffthompy_gb300.tensorsLowRank.homogenisation as H
    from ffthompy_gb300.engine import GalerkinPlan
    meta, arr = golden_io.load('pot_s3_fun_aniso')
    N = tuple(meta['N'])
    Nbar = tuple(2 * n - 1 for n in N)
    pars = H.Struct(Y=np.ones(3), solver={'tol': 1e-10, 'maxiter': 500})
    for A, solve in ((arr['A_gani'], 'gani'), (arr['A_ga'], 'ga')):
        if solve == 'gani':
            full = H.homog_GaNi_full_potential(_tensor(A), None, pars, loads=3)
            one = H.homog_GaNi_full_potential(_tensor(A), None, pars)
            plan = GalerkinPlan(N, np.ones(3), physics='scalar', nloads=3)
        else:
            full = H.homog_Ga_full_potential(_tensor(A), pars, loads=3)
            one = H.homog_Ga_full_potential(_tensor(A), pars)
            plan = GalerkinPlan(Nbar, np.ones(3), physics='scalar', nloads=3, band=N)
        AH = full.AH
        assert AH.shape == (3, 3)
        assert _relmax(AH, AH.T) < 1e-9
        assert abs(AH[0, 0] - one.AH) <= 1e-9 * abs(one.AH)
        plan.set_coefficient(A)
        X, info = plan.cg(plan.rhs_macro(1), tol=1e-10, maxiter=500)
        AHg = plan.energy(X)
        assert _relmax(AH, AHg) < 1e-8, (solve, AH, AHg)


def test_potential_fp32():
    import ffthompy_gb300.tensorsLowRank.homogenisation as H
    meta, arr = golden_io.load('pot_s3_fun5')
    res = {}
    for prec in ('f64', 'f32'):
        pars = H.Struct(Y=np.ones(3), solver={'tol': 1e-6, 'maxiter': 300}, precision=prec)
        res[prec] = H.homog_Ga_full_potential(_tensor(arr['A_ga']), pars).AH
    assert abs(res['f32'] - res['f64']) <= 1e-5 * abs(res['f64']), res


def test_potential_larger_grid_vs_oracle():
    """3D GaNi 31^3 and Ga 15^3 -> 29^3 with a contrast-100 random material:
    A_H and iteration counts against the oracle."""
    import ffthompy_gb300.tensorsLowRank.homogenisation as H
    rng = np.random.default_rng(5)
    for N, kind in (((31, 31, 31), 'gani'), ((15, 15, 15), 'ga')):
        grid = N if kind == 'gani' else tuple(2 * n - 1 for n in N)
        a = 1. + 99. * (rng.random(grid) < 0.3)
        A = np.einsum('ij,...->ij...', np.eye(3), a)
        pars = H.Struct(Y=np.ones(3), solver={'tol': 1e-8, 'maxiter': 400})
        if kind == 'gani':
            r = H.homog_GaNi_full_potential(_tensor(A), None, pars)
            o = oracle.homog_potential(A, N, np.ones(3), 1e-8, 400)
        else:
            r = H.homog_Ga_full_potential(_tensor(A), pars)
            o = oracle.homog_potential(A, N, np.ones(3), 1e-8, 400, Nbar=grid)
        assert abs(r.AH - o['AH']) <= 1e-9 * abs(o['AH']), (kind, r.AH, o['AH'])
        assert abs(r.info['kit'] - o['info']['kit']) <= 1, (kind, r.info['kit'], o['info']['kit'])


def test_potential_rejects_unsupported_plans():
    from ffthompy_gb300.engine import GalerkinPlan
    A = np.einsum('ij,...->ij...', np.eye(2), np.ones((7, 7)))
    pe = GalerkinPlan((7, 7), np.ones(2), physics='elasticity', nloads=1)
    pe.set_coefficient(np.einsum('ij,...->ij...', np.eye(3), np.ones((7, 7))))
    with pytest.raises(ValueError):
        pe.potential_rhs()
    pb = GalerkinPlan((4, 4), np.ones(2), physics='scalar', nloads=1, integ=(8, 8))
    pb.set_coefficient(np.einsum('ij,...->ij...', np.eye(2), np.ones((8, 8))))
    with pytest.raises(ValueError):
        pb.potential_rhs()
    pg = GalerkinPlan((7, 7), np.ones(2), physics='scalar', nloads=1, band=(4, 4))
    pg.set_coefficient(A)
    with pytest.raises(ValueError):
        pg.potential_rhs()
