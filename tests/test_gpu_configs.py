"""Configurations beyond the golden problems, on the GPU through the package
API (Problem -> GalerkinPlan -> C ABI).

* Elasticity with parallel fibres (Mandel 6x6 stiffness per voxel, 6 load
  cases in one batch, GaNi solve with Ga order-0 postprocessing): a 15^3
  instance against the oracle; the 127^3 configuration through properties
  that hold at any size (symmetry, the Voigt / Reuss and primal / dual bound
  ordering, mixed precision against FP64).
"""
import time

import numpy as np
import pytest

import oracle
from ffthompy_gb300 import workloads

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _relmax(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _fibre_problem(n, tol, precision='f64', seed=0):
    vals = workloads.fibres_coefficient((n, n, n), seed=seed)
    N = np.array([n, n, n])
    return {'name': 'fibres%d' % n, 'physics': 'elasticity',
            'material': workloads.fun_material(vals),
            'solve': {'kind': 'GaNi', 'N': N, 'primaldual': ['primal', 'dual'],
                      'precision': precision},
            'solver': {'kind': 'CG', 'tol': tol, 'maxiter': 1000},
            'postprocess': [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': 0, 'P': N}]}, vals


def _solve(prob):
    from ffthompy_gb300.problem import Problem
    pb = Problem(prob, None)
    t0 = time.perf_counter()
    pb.calculate()
    torch.cuda.synchronize()
    return pb, time.perf_counter() - t0


def test_fibres_elasticity_small_matches_oracle():
    prob, _ = _fibre_problem(15, 1e-8)
    ref = oracle.solve_problem(prob)
    pb, _ = _solve(prob)
    for pd in ('primal', 'dual'):
        got = pb.output['mat_' + pd]
        assert set(got) == set(ref['mat_' + pd])
        for key, AH in ref['mat_' + pd].items():
            assert _relmax(got[key], AH) < 1e-10, (key, _relmax(got[key], AH))
        kits = [r['info']['kit'] for r in pb.output['res_' + pd]]
        kits_ref = [r['kit'] for r in ref['res_' + pd]]
        assert all(abs(a - b) <= 1 for a, b in zip(kits, kits_ref)), (kits, kits_ref)


def _psd_min_eig(M):
    return float(np.linalg.eigvalsh(0.5 * (M + M.T)).min())


def test_fibres_elasticity_127_properties():
    """127^3, 6 loads: bounds ordering, symmetry, mixed precision vs FP64."""
    prob64, vals = _fibre_problem(127, 1e-6, 'f64')
    pb64, t64 = _solve(prob64)
    probm, _ = _fibre_problem(127, 1e-6, 'mixed')
    pbm, tm = _solve(probm)
    kits = [r['info']['kit'] for r in pb64.output['res_primal']]
    print('127^3 fibres: f64 %.2f s, mixed %.2f s, kits %s' % (t64, tm, kits))
    p = pb64.output['mat_primal']
    d = pb64.output['mat_dual']
    scale = np.abs(p['AH_GaNi_primal']).max()
    for M in (p['AH_GaNi_primal'], p['AH_Ga_o0_P127_primal'], d['AH_GaNi_dual']):
        assert np.abs(M - M.T).max() < 1e-8 * scale
    # Voigt >= primal (GaNi and Ga) >= dual >= Reuss in the Loewner order
    C = vals.reshape(6, 6, -1)
    voigt = C.mean(-1)
    reuss = np.linalg.inv(np.linalg.inv(np.moveaxis(C, -1, 0)).mean(0))
    tol = 1e-6 * scale
    assert _psd_min_eig(voigt - p['AH_Ga_o0_P127_primal']) > -tol
    assert _psd_min_eig(p['AH_Ga_o0_P127_primal'] - d['AH_Ga_o0_P127_dual']) > -tol
    assert _psd_min_eig(p['AH_GaNi_primal'] - d['AH_GaNi_dual']) > -tol
    assert _psd_min_eig(d['AH_Ga_o0_P127_dual'] - reuss) > -tol
    # fibre stiffness 10x the matrix: the fibre-direction stiffness exceeds the transverse one
    assert p['AH_GaNi_primal'][2, 2] > p['AH_GaNi_primal'][0, 0]
    # mixed precision: A_H within 1e-6 of the FP64 solve
    for pd in ('primal', 'dual'):
        for key, AH in pb64.output['mat_' + pd].items():
            err = _relmax(pbm.output['mat_' + pd][key], AH)
            assert err < 1e-6, (key, err)


# ---------------------------------------------------------------------------
# coefficient gradient: dA_H / da(x) through torch.autograd
# ---------------------------------------------------------------------------
def _oracle_ah00(a, N, tol=1e-13):
    d = len(N)
    A = np.einsum('ij,...->ij...', np.eye(d), a)
    G, _ = oracle.green_operator('scalar', np.asarray(N), np.ones(d), 'GaNi', 1)
    Afun = lambda v: oracle.apply_GA(G, A, v)
    E = np.zeros((d,) + tuple(N))
    E[0] = 1.
    X, _ = oracle.cg(Afun, Afun(-E), np.zeros_like(E), tol=tol, maxiter=3000)
    return oracle.assembly_matrix(A, [X + E])[0, 0]


def test_gradient_matches_oracle_central_differences():
    """dA_H[0,0]/da(x), exp of a Gaussian random field on 15^3, at 8 voxels."""
    from ffthompy_gb300.adjoint import homogenized_matrix
    N = (15, 15, 15)
    a_np = np.exp(workloads.gaussian_field(N, 0.15, seed=5))
    a = torch.tensor(a_np, device='cuda', requires_grad=True)
    AH = homogenized_matrix(a, tol=1e-12)
    AH[0, 0].backward()
    grad = a.grad.cpu().numpy()
    rng = np.random.default_rng(1)
    for _ in range(8):
        v = tuple(int(rng.integers(n)) for n in N)
        h = 1e-4 * a_np[v]
        ap, am = a_np.copy(), a_np.copy()
        ap[v] += h
        am[v] -= h
        fd = (_oracle_ah00(ap, N) - _oracle_ah00(am, N)) / (2 * h)
        assert abs(fd - grad[v]) < 1e-6 * abs(grad[v]), (v, fd, grad[v])
    # forward value against the oracle as well
    assert abs(float(AH[0, 0]) - _oracle_ah00(a_np, N)) < 1e-11 * abs(float(AH[0, 0]))


def test_gradient_127_matches_gpu_central_differences():
    """127^3 exp-GRF coefficient: gradient vs central differences of the GPU
    A_H[0,0] (one-load FP64 plan) on 8 seeded voxels, step 1e-2 a(x)
    (truncation ~1e-4 relative; FP64 energy roundoff ~1e-7 of the signal)."""
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.adjoint import homogenized_matrix
    from ffthompy_gb300.engine import GalerkinPlan
    N = (127, 127, 127)
    a_np = np.exp(workloads.gaussian_field(N, 0.15, seed=7))
    a = torch.tensor(a_np, device='cuda', requires_grad=True)
    t0 = time.perf_counter()
    AH = homogenized_matrix(a, tol=1e-10)
    AH[0, 0].backward()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    grad = a.grad.cpu().numpy()
    plan = GalerkinPlan(N, np.ones(3), physics='scalar', nloads=1, precision='f64')
    base = torch.tensor(a_np, device='cuda').reshape((1,) + N)

    def ah00(vals):
        plan.set_coefficient_packed(vals, _lib.FHP_COEF_ISO)
        X, info = plan.cg(plan.rhs_macro(1), tol=1e-10, maxiter=2000)
        assert info['status'] == [0]
        return plan.energy(X)[0, 0]

    assert abs(ah00(base) - float(AH[0, 0])) < 1e-10 * abs(float(AH[0, 0]))
    rng = np.random.default_rng(2)
    t0 = time.perf_counter()
    for _ in range(8):
        v = tuple(int(rng.integers(n)) for n in N)
        h = 1e-2 * a_np[v]
        vp = base.clone()
        vp[(0,) + v] += h
        vm = base.clone()
        vm[(0,) + v] -= h
        fd = (ah00(vp) - ah00(vm)) / (2 * h)
        assert abs(fd - grad[v]) < 2e-3 * abs(grad[v]), (v, fd, grad[v])
    print('127^3 gradient %.2f s (forward + backward); 16 FD solves %.2f s'
          % (t_grad, time.perf_counter() - t0))


def test_gradient_127_mixed_64_voxels_within_1e4():
    """The adjoint configuration as specified: a(x) = exp(g(x)) on 127^3
    (g a seeded Gaussian random field, length 0.15), dA_H[0,0]/da(x) from
    the mixed-precision solve (FP32 inner CG, FP64 refinement) through
    torch.autograd, against central differences of the mixed-precision
    A_H[0,0] (one-load plan, same tolerance) on 64 seeded voxels with step
    1e-3 a(x): truncation ~1e-6 relative, so the bar is 1e-4."""
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.adjoint import homogenized_matrix
    from ffthompy_gb300.engine import GalerkinPlan
    N = (127, 127, 127)
    a_np = np.exp(workloads.gaussian_field(N, 0.15, seed=11))
    a = torch.tensor(a_np, device='cuda', requires_grad=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    AH = homogenized_matrix(a, tol=1e-10, precision='mixed')
    AH[0, 0].backward()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    grad = a.grad.cpu().numpy()
    plan = GalerkinPlan(N, np.ones(3), physics='scalar', nloads=1, precision='mixed')
    base = torch.tensor(a_np, device='cuda').reshape((1,) + N)

    def ah00(vals):
        plan.set_coefficient_packed(vals, _lib.FHP_COEF_ISO)
        X, info = plan.cg(plan.rhs_macro(1), tol=1e-10, maxiter=2000)
        assert info['status'] == [0]
        return plan.energy(X)[0, 0]

    assert abs(ah00(base) - float(AH[0, 0])) < 1e-10 * abs(float(AH[0, 0]))
    rng = np.random.default_rng(64)
    worst = 0.
    for _ in range(64):
        v = tuple(int(rng.integers(n)) for n in N)
        h = 1e-3 * a_np[v]
        vp = base.clone()
        vp[(0,) + v] += h
        vm = base.clone()
        vm[(0,) + v] -= h
        fd = (ah00(vp) - ah00(vm)) / (2 * h)
        err = abs(fd - grad[v]) / abs(grad[v])
        worst = max(worst, err)
        assert err < 1e-4, (v, fd, grad[v])
    print('127^3 mixed gradient %.2f s (forward + backward); worst FD error %.2e'
          % (t_grad, worst))


def test_gradient_elasticity_packed_matches_central_differences():
    """Mandel 6x6 packed (SYM) coefficient, 6 loads, general adjoint seed W."""
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.engine import GalerkinPlan, pack_coefficient
    N = (9, 9, 9)
    vals = workloads.fibres_coefficient(N, n_fibres=2, radius=0.2, min_dist=0.45, seed=3)
    packed = pack_coefficient(vals, _lib.FHP_COEF_SYM)
    plan = GalerkinPlan(N, np.ones(3), physics='elasticity', precision='f64')
    rng = np.random.default_rng(4)
    W = rng.standard_normal((6, 6))

    def solve(p):
        plan.set_coefficient_packed(p, _lib.FHP_COEF_SYM)
        X, info = plan.cg(plan.rhs_macro(1), tol=1e-12, maxiter=3000)
        return X, float(np.sum(W * plan.energy(X)))

    X, _ = solve(packed)
    grad = plan.energy_gradient(X, W).cpu().numpy()
    for _ in range(6):
        t = int(rng.integers(packed.shape[0]))
        v = tuple(int(rng.integers(n)) for n in N)
        # step 1e-3 of the entry (or of 1e-2 for zero couplings): truncation
        # ~1e-6 relative, FP64 energy roundoff ~1e-9 absolute in the quotient
        h = 1e-3 * max(abs(packed[(t,) + v]), 1e-2)
        pp, pm = packed.copy(), packed.copy()
        pp[(t,) + v] += h
        pm[(t,) + v] -= h
        fd = (solve(pp)[1] - solve(pm)[1]) / (2 * h)
        g = grad[(t,) + v]
        assert abs(fd - g) < 1e-5 * abs(g) + 1e-8, (t, v, fd, g)


# ---------------------------------------------------------------------------
# ensembles of independent 2D cells (thresholded Gaussian random fields)
# ---------------------------------------------------------------------------
def _grf_instances(count, sizes, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        contrast = float(np.exp(rng.uniform(np.log(2.), np.log(1000.))))
        out.append(workloads.grf_phase_coefficient((n, n), ell=0.1, quantile=0.4,
                                                   contrast=contrast,
                                                   seed=int(rng.integers(1 << 30))))
    return out


def test_batched_2d_instances_match_oracle():
    from ffthompy_gb300.batch import homogenize_many
    coefs = _grf_instances(10, [15, 21, 33, 63], seed=11)
    res = homogenize_many(coefs, tol=1e-8, primaldual=('primal', 'dual'), workers=4)
    for A, r in zip(coefs, res):
        N = np.array(A.shape[2:])
        prob = {'physics': 'scalar', 'material': workloads.fun_material(A),
                'solve': {'kind': 'GaNi', 'N': N, 'primaldual': ['primal', 'dual']},
                'solver': {'tol': 1e-8, 'maxiter': 1000}, 'postprocess': [{'kind': 'GaNi'}]}
        ref = oracle.solve_problem(prob)
        assert _relmax(r['primal'], ref['mat_primal']['AH_GaNi_primal']) < 1e-10
        assert _relmax(r['dual'], ref['mat_dual']['AH_GaNi_dual']) < 1e-10
        for pd in ('primal', 'dual'):
            # contrast up to 1000: long CG runs drift by a few % under different
            # (equally accurate) FFT roundoff, as in the band-mode golden checks
            kr = [x['kit'] for x in ref['res_' + pd]]
            assert all(abs(a - b) <= max(1, int(0.02 * b)) for a, b in zip(r['kit_' + pd], kr)), \
                (r['kit_' + pd], kr)


def test_batched_2d_ensemble_512():
    """512 instances, n in {63, 127, 255, 511}, contrast log-uniform in
    [2, 1000], 2 loads each, FP64 to tol 1e-6: every instance converges and
    its A_H lies between the Reuss and Voigt bounds."""
    from ffthompy_gb300.batch import homogenize_many
    coefs = _grf_instances(512, [63, 127, 255, 511], seed=12)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = homogenize_many(coefs, tol=1e-6, workers=16)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    vox_it = sum(int(np.prod(A.shape[2:])) * sum(r['kit_primal']) for A, r in zip(coefs, res))
    print('512 instances, %.1f Mvoxels: %.2f s, %.0f Mvoxel-iter/s'
          % (sum(np.prod(A.shape[2:]) for A in coefs) / 1e6, dt, vox_it / dt / 1e6))
    for A, r in zip(coefs, res):
        assert r['status_primal'] == [0, 0]
        a = A[0, 0]
        voigt, reuss = a.mean(), 1. / (1. / a).mean()
        AH = r['primal']
        assert abs(AH[0, 1] - AH[1, 0]) < 1e-10 * abs(AH).max()
        ev = np.linalg.eigvalsh(0.5 * (AH + AH.T))
        assert ev.min() > reuss * (1 - 1e-8) and ev.max() < voigt * (1 + 1e-8), (ev, reuss, voigt)


@pytest.mark.parametrize('precision', ['f64', 'f32', 'mixed'])
def test_cg_many_equals_single_plan_solves(precision):
    """fhp_cg_solve_many (all cells of an ensemble advanced together, one CUDA
    graph per iteration) runs each cell's own CG: the same iteration counts,
    statuses and solutions as one fhp_cg_solve per cell, on cells of three
    grid sizes and both projections."""
    from ffthompy_gb300.engine import GalerkinPlan, cg_many
    coefs = _grf_instances(9, [15, 31, 64], seed=3)
    for proj in (1, 2):
        plans_a = [GalerkinPlan(A.shape[2:], np.ones(2), precision=precision) for A in coefs]
        plans_b = [GalerkinPlan(A.shape[2:], np.ones(2), precision=precision) for A in coefs]
        for A, pa, pb in zip(coefs, plans_a, plans_b):
            pa.set_coefficient(A)
            pb.set_coefficient(A)
        tol = 1e-5 if precision == 'f32' else 1e-9
        many = cg_many(plans_a, [p.rhs_macro(proj) for p in plans_a], tol=tol, maxiter=400,
                       proj=proj)
        for (X, info), pb in zip(many, plans_b):
            Xb, ib = pb.cg(pb.rhs_macro(proj), tol=tol, maxiter=400, proj=proj)
            assert info['kit'] == ib['kit'], (info['kit'], ib['kit'])
            assert info['status'] == ib['status']
            d = float((X - Xb).abs().max()) / max(float(Xb.abs().max()), 1e-300)
            assert d < (1e-12 if precision != 'f32' else 1e-6), d


def test_batched_and_threaded_ensembles_agree():
    """homogenize_many's batched mode (one fhp_cg_solve_many over the
    ensemble) and its thread-pool mode give the same per-cell A_H."""
    from ffthompy_gb300.batch import homogenize_many
    coefs = _grf_instances(12, [31, 63, 127], seed=21)
    a = homogenize_many(coefs, tol=1e-8, primaldual=('primal', 'dual'), mode='batched')
    b = homogenize_many(coefs, tol=1e-8, primaldual=('primal', 'dual'), mode='threads',
                        workers=4)
    for ra, rb in zip(a, b):
        for pd in ('primal', 'dual'):
            assert ra['kit_' + pd] == rb['kit_' + pd]
            assert np.abs(ra[pd] - rb[pd]).max() < 1e-12 * np.abs(rb[pd]).max()


def _spd_field(dv, N, rng):
    """A symmetric positive definite (dv, dv) + N coefficient with varying
    eigenvalues (full-kind packing for dv > 1)."""
    B = 0.3 * rng.standard_normal((dv, dv) + N)
    A = np.einsum('ik...,jk...->ij...', B, B)
    for i in range(dv):
        A[i, i] += 1.0 + 9.0 * rng.random(N)
    return A


def _cell_cases(case, rng):
    if case == '2d':       # same size, contrasts 2..1000: different iteration counts
        return 'scalar', _grf_instances(5, [33], seed=4)
    if case == '3d':
        return 'scalar', [_spd_field(3, (15, 15, 15), rng) for _ in range(3)]
    return 'elasticity', [_spd_field(6, (9, 9, 9), rng) for _ in range(2)]


@pytest.mark.parametrize('precision', ['f64', 'f32', 'mixed'])
@pytest.mark.parametrize('case', ['2d', '3d', 'elast'])
def test_cell_plan_equals_single_cell_plans(case, precision):
    """A plan of several cells of one grid (fhp_plan_create_cells: every pass
    one launch for all cells) runs each cell's own CG: per cell the same
    iteration counts, statuses, solutions and A_H as a plan of that cell
    alone, for both projections; 2D and 3D scalar, 3D elasticity."""
    from ffthompy_gb300.engine import GalerkinPlan, coef_kind_of, pack_coefficient
    rng = np.random.default_rng(7)
    physics, coefs = _cell_cases(case, rng)
    N = coefs[0].shape[2:]
    K = len(coefs)
    Y = np.ones(len(N))
    kind = max(coef_kind_of(A) for A in coefs)
    vals = np.stack([pack_coefficient(A, kind) for A in coefs])
    tol = 1e-5 if precision == 'f32' else 1e-9
    cells = GalerkinPlan(N, Y, physics=physics, precision=precision, ncells=K)
    assert int(cells.lib.fhp_plan_cells(cells.handle)) == K
    cells.set_coefficient_packed(vals, kind)
    singles = [GalerkinPlan(N, Y, physics=physics, precision=precision) for _ in coefs]
    for p, v in zip(singles, vals):
        p.set_coefficient_packed(v, kind)
    L = cells.nloads
    for proj in (1, 2):
        b = cells.rhs_macro(proj)
        assert tuple(b.shape) == (K, L, cells.dv) + tuple(N)
        X, info = cells.cg(b, tol=tol, maxiter=600, proj=proj)
        AH = cells.energy(X)
        assert AH.shape == (K, L, L)
        for k, p in enumerate(singles):
            bk = p.rhs_macro(proj)
            assert float((b[k] - bk).abs().max()) <= 1e-12 * float(bk.abs().max())
            Xk, ik = p.cg(bk, tol=tol, maxiter=600, proj=proj)
            assert info['kit'][k * L:(k + 1) * L] == ik['kit'], (k, info['kit'], ik['kit'])
            assert info['status'][k * L:(k + 1) * L] == ik['status']
            d = float((X[k] - Xk).abs().max()) / max(float(Xk.abs().max()), 1e-300)
            assert d < (1e-6 if precision == 'f32' else 1e-12), (k, d)
            AHk = p.energy(Xk)
            assert np.abs(AH[k] - AHk).max() <= (1e-6 if precision == 'f32' else 1e-12) * \
                np.abs(AHk).max()
    if case == '2d':
        kits = [info['kit'][k * L] for k in range(K)]
        assert len(set(kits)) > 1, kits      # the cells stopped at different iterations


def test_cells_mode_matches_threads():
    """homogenize_many(mode='cells') - one plan of several cells per grid size,
    the sizes advanced together - gives each cell the A_H and iteration counts
    of the thread-pool mode, primal and dual."""
    from ffthompy_gb300.batch import homogenize_many
    coefs = _grf_instances(14, [31, 63, 127], seed=21)
    a = homogenize_many(coefs, tol=1e-8, primaldual=('primal', 'dual'), mode='cells')
    b = homogenize_many(coefs, tol=1e-8, primaldual=('primal', 'dual'), mode='threads',
                        workers=4)
    # the launch shapes are tuned per plan (cells or single), so reductions
    # may group differently: equally accurate roundoff, a few % of the
    # iteration count at contrast 1000
    for ra, rb in zip(a, b):
        for pd in ('primal', 'dual'):
            assert all(abs(x - y) <= max(1, int(0.02 * y))
                       for x, y in zip(ra['kit_' + pd], rb['kit_' + pd])), \
                (ra['kit_' + pd], rb['kit_' + pd])
            assert ra['status_' + pd] == [0, 0]
            assert np.abs(ra[pd] - rb[pd]).max() < 1e-10 * np.abs(rb[pd]).max()
