"""Pin the CPU oracle against the reference's golden data (no GPU)."""
import numpy as np
import pytest

import golden_io
import oracle

PROBLEMS = golden_io.names('ref_') + golden_io.names('run_')
OPS = golden_io.names('op_')


@pytest.mark.parametrize('name', PROBLEMS)
def test_oracle_problem_matches_reference(name):
    prob, exp = golden_io.problem(name)
    out = oracle.solve_problem(prob)
    for pd, mats in exp['mat'].items():
        assert set(out['mat_' + pd]) == set(mats)
        for key, ref in mats.items():
            got = out['mat_' + pd][key]
            # run_unittests.py:61-64 compares at delta 1e-9 (inf-norm)
            assert np.abs(got - ref).max() <= 1e-9 * max(1., np.abs(ref).max()), key
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), key
        kits = [r['kit'] for r in out['res_' + pd]]
        np.testing.assert_array_equal(kits, exp['kit'][pd])
        sol = np.stack(out['sol_' + pd])
        if name.startswith('ref_'):
            # the pickled solutions were stored with a centred origin
            sol = np.fft.fftshift(sol, axes=tuple(range(2, sol.ndim)))
        np.testing.assert_allclose(sol, exp['sol'][pd], rtol=0, atol=1e-9)


@pytest.mark.parametrize('name', OPS)
def test_oracle_operator_matches_reference(name):
    meta, arr = golden_io.load(name)
    for ip in (1, 2):
        G, Ns = oracle.green_operator(meta['physics'], np.array(meta['N']),
                                      np.array(meta['Y']), meta['kind'], ip)
        assert tuple(Ns) == tuple(meta['Nbar'])
        y = oracle.apply_GA(G, arr['A'], arr['x'])
        ref = arr['y%d' % ip]
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()


def test_projection_idempotent_orthogonal():
    """unittest_operators.py:177-203: P*P = P and G1*G2 = 0 (odd N, 2D/3D)."""
    for physics in ('scalar', 'elasticity'):
        for N in ([5, 5], [5, 7, 9]):
            N = np.array(N)
            Y = np.ones(N.size)
            fn = oracle.projection_scalar if physics == 'scalar' else oracle.projection_elasticity
            G1, G2 = fn(N, Y)
            mm = lambda a, b: np.einsum('ij...,jk...->ik...', a, b)
            assert np.abs(mm(G1, G1) - G1).max() < 1e-13
            assert np.abs(mm(G2, G2) - G2).max() < 1e-13
            assert np.abs(mm(G1, G2)).max() < 1e-13


def test_cfg1_known_values():
    """Config-1 values quoted from the reference run (2D GaNi 45^2)."""
    prob, exp = golden_io.problem('run_cfg1_square45')
    m = exp['mat']
    assert abs(m['primal']['AH_GaNi_primal'][0, 0] - 1.901848083527682) < 1e-12
    assert abs(m['primal']['AH_Ga_primal'][0, 0] - 1.979683324453124) < 1e-12
    assert abs(m['dual']['AH_Ga_dual'][0, 0] - 1.8847530656481177) < 1e-12
    np.testing.assert_array_equal(exp['kit']['primal'], [25, 25])
    np.testing.assert_array_equal(exp['kit']['dual'], [22, 22])


def test_project_interpolates_nodes():
    """unittest_tensors.py:29-51: projection to 2N keeps the nodal values."""
    rng = np.random.default_rng(0)
    for N in ([5, 5], [4, 6], [5, 4, 3]):
        x = rng.standard_normal((1,) + tuple(N))
        M = 2 * np.array(N)
        xm = oracle.project(x, M)
        sl = (slice(None),) + tuple(slice(0, m, 2) for m in M)
        np.testing.assert_allclose(xm[sl], x, atol=1e-12)
