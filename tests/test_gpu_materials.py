"""GPU material assembly against the oracle (the NumPy restatement of the
reference): ball characteristic functions (fhp_ball_characteristic; the
reference's get_weights_circ, get_shift_inclusion and centred inverse DFT,
ffthompy/materials.py:125-169, 317-330, 392-425), GaNi topologies of balls,
boxes and pyramids (fhp_ball_topology, fhp_separable_char;
materials.py:212-301), separable Ga characteristic functions of boxes and
pyramids, the sums over inclusions and the reference's own problems.

Bars: ball and box topologies bit-identical (their values are sums of 0/1
indicators); pyramid topologies within 1e-15 (a product of per-axis image
sums against a sum of products); characteristic functions within 1e-11 of
their maximum (CUDA's j1 against scipy's jv, and transforms of different
summation order); coefficients of the golden problems within 1e-12.
"""
import numpy as np
import pytest

import golden_io
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

CHAR_TOL = 1e-11


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _balls(d, pos, rads, Y):
    n = len(rads)
    return {'inclusions': ['ball'] * n + ['otherwise'],
            'positions': [np.asarray(p, dtype=np.float64) for p in pos] + [''],
            'params': list(rads) + [''],
            'vals': [(10. + 5 * i) * np.eye(d) for i in range(n)] + [np.eye(d)],
            'Y': np.asarray(Y, dtype=np.float64), 'order': None}


CASES = [
    ('2d_centred', 2, [(0., 0.)], [0.5], (1., 1.), (9, 9)),
    ('2d_offset_aniso', 2, [(0.1, -0.2)], [0.4], (1., 2.), (31, 45)),
    ('2d_two_balls', 2, [(-0.25, -0.25), (0.25, 0.2)], [0.3, 0.2], (1., 1.), (63, 63)),
    ('3d_offset', 3, [(0.1, 0.2, -0.3)], [0.35], (1., 1., 1.), (15, 17, 13)),
    ('3d_two_balls', 3, [(-0.2, 0., 0.), (0.25, 0.1, 0.)], [0.3, 0.25], (1., 1.5, 1.), (33, 29, 31)),
]


@pytest.mark.parametrize('name,d,pos,rads,Y,N', CASES, ids=[c[0] for c in CASES])
def test_ball_characteristic_matches_oracle(name, d, pos, rads, Y, N):
    from ffthompy_gb300.materials import Material
    conf = _balls(d, pos, rads, Y)
    gpu = Material(dict(conf)).get_shape_functions(np.array(N))
    ref = oracle.Material(dict(conf)).shape_functions(np.array(N))
    for g, h in zip(gpu, ref):
        err = np.abs(g - h).max() / max(np.abs(h).max(), 1e-300)
        assert err < CHAR_TOL, (name, err)


@pytest.mark.parametrize('name,d,pos,rads,Y,N', CASES, ids=[c[0] for c in CASES])
def test_ball_topology_bit_identical(name, d, pos, rads, Y, N):
    from ffthompy_gb300.materials import Material
    conf = _balls(d, pos, rads, Y)
    for Ng in (N, tuple(n + 1 for n in N)):     # odd and even grids
        gpu = Material(dict(conf)).get_A_GaNi(np.array(Ng), 'primal').val
        ref = oracle.Material(dict(conf)).get_A_GaNi(np.array(Ng), 'primal')
        np.testing.assert_array_equal(gpu, ref)


def test_ball_coefficients_match_oracle():
    """Ga (order None) and GaNi coefficients of ball materials against the
    oracle's restatement of the reference."""
    from ffthompy_gb300.materials import Material
    for name, d, pos, rads, Y, N in CASES[1:4]:
        conf = _balls(d, pos, rads, Y)
        Nbar = np.array(N)
        ours = Material(dict(conf)).get_A_Ga(Nbar, 'primal', order=None).val
        ref = oracle.Material(dict(conf)).get_A_Ga(Nbar, 'primal', order=None)
        assert np.abs(ours - ref).max() <= CHAR_TOL * 20 * np.abs(ref).max(), name
        Ng = np.array([(n + 1) // 2 for n in N])
        ours = Material(dict(conf)).get_A_GaNi(Ng, 'primal').val
        ref = oracle.Material(dict(conf)).get_A_GaNi(Ng, 'primal')
        np.testing.assert_allclose(ours, ref, rtol=0, atol=1e-14)


def test_reference_ball_problem_through_gpu_assembly():
    """The reference's own 2D ball problem (Ga solve, Ga bounds) with its
    coefficients assembled on the GPU: A_H as stored by the reference."""
    from ffthompy_gb300.problem import Problem
    prob, exp = golden_io.problem('ref_scalar_2d_prob5')
    pb = Problem(prob, None)
    pb.calculate()
    assert exp['mat']
    for pd, mats in exp['mat'].items():
        for key, val in mats.items():
            got = pb.output['mat_' + pd][key]
            assert np.abs(got - val).max() <= 1e-9 * np.abs(val).max(), (pd, key)


def _boxes(d):
    return {'inclusions': ['cube', 'pyramid', 'otherwise'],
            'positions': [np.full(d, -0.2), np.full(d, 0.25), ''],
            'params': [np.full(d, 0.3), np.full(d, 0.35), ''],
            'vals': [np.eye(d) * 7. + 1., np.diag(np.arange(1., d + 1.)) * 3., np.eye(d)],
            'Y': np.ones(d), 'order': None}


@pytest.mark.parametrize('d,N', [(2, (31, 45)), (3, (15, 17, 13)), (2, (30, 44))])
def test_box_pyramid_assembly_matches_oracle(d, N):
    """Boxes, pyramids and 'otherwise': GaNi topologies (per-axis image sums
    multiplied on the GPU) and Ga coefficients (per-axis transforms
    multiplied on the GPU, summed over the inclusions there), primal and
    dual, 2D and 3D, odd and even grids."""
    from ffthompy_gb300.materials import Material
    conf = _boxes(d)
    for pd in ('primal', 'dual'):
        got = Material(dict(conf)).get_A_GaNi(np.array(N), pd).val
        ref = oracle.Material(dict(conf)).get_A_GaNi(np.array(N), pd)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-15 * np.abs(ref).max())
        if all(n % 2 for n in N):
            got = Material(dict(conf)).get_A_Ga(np.array(N), pd, order=None).val
            ref = oracle.Material(dict(conf)).get_A_Ga(np.array(N), pd, order=None)
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_elasticity_inclusion_sum_36_values():
    """A 3D elasticity material (6 x 6 Mandel values, nv = 36 in
    fhp_outer_accumulate) with a ball and a box: Ga (order None) and GaNi
    against the oracle."""
    from ffthompy_gb300.materials import Material
    C1 = oracle.mandel_isotropic(1., 0.5)
    C2 = oracle.mandel_isotropic(8., 3.)
    conf = {'inclusions': ['ball', 'cube', 'otherwise'],
            'positions': [np.array([0.1, -0.1, 0.2]), np.array([-0.3, 0.25, -0.2]), ''],
            'params': [0.4, np.array([0.2, 0.3, 0.25]), ''],
            'vals': [C2, 0.5 * (C1 + C2), C1], 'Y': np.ones(3), 'order': None}
    N = np.array([15, 13, 17])
    for pd in ('primal', 'dual'):
        got = Material(dict(conf)).get_A_Ga(N, pd, order=None).val
        ref = oracle.Material(dict(conf)).get_A_Ga(N, pd, order=None)
        assert np.abs(got - ref).max() <= CHAR_TOL * 20 * np.abs(ref).max()
        got = Material(dict(conf)).get_A_GaNi(N, pd).val
        ref = oracle.Material(dict(conf)).get_A_GaNi(N, pd)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14 * np.abs(ref).max())


def test_materials_match_oracle():
    """Coefficient assembly of the golden problems (GaNi, Ga of their order,
    and the postprocess kinds) against the oracle restatement."""
    from ffthompy_gb300.materials import Material
    for name in golden_io.names('ref_') + ['run_cfg1_square45', 'run_s3_ga_7', 'run_e3_gani_5']:
        prob, _ = golden_io.problem(name)
        N = np.asarray(prob['solve']['N'])
        for pd in prob['solve']['primaldual']:
            m1 = Material(dict(prob['material']))
            m2 = oracle.Material(dict(prob['material']))
            np.testing.assert_allclose(m1.get_A_GaNi(N, pd).val, m2.get_A_GaNi(N, pd),
                                       rtol=0, atol=1e-12)
            if 'order' in prob['material']:
                got = m1.get_A_Ga(2 * N - 1, pd).val
                ref = m2.get_A_Ga(2 * N - 1, pd)
                np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
            for pp in prob['postprocess']:
                if pp.get('order', -1) in (None, 0, 1) and 'order' in pp:
                    P = pp.get('P')
                    got = m1.get_A_Ga(2 * N - 1, pd, order=pp['order'], P=P).val
                    ref = m2.get_A_Ga(2 * N - 1, pd, order=pp['order'], P=P)
                    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
