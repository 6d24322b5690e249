"""GPU material assembly for ball inclusions against the host restatement and
the oracle: the Ga characteristic function (fhp_ball_characteristic; the
reference's get_weights_circ, get_shift_inclusion and centred inverse DFT,
ffthompy/materials.py:125-169, 317-330, 392-425) and the GaNi topology
(fhp_ball_topology; materials.py:212-301).

Bars: topologies bit-identical; characteristic functions within 1e-11 of
their maximum (the GPU evaluates J1 with CUDA's j1, the host with scipy's jv,
and the transforms differ in summation order).
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


def _host(monkeypatch, fn):
    import ffthompy_gb300.materials as M
    with monkeypatch.context() as m:
        m.setattr(M, '_gpu_available', lambda: False)
        return fn()


@pytest.mark.parametrize('name,d,pos,rads,Y,N', CASES, ids=[c[0] for c in CASES])
def test_ball_characteristic_matches_host(monkeypatch, name, d, pos, rads, Y, N):
    from ffthompy_gb300.materials import Material
    conf = _balls(d, pos, rads, Y)
    gpu = Material(dict(conf)).get_shape_functions(np.array(N))
    host = _host(monkeypatch, lambda: Material(dict(conf)).get_shape_functions(np.array(N)))
    for g, h in zip(gpu, host):
        err = np.abs(g - h).max() / max(np.abs(h).max(), 1e-300)
        assert err < CHAR_TOL, (name, err)


@pytest.mark.parametrize('name,d,pos,rads,Y,N', CASES, ids=[c[0] for c in CASES])
def test_ball_topology_bit_identical(monkeypatch, name, d, pos, rads, Y, N):
    from ffthompy_gb300.materials import Material
    conf = _balls(d, pos, rads, Y)
    for Ng in (N, tuple(n + 1 for n in N)):     # odd and even grids
        gpu = Material(dict(conf)).get_A_GaNi(np.array(Ng), 'primal').val
        host = _host(monkeypatch, lambda: Material(dict(conf)).get_A_GaNi(np.array(Ng), 'primal').val)
        np.testing.assert_array_equal(gpu, host)


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


def test_inclusion_sum_on_gpu_is_bit_identical(monkeypatch):
    """Material.get_A_Ga (order None): the sum over inclusions on the GPU
    (fhp_outer_accumulate) equals the host sum bit for bit when the
    characteristic functions are the same (boxes, pyramids and 'otherwise',
    whose transforms are host code), primal and dual, 2D and 3D."""
    from ffthompy_gb300.materials import Material
    for d, N in ((2, (31, 45)), (3, (15, 17, 13))):
        conf = {'inclusions': ['cube', 'pyramid', 'otherwise'],
                'positions': [np.full(d, -0.2), np.full(d, 0.25), ''],
                'params': [np.full(d, 0.3), np.full(d, 0.35), ''],
                'vals': [np.eye(d) * 7. + 1., np.diag(np.arange(1., d + 1.)) * 3., np.eye(d)],
                'Y': np.ones(d), 'order': None}
        for pd in ('primal', 'dual'):
            gpu = Material(dict(conf)).get_A_Ga(np.array(N), pd, order=None).val
            host = _host(monkeypatch,
                         lambda: Material(dict(conf)).get_A_Ga(np.array(N), pd, order=None).val)
            np.testing.assert_array_equal(gpu, host)
