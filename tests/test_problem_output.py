"""Problem.postprocessing output file in the reference's layout
(ffthompy/problem.py:98-126): a protocol-3 pickle of Problem.output plus the
problem definition, with mat_<pd> dicts of homogenised matrices, sol_<pd>
lists of Tensors and res_<pd> lists of {'cb': CallBack, 'info': {...}}.  A
downstream script reads it as the reference's run_unittests.py:46-64 reads
its golden pickles: res['mat_' + pd][key].
"""
import os
import pickle
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import golden_io  # noqa: E402

torch = pytest.importorskip('torch')


def test_tensor_pickles_through_host_values():
    from ffthompy_gb300.tensors.objects import Tensor
    t = Tensor(name='X+E', val=np.arange(24.).reshape(2, 3, 4), order=1, Y=[1., 2.])
    u = pickle.loads(pickle.dumps(t, protocol=3))
    assert isinstance(u.val, np.ndarray) and np.array_equal(u.val, t.val)
    assert (u.name, u.order, u.N) == (t.name, t.order, t.N)
    assert np.array_equal(u.Y, t.Y)


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['ref_scalar_2d_prob1', 'ref_linelas_3d_prob1'])
def test_postprocessing_pickle_has_the_reference_layout(name, tmp_path):
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()
    from ffthompy_gb300.problem import Problem
    prob, exp = golden_io.problem(name)
    prob['save'] = {'filename': str(tmp_path / 'out' / name)}
    pb = Problem(prob, None)
    pb.calculate()
    pb.postprocessing()
    with open(prob['save']['filename'], 'rb') as f:
        res = pickle.load(f)
    for key in ('physics', 'solve', 'solver', 'postprocess', 'save', 'material'):
        assert key in res, key
    for pd in pb.solve['primaldual']:
        # the reference's consumer: res['mat_' + pd][kw] for every kw computed
        assert set(res['mat_' + pd]) == set(exp['mat'][pd])
        for kw, ref in exp['mat'][pd].items():
            assert np.abs(res['mat_' + pd][kw] - ref).max() < 1e-10 * np.abs(ref).max()
        sols = res['sol_' + pd]
        assert len(sols) == len(exp['kit'][pd])
        for s in sols:
            assert isinstance(s.val, np.ndarray) and s.val.ndim == 1 + len(pb.solve['N'])
        kits = [r['info']['kit'] for r in res['res_' + pd]]
        assert kits == [int(k) for k in pb_kits(pb, pd)]
        assert all(len(r['cb'].res_norm) == r['info']['kit'] + 1 for r in res['res_' + pd])


def pb_kits(pb, pd):
    return [r['info']['kit'] for r in pb.output['res_' + pd]]
