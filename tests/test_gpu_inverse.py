"""GPU parity of the per-voxel coefficient inverse (fhp_coefficient_inverse)
with the reference's get_inverse (ffthompy/trigpol.py:120-159; fixtures
tests/golden/inv_*.npz) and with the oracle at larger sizes.

Bar: bit-identical (np.testing.assert_array_equal, Inf / NaN in the same
places) - the kernel rounds each product and difference as NumPy does.
"""
import warnings

import numpy as np
import pytest

import golden_io
import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

INV = golden_io.names('inv_')


@pytest.fixture(scope='module', autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import __graft_entry__
    __graft_entry__.build()


def _oracle_inv(A):
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return oracle.get_inverse(A)


def _field(rng, d, N, sym=True):
    A = rng.standard_normal((d, d) + N)
    if sym:
        A = 0.5 * (A + np.swapaxes(A, 0, 1))
    return A + np.einsum('ij,...->ij...', d * np.eye(d), np.ones(N))


@pytest.mark.parametrize('name', INV)
def test_inverse_matches_reference_bit_for_bit(name):
    from ffthompy_gb300.engine import coefficient_inverse
    _, arr = golden_io.load(name)
    out = coefficient_inverse(arr['A']).cpu().numpy()
    np.testing.assert_array_equal(out, arr['inv'])


@pytest.mark.parametrize('d,N', [(1, (33,)), (2, (64, 45)), (3, (31, 32, 17)),
                                 (4, (9, 130)), (5, (7, 6, 129)), (6, (20, 21, 22))])
@pytest.mark.parametrize('shift', [False, True])
def test_inverse_matches_oracle_with_and_without_shift(d, N, shift):
    from ffthompy_gb300.engine import coefficient_inverse
    rng = np.random.default_rng(d * 100 + len(N))
    A = _field(rng, d, N, sym=(d % 2 == 0))
    ref = _oracle_inv(A)
    if shift:
        ref = np.fft.ifftshift(ref, axes=tuple(range(2, 2 + len(N))))
    out = coefficient_inverse(A, shift=shift).cpu().numpy()
    np.testing.assert_array_equal(out, ref)


def test_inverse_large_grid_round_trip():
    """Mandel 6 x 6 elasticity coefficients on 128^3 (4.7e8 bytes each way):
    A^-1 A = I to 1e-12 on a sample of voxels, and the sampled voxels
    bit-identical to the oracle."""
    from ffthompy_gb300.engine import coefficient_inverse
    g = torch.Generator(device='cuda').manual_seed(3)
    N = (128, 128, 128)
    R = torch.randn((6, 6) + N, dtype=torch.float64, device='cuda', generator=g)
    A = 0.5 * (R + R.transpose(0, 1)) + 6. * torch.eye(6, dtype=torch.float64,
                                                        device='cuda').reshape(6, 6, 1, 1, 1)
    Ai = coefficient_inverse(A)
    idx = torch.randint(0, 128, (3, 512), generator=g, device='cuda')
    a = A[:, :, idx[0], idx[1], idx[2]].permute(2, 0, 1)
    ai = Ai[:, :, idx[0], idx[1], idx[2]].permute(2, 0, 1)
    err = (torch.bmm(ai, a) - torch.eye(6, dtype=torch.float64, device='cuda')).abs().max()
    assert float(err) < 1e-12
    an = A[:, :, idx[0], idx[1], idx[2]].cpu().numpy()
    np.testing.assert_array_equal(ai.permute(1, 2, 0).cpu().numpy(), _oracle_inv(an))


def test_dual_coefficients_of_materials_match_oracle():
    """Material.get_A_GaNi(dual) (inverse + origin shift in one launch) and the
    grid-based Ga dual (inverse on the P grid, then the Ga assembly) against
    the oracle's host assembly."""
    from ffthompy_gb300.materials import Material
    prob, _ = golden_io.problem('run_e3_gani_5')
    mat = dict(prob['material'])
    N = np.asarray(prob['solve']['N'])
    ours = Material(dict(mat)).get_A_GaNi(N, 'dual').val
    ref = oracle.Material(dict(mat)).get_A_GaNi(N, 'dual')
    np.testing.assert_allclose(ours, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    d = 3
    rng = np.random.default_rng(8)
    vals = _field(rng, d, (15, 15, 15))
    conf = {'fun': lambda coord: vals.copy(), 'Y': np.ones(d), 'order': 0, 'P': np.array([15] * 3)}
    Nbar = np.array([9, 9, 9])
    ours = Material(dict(conf)).get_A_Ga(Nbar, 'dual', order=0, P=np.array([15] * 3)).val
    ref = oracle.Material(dict(conf)).get_A_Ga(Nbar, 'dual', order=0, P=np.array([15] * 3))
    np.testing.assert_allclose(ours, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_tensor_inv_and_batch_dual():
    from ffthompy_gb300.batch import homogenize_many
    from ffthompy_gb300.tensors.objects import Tensor
    rng = np.random.default_rng(4)
    A = _field(rng, 2, (15, 16))
    T = Tensor(name='A', val=A, order=2, multype=21)
    np.testing.assert_array_equal(T.inv().val, _oracle_inv(A))
    a = 1. + 9. * (rng.random((15, 15)) < 0.4)
    Aiso = np.einsum('ij,...->ij...', np.eye(2), a)
    host, dev = homogenize_many([Aiso, torch.from_numpy(Aiso)], tol=1e-10,
                                primaldual=('primal', 'dual'))
    # GaNi primal and dual energies coincide up to the CG tolerance on one grid
    for r in (host, dev):
        np.testing.assert_allclose(r['dual'], r['primal'], rtol=1e-7)
    np.testing.assert_allclose(host['dual'], dev['dual'], rtol=1e-12)
    np.testing.assert_allclose(host['primal'], dev['primal'], rtol=1e-12)
