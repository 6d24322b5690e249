"""Ensemble cells split across ranks (ffthompy_gb300/partition.py) on CPU.

Two gloo ranks on 127.0.0.1 split an ensemble of small 2D cells, each rank
solves its share, and rank 0 gathers the per-cell A_H.  The cell solver here
is the oracle's GaNi solve (CPU; on a GPU it is homogenize_many): the test is
about the split and the gather, which must cover every cell exactly once and
give the single-process result.
"""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip('torch')
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from ffthompy_gb300.partition import homogenize_partitioned, partition_costs  # noqa: E402


def _cells(count=13, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice([5, 7, 9]))
        a = 1. + 9. * (rng.random((n, n)) < 0.4)
        out.append(np.einsum('ij,...->ij...', np.eye(2), a))
    return out


def _oracle_solve(coefs):
    import oracle
    res = []
    for A in coefs:
        N = np.array(A.shape[2:])
        G, _ = oracle.green_operator('scalar', N, np.ones(2), 'GaNi', 1)
        Af = lambda v, _G=G, _A=A: oracle.apply_GA(_G, _A, v)
        sols = []
        for l in range(2):
            E = np.zeros((2,) + tuple(N))
            E[l] = 1.
            x, _ = oracle.cg(Af, Af(-E), np.zeros_like(E), tol=1e-10, maxiter=200)
            sols.append(x + E)
        res.append(oracle.assembly_matrix(A, sols))
    return res


def test_partition_covers_each_unit_once_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 100, size=57).tolist()
    for world in (1, 2, 3, 8):
        parts = partition_costs(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        # longest-first greedy: within the largest cost of the optimum
        assert max(loads) - min(loads) <= max(costs)
    assert partition_costs([], 4) == [[], [], [], []]


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, 'tests'))
    import torch.distributed as dist
    from ffthompy_gb300.partition import homogenize_partitioned, torch_gather
    dist.init_process_group('gloo')
    seen = []

    def solve(cs):
        seen.extend(c.shape for c in cs)
        return _oracle_solve(cs)
    out = homogenize_partitioned(_cells(), dist.get_rank(), dist.get_world_size(), solve,
                                 gather=torch_gather())
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, len(seen), None if out is None else [o.tolist() for o in out]))


def test_two_gloo_ranks_gather_equals_single_process():
    world = 2
    port = _free_port()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cells = _cells()
    (r0, n0, out0), (r1, n1, out1) = res
    assert out1 is None and out0 is not None
    assert n0 + n1 == len(cells) and n0 > 0 and n1 > 0
    single = homogenize_partitioned(cells, 0, 1, _oracle_solve)
    assert len(out0) == len(single)
    for a, b in zip(out0, single):
        assert np.array_equal(np.asarray(a), b)


def test_cell_groups_cover_each_cell_once_within_the_field_cap():
    """homogenize_many's cell plans: the cells of one grid size in parts whose
    FP64 fields stay below the cap, every cell in exactly one part."""
    from ffthompy_gb300.batch import _cell_groups
    rng = np.random.default_rng(3)
    sizes = [(int(n), int(n)) for n in rng.choice([15, 31, 63], size=40)]
    coefs = [np.zeros((2, 2) + N) for N in sizes]
    groups = _cell_groups(coefs, None, 'scalar', field_cap=63 * 63 * 4 * 8 * 5)
    seen = sorted(i for idx in groups.values() for i in idx)
    assert seen == list(range(len(coefs)))
    for (N, Y, part), idx in groups.items():
        assert all(tuple(coefs[i].shape[2:]) == N for i in idx)
        assert len(idx) * np.prod(N) * 4 * 8 <= max(63 * 63 * 4 * 8 * 5, np.prod(N) * 4 * 8)
    big = [k for k in groups if k[0] == (63, 63)]
    assert all(len(groups[k]) <= 5 for k in big)
