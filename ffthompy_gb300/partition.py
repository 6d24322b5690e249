"""Ensembles of cells split across ranks (one process per GPU).

The independent units of the Fourier-Galerkin homogenisation are the cells
of an ensemble: each is a complete cell problem with its own CG and A_H
(the reference runs applications.scalar once per cell,
ffthompy/applications.py:11-90), so they need no exchange while they are
solved.  A rank solves its share of the cells on its own GPU and the per-cell
results are gathered on rank 0 at the end: no collective touches the data
path.

Load cases of one cell are not split across ranks: A_H[i][j] pairs the
fields of loads i and j (ffthompy/postprocess.py:53-70), so splitting them
would need the fields exchanged.
"""
import numpy as np


def partition_costs(costs, world):
    """Assign units with the given costs to `world` ranks: longest first, each
    to the least loaded rank (ties to the lower rank).  Deterministic; every
    unit goes to exactly one rank.  Returns a list of index lists (in input
    order within a rank)."""
    if world < 1:
        raise ValueError('world must be >= 1')
    costs = [float(c) for c in costs]
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def cell_cost(coef):
    """Work estimate of one cell: its voxel count (CG iterations are not
    known in advance)."""
    return float(np.prod(coef.shape[2:]))


def homogenize_partitioned(coefs, rank, world, solve, gather=None, costs=None):
    """Solve the cells of this rank's share with solve(list_of_coefs) ->
    list_of_results and gather every result on rank 0.

    gather(obj) -> list of the objects of all ranks on rank 0 (None elsewhere),
    e.g. torch.distributed.gather_object; None for a single process.  Returns
    the results in input order on rank 0 and None on the other ranks."""
    costs = [cell_cost(c) for c in coefs] if costs is None else costs
    parts = partition_costs(costs, world)
    mine = parts[rank]
    res = solve([coefs[i] for i in mine]) if mine else []
    pairs = list(zip(mine, res))
    if world == 1 or gather is None:
        allp = [pairs]
    else:
        allp = gather(pairs)
    if rank != 0:
        return None
    out = [None] * len(coefs)
    for plist in allp:
        for i, r in plist:
            if out[i] is not None:
                raise RuntimeError('cell %d solved twice' % i)
            out[i] = r
    missing = [i for i, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError('cells without a result: %s' % missing[:10])
    return out


def torch_gather(group=None):
    """A gather for homogenize_partitioned over torch.distributed (gloo or
    NCCL): the per-rank result lists arrive on rank 0."""
    import torch.distributed as dist

    def gather(obj):
        world = dist.get_world_size(group)
        out = [None] * world if dist.get_rank(group) == 0 else None
        dist.gather_object(obj, out, dst=0, group=group)
        return out
    return gather
