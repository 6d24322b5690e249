"""Many independent cells on one GPU (ensembles of microstructures).

homogenize_many() solves the GaNi cell problems of a list of coefficient
fields of possibly different grids - the reference would run
applications.scalar / elasticity (ffthompy/applications.py:11-90, 93-176) once
per instance - and returns one A_H per instance.

mode='cells' (the default), mode='threads' and mode='batched' give the same
per-cell results.  On the 512-cell 2D ensemble (n in 63..511, 2 loads, tol
1e-6) a GB300 takes 1.8 s mixed and 8.7 s FP64 in mode='cells', 2.7 s and
9.8 s in mode='threads', 4.5 s and 13.2 s in mode='batched'.  FP64 time is
bound by the FP64 arithmetic of the Bluestein lines (127- and 511-point).

mode='cells': the cells of one grid size share one plan of several cells
(GalerkinPlan(ncells=K), fhp_plan_create_cells): every pass of an iteration is
one launch for all K cells, each load of each cell keeps its own CG scalars
and stopping test, and the passes skip the cells whose loads have all
stopped.  The plans of the different sizes advance together in one
fhp_cg_solve_many call (one CUDA graph per iteration).  Plans are kept in a
process-wide pool per size, cell count and precision.

mode='batched': every cell gets a plan from a pool kept across
calls (one plan per cell and grid size, created once, each with its own
buffers and CG state); the coefficients are uploaded, the right-hand sides
built, and all cells of all sizes are solved by one fhp_cg_solve_many call:
each CG iteration of the whole ensemble is one CUDA graph whose branches are
the cells' kernels, and the host polls one combined done flag.  Mixed
precision refines every cell in FP64 with each outer step's FP32 solves of
all cells advanced together.  Launch shapes are autotuned once per grid size
and precision (fhp_plan_autotune) and cached.

mode='threads': each worker thread owns a CUDA stream and one GalerkinPlan per grid size it
meets (plans keep their buffers, so nothing is allocated per instance after
the first of a size; launch shapes autotuned once per size and precision).  A host coefficient's primal problem is solved by one
library call (fhp_homogenize_host: upload, right-hand sides, CG, A_H); its
dual coefficient is uploaded and inverted on the GPU (fhp_coefficient_inverse).  The library's C calls release the GIL (ctypes), so the
instances of different workers run concurrently on the GPU: small grids,
whose launches alone would leave most SMs idle, fill the GPU together.  Each
instance is solved with its own CG scalars and stopping test, exactly as a
separate run would be.
"""
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import _lib
from .engine import (GalerkinPlan, coef_kind_of, coef_kind_of_torch, coefficient_inverse,
                     pack_coefficient, pack_coefficient_torch, require_cuda)


_POOL = {}


def _pooled_plans(key, count, make):
    """count plans of one kind from the process-wide pool (created on demand,
    kept for later calls)."""
    lst = _POOL.setdefault(key, [])
    while len(lst) < count:
        lst.append(make())
    return lst[:count]


def homogenize_many(coefs, Y=None, physics='scalar', tol=1e-6, maxiter=1000,
                    precision='f64', workers=16, primaldual=('primal',), mode='cells'):
    """coefs: sequence of (dv, dv) + N coefficient arrays (numpy or torch),
    origin-0 grid values as Material.get_A_GaNi returns them.  Returns a list
    of {'primal': A_H (L x L numpy), 'kit': [...], 'status': [...]} (and
    'dual', the inverted dual energy matrix, if requested) in input order.
    workers: threads of mode='threads'."""
    if mode == 'batched':
        return _homogenize_batched(coefs, Y, physics, tol, maxiter, precision, primaldual)
    if mode == 'cells':
        return _homogenize_cells(coefs, Y, physics, tol, maxiter, precision, primaldual)
    if mode != 'threads':
        raise ValueError("mode must be 'threads', 'cells' or 'batched'")
    require_cuda()
    device = torch.device('cuda', torch.cuda.current_device())
    order = sorted(range(len(coefs)), key=lambda i: -int(np.prod(coefs[i].shape[2:])))
    out = [None] * len(coefs)
    local = threading.local()

    def state():
        if not hasattr(local, 'stream'):
            local.stream = torch.cuda.Stream(device=device)
            local.plans = {}
        return local

    def run(i):
        st = state()
        A = coefs[i]
        N = tuple(int(n) for n in A.shape[2:])
        d = len(N)
        Yi = np.ones(d) if Y is None else np.asarray(Y, dtype=np.float64)
        with torch.cuda.stream(st.stream):
            key = (N, tuple(Yi))
            plan = st.plans.get(key)
            if plan is None:
                plan = GalerkinPlan(N, Yi, physics=physics, precision=precision)
                st.plans[key] = plan
            res = {}
            on_device = list(primaldual)
            if not isinstance(A, torch.Tensor):
                Ah = np.asarray(A, dtype=np.float64)
                if 'primal' in primaldual:
                    # host coefficient: one library call (upload, right-hand
                    # sides, CG, A_H) on this worker's stream, GIL released
                    kind = coef_kind_of(Ah)
                    if not getattr(plan, '_tuned', False):
                        # launch shapes of this grid size: timed once per size and
                        # precision in the process, then taken from the cache
                        plan.set_coefficient_packed(pack_coefficient(Ah, kind), kind)
                        plan.autotune()
                        plan._tuned = True
                    AH, kit, nres, _ = plan.homogenize_host(packed=pack_coefficient(Ah, kind),
                                                            kind=kind, proj=1, tol=tol,
                                                            maxiter=maxiter)
                    res['primal'] = AH
                    res['kit_primal'] = kit
                    res['status_primal'] = [0 if (k == 0 or r <= tol) else _lib.FHP_NONCONVERGED
                                            for k, r in zip(kit, nres)]
                on_device = [pd for pd in primaldual if pd == 'dual']
                if not on_device:
                    out[i] = res
                    return
                # the dual coefficient is inverted on the GPU
                A = torch.from_numpy(Ah)
            At = A.to(device, torch.float64, non_blocking=False)
            for pd in on_device:
                proj = 1 if pd == 'primal' else 2
                Ap = At if pd == 'primal' else _inverse_field(At)
                kind = coef_kind_of_torch(Ap)
                plan.set_coefficient_packed(pack_coefficient_torch(Ap, kind), kind)
                X, info = plan.cg(plan.rhs_macro(proj), tol=tol, maxiter=maxiter, proj=proj)
                AH = plan.energy(X)
                res[pd] = AH if pd == 'primal' else np.linalg.inv(AH)
                res['kit_' + pd] = info['kit']
                res['status_' + pd] = info['status']
            st.stream.synchronize()
        out[i] = res

    with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
        for f in [ex.submit(run, i) for i in order]:
            f.result()
    return out


def _homogenize_batched(coefs, Y, physics, tol, maxiter, precision, primaldual):
    require_cuda()
    from .engine import cg_many
    device = torch.device('cuda', torch.cuda.current_device())
    groups = {}
    for i, A in enumerate(coefs):
        N = tuple(int(n) for n in A.shape[2:])
        Yi = np.ones(len(N)) if Y is None else np.asarray(Y, dtype=np.float64)
        groups.setdefault((N, tuple(Yi)), []).append(i)
    cell_plan = {}
    for (N, Yi), idx in groups.items():
        key = (device.index, N, Yi, physics, precision)
        plans = _pooled_plans(key, len(idx), lambda: GalerkinPlan(N, np.asarray(Yi),
                                                                  physics=physics,
                                                                  precision=precision))
        for i, p in zip(idx, plans):
            cell_plan[i] = p
    out = [dict() for _ in coefs]
    order = list(range(len(coefs)))
    for pd in primaldual:
        proj = 1 if pd == 'primal' else 2
        bs = []
        for i in order:
            plan, A = cell_plan[i], coefs[i]
            if pd == 'primal' and not isinstance(A, torch.Tensor):
                Ah = np.asarray(A, dtype=np.float64)
                kind = coef_kind_of(Ah)
                plan.set_coefficient_packed(pack_coefficient(Ah, kind), kind)
            else:
                At = torch.as_tensor(A).to(device, torch.float64)
                Ap = At if pd == 'primal' else _inverse_field(At)
                kind = coef_kind_of_torch(Ap)
                plan.set_coefficient_packed(pack_coefficient_torch(Ap, kind), kind)
            # launch shapes per grid size: timed for the first plan of a size,
            # taken from the tuner's cache for the others
            plan.autotune()
            bs.append(plan.rhs_macro(proj))
        sols = cg_many([cell_plan[i] for i in order], bs, tol=tol, maxiter=maxiter, proj=proj)
        for i, (X, info) in zip(order, sols):
            AH = cell_plan[i].energy(X)
            out[i][pd] = AH if pd == 'primal' else np.linalg.inv(AH)
            out[i]['kit_' + pd] = info['kit']
            out[i]['status_' + pd] = info['status']
    return out


def _cell_groups(coefs, Y, physics, field_cap=4e9):
    """{(N, Y, part): [cell indices]}: the cells of each grid size, in parts
    whose fields stay below field_cap bytes (FP64) each."""
    groups = {}
    for i, A in enumerate(coefs):
        N = tuple(int(n) for n in A.shape[2:])
        Yi = np.ones(len(N)) if Y is None else np.asarray(Y, dtype=np.float64)
        groups.setdefault((N, tuple(Yi)), []).append(i)
    out = {}
    for (N, Yi), idx in groups.items():
        d = len(N)
        dv = d if physics == 'scalar' else d * (d + 1) // 2
        per = float(np.prod(N)) * dv * dv * 8.0      # one cell's field: dv loads x dv comps
        cap = max(1, int(field_cap // per))
        for k in range(0, len(idx), cap):
            out[(N, Yi, k // cap)] = idx[k:k + cap]
    return out


def _homogenize_cells(coefs, Y, physics, tol, maxiter, precision, primaldual):
    require_cuda()
    from .engine import cg_many
    device = torch.device('cuda', torch.cuda.current_device())
    groups = _cell_groups(coefs, Y, physics)
    plans = {}
    for (N, Yi, part), idx in groups.items():
        key = ('cells', device.index, N, Yi, physics, precision, len(idx), part)
        plans[(N, Yi, part)] = _pooled_plans(
            key, 1, lambda: GalerkinPlan(N, np.asarray(Yi), physics=physics,
                                         precision=precision, ncells=len(idx)))[0]
    out = [dict() for _ in coefs]
    for pd in primaldual:
        proj = 1 if pd == 'primal' else 2
        bs = []
        for gk, idx in groups.items():
            plan = plans[gk]
            host = pd == 'primal' and not any(isinstance(coefs[i], torch.Tensor) for i in idx)
            if host:
                As = [np.asarray(coefs[i], dtype=np.float64) for i in idx]
                kind = max(coef_kind_of(A) for A in As)
                vals = np.stack([pack_coefficient(A, kind) for A in As])
            else:
                As = []
                for i in idx:
                    At = torch.as_tensor(coefs[i]).to(device, torch.float64)
                    As.append(At if pd == 'primal' else _inverse_field(At))
                kind = max(coef_kind_of_torch(A) for A in As)
                vals = torch.stack([pack_coefficient_torch(A, kind) for A in As])
            # every cell's coefficient, packed with the most general kind
            plan.set_coefficient_packed(vals, kind)
            plan.autotune()
            bs.append(plan.rhs_macro(proj))
        sols = cg_many([plans[gk] for gk in groups], bs, tol=tol, maxiter=maxiter, proj=proj)
        for (gk, idx), (X, info) in zip(groups.items(), sols):
            plan = plans[gk]
            AH = plan.energy(X)
            L = plan.nloads
            for j, i in enumerate(idx):
                out[i][pd] = AH[j] if pd == 'primal' else np.linalg.inv(AH[j])
                out[i]['kit_' + pd] = info['kit'][j * L:(j + 1) * L]
                out[i]['status_' + pd] = info['status'][j * L:(j + 1) * L]
    return out


def _inverse_field(A):
    """Per-voxel inverse of a (dv, dv) + N field (the dual coefficient,
    ffthompy/materials.py get_A_GaNi with primaldual='dual'), on the GPU."""
    return coefficient_inverse(A)


def homogenize_many_ranks(coefs, group=None, **kw):
    """homogenize_many with the cells split across the ranks of an initialised
    torch.distributed process group (one process per GPU, each on its own
    device): every rank solves its share (partition.partition_costs by voxel
    count) and rank 0 receives all results in input order (None on the other
    ranks).  Without an initialised group this is homogenize_many."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return homogenize_many(coefs, **kw)
    from .partition import homogenize_partitioned, torch_gather
    return homogenize_partitioned(coefs, dist.get_rank(group), dist.get_world_size(group),
                                  lambda cs: homogenize_many(cs, **kw),
                                  gather=torch_gather(group))
