"""Many independent cells on one GPU (ensembles of microstructures).

homogenize_many() solves the GaNi cell problems of a list of coefficient
fields of possibly different grids - the reference would run
applications.scalar / elasticity (ffthompy/applications.py:11-90, 93-176) once
per instance - and returns one A_H per instance.

Each worker thread owns a CUDA stream and one GalerkinPlan per grid size it
meets (plans keep their buffers, so nothing is allocated per instance after
the first of a size).  A host coefficient's primal problem is solved by one
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


def homogenize_many(coefs, Y=None, physics='scalar', tol=1e-6, maxiter=1000,
                    precision='f64', workers=8, primaldual=('primal',)):
    """coefs: sequence of (dv, dv) + N coefficient arrays (numpy or torch),
    origin-0 grid values as Material.get_A_GaNi returns them.  Returns a list
    of {'primal': A_H (L x L numpy), 'kit': [...], 'status': [...]} (and
    'dual', the inverted dual energy matrix, if requested) in input order."""
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
