"""Generate the FP64 oracle fixtures of the 3D spheres configuration.

The benchmark workload is 3D scalar conductivity with seeded spheres
(radius 0.08, union volume fraction >= 0.3 on the voxel image, phases 1 and
100), Galerkin with exact integration, grid-based coefficient of order 0 with
P = N on the 2N-1 grid, and the 3 unit loads.  At the benchmark's size
(N = 255) the CPU cannot solve it; this script solves the same configuration
at N = 31 (61^3 grid) and N = 63 (125^3 grid) with the oracle in FP64
(oracle/ffth_oracle.py: Material.get_A_Ga = ffthompy/materials.py:54-113,
green_operator = applications.py:24-37 with the Ga scale of Tensor.enlarge,
cg = general/solver.py:80-139, assembly_matrix = postprocess.py:53-70).

Stored per size (tests/golden/hl_spheres_<N>.npz):
  AH            A_H of the CG solution at tol 1e-9 (the converged value)
  AH_tol1e-3    A_H of the iterate where the residual first reaches 1e-3
  AH_tol1e-6    same at 1e-6
  kit_tol*      per-load CG iteration counts at those tolerances
  res_log       per-load residual histories of the tight solve (padded NaN)

The oracle is test infrastructure and is pinned to the reference's own runs
by tests/test_oracle_golden.py.  Runtime: about a minute at N = 31 and about
ten at N = 63 on one core.

Usage:  python tests/golden/make_headline.py [31 63 ...]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ffthompy_gb300.workloads import spheres_coefficient  # noqa: E402

SEED = 2026
TOLS = (1e-3, 1e-6)
TIGHT = 1e-9


def make(N):
    t0 = time.time()
    Nn = np.array([N] * 3)
    vals = spheres_coefficient((N,) * 3, radius=0.08, vf=0.3, contrast=100., seed=SEED)
    mat = oracle.Material({'fun': lambda c, _v=vals: _v, 'Y': np.ones(3), 'order': 0,
                           'P': Nn})
    A = mat.get_A_Ga(2 * Nn - 1, 'primal')
    G, Ns = oracle.green_operator('scalar', Nn, np.ones(3), 'Ga', 1)
    Afun = lambda v: oracle.apply_GA(G, A, v)
    arrays = {}
    logs, kits = [], {t: [] for t in TOLS}
    sols = {t: [] for t in TOLS}
    tight = []
    for l in range(3):
        E = np.zeros((3,) + tuple(Ns))
        E[l] = 1.
        B = Afun(-E)
        X, info = oracle.cg(Afun, B, np.zeros_like(E), tol=TIGHT, maxiter=5000)
        tight.append(X + E)
        log = np.asarray(info['res_log'])
        logs.append(log)
        want = {}
        for t in TOLS:
            k = int(np.argmax(log <= t))
            kits[t].append(k)
            want[k] = t
        # replay the same iterates up to the largest wanted count
        seen = {}

        def grab(x, _c=[0], _w=want):
            if _c[0] in _w:
                seen[_w[_c[0]]] = x.copy()
            _c[0] += 1
        oracle.cg(Afun, B, np.zeros_like(E), tol=0., maxiter=max(want), callback=grab)
        for t in TOLS:
            sols[t].append(seen[t] + E)
        print('N=%d load %d: kit %s (tight %d) %.0fs' % (N, l, [kits[t][-1] for t in TOLS],
                                                         info['kit'], time.time() - t0),
              flush=True)
    arrays['AH'] = oracle.assembly_matrix(A, tight)
    for t in TOLS:
        arrays['AH_tol%g' % t] = oracle.assembly_matrix(A, sols[t])
        arrays['kit_tol%g' % t] = np.array(kits[t], dtype=np.int64)
    width = max(len(g) for g in logs)
    arrays['res_log'] = np.stack([np.pad(g, (0, width - len(g)), constant_values=np.nan)
                                  for g in logs])
    meta = dict(N=N, seed=SEED, radius=0.08, vf=0.3, contrast=100., grid=list(map(int, Ns)),
                tight_tol=TIGHT, tols=list(TOLS), kind='Ga', order=0, P=N, loads=3,
                generator='tests/golden/make_headline.py (oracle, FP64)')
    path = os.path.join(HERE, 'hl_spheres_%d.npz' % N)
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)
    print('wrote', path, 'AH', arrays['AH'].diagonal(), '%.0fs' % (time.time() - t0))


if __name__ == '__main__':
    for n in (sys.argv[1:] or ['31', '63']):
        make(int(n))
