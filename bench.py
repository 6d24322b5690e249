"""Benchmark of the GB300 Fourier-Galerkin homogenisation (one JSON line).

Workload (default 'spheres509', the 3D scalar configuration): seeded spheres
of radius 0.08, union volume fraction >= 0.3 on a 255^3 voxel image, phases
1 / 100, Galerkin with exact integration (grid-based, order 0, P = 255) on the
509^3 double grid, the 3 unit loads solved together.  One step = one
time-to-A_H: right-hand sides, batched CG to the tolerance that gives A_H
within 1e-6 of the FP64-refined value, and the A_H energy assembly, with the
coefficient resident in HBM.  Fields (4.7 GB per vector) exceed L2.

--impl reference runs the reference's algorithm on the host cores: its NumPy
restatement (the oracle; the reference source tree is not present on the GPU
host) on a bounded sample of the same workload (Ga N=63 -> 125^3 grid, same
sphere statistics, 3 loads, one CG iteration per load and step), one worker
process per host core.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N (solve on 2N-1), P image, L loads, radius, vf, contrast, tol)
    'spheres509': dict(N=255, P=255, radius=0.08, vf=0.3, contrast=100., tol=1e-3, seed=2026),
    'spheres255': dict(N=127, P=127, radius=0.08, vf=0.3, contrast=100., tol=1e-3, seed=2026),
    'spheres125': dict(N=63, P=63, radius=0.08, vf=0.3, contrast=100., tol=1e-3, seed=2026),
    # small anisotropic cases with the line lengths of spheres509 (255 solve,
    # 512 integration) on some axes, for profiling captures of a few GB:
    # axes 0 and 1 (the axis passes), axis 2 (the last-axis integration pass)
    'spheres255x255x127': dict(N=(255, 255, 127), P=(255, 255, 127), radius=0.08, vf=0.3,
                               contrast=100., tol=1e-3, seed=2026),
    'spheres63x127x255': dict(N=(63, 127, 255), P=(63, 127, 255), radius=0.08, vf=0.3,
                              contrast=100., tol=1e-3, seed=2026),
}


def _dims(v):
    return tuple(v) if isinstance(v, (tuple, list)) else (v,) * 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default='spheres509', choices=sorted(WORKLOADS))
    ap.add_argument('--precision', default='f32', choices=['f32', 'mixed'])
    ap.add_argument('--ga-mode', default='band', choices=['band', 'full'],
                    help='band: CG fields on the N grid, coefficient on a smooth integration '
                         'grid >= 2N-1; full: CG on the 2N-1 grid (the reference layout)')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-fp64', action='store_true')
    ap.add_argument('--no-fibres', action='store_true',
                    help='skip the 127^3 elasticity (fibres) time to A_H')
    ap.add_argument('--no-ensemble', action='store_true',
                    help='skip the 512-instance 2D ensemble measurement')
    ap.add_argument('--no-potential', action='store_true',
                    help='skip the potential-formulation measurement (GaNi on the image grid)')
    ap.add_argument('--kernels-only', action='store_true',
                    help='only the warm-up and timed steps of the workload (for profiler '
                         'captures): no FP64-refined reference, FP64 run, end-to-end run, '
                         'extra workloads or CPU baseline')
    ap.add_argument('--fibres-only', default=None, choices=['f64', 'mixed', 'both'],
                    help='only the 127^3 elasticity (fibres) Problem.calculate in this '
                         'precision, one JSON line (for profiler captures)')
    return ap.parse_args()


# ----------------------------------------------------------------------------
# distributed helpers (one process per GPU; replicas of the workload)
# ----------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    backend = 'nccl' if __import__('torch').cuda.is_available() else 'gloo'
    dist.init_process_group(backend=backend)
    return dist.get_rank(), dist.get_world_size(), dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    dev = 'cuda' if torch.cuda.is_available() and dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------
# workload construction
# ----------------------------------------------------------------------------
def image_values(w):
    from ffthompy_gb300.workloads import spheres_coefficient
    return spheres_coefficient(_dims(w['P']), radius=w['radius'], vf=w['vf'],
                               contrast=w['contrast'], seed=w['seed'])


def ga_coefficient(vals, w, grid=None):
    """Grid-based Ga coefficient (order 0) of the 2N-1 grid, assembled on the
    GPU, sampled on `grid` (default 2N-1)."""
    from ffthompy_gb300.materials import Material
    N = np.array(_dims(w['N']))
    mat = Material({'fun': lambda coord, _v=vals: _v, 'Y': np.ones(3), 'order': 0,
                    'P': np.array(_dims(w['P']))})
    return mat.get_A_Ga(Nbar=2 * N - 1, primaldual='primal', grid=grid)


def make_plan(w, precision, ga_mode):
    from ffthompy_gb300.engine import GalerkinPlan, nice_size
    N = _dims(w['N'])
    Ns = tuple(2 * n - 1 for n in N)
    if ga_mode == 'band':
        return GalerkinPlan(N, np.ones(3), physics='scalar', nloads=3,
                            integ=tuple(nice_size(n) for n in Ns), precision=precision)
    return GalerkinPlan(Ns, np.ones(3), physics='scalar', nloads=3, band=N,
                        precision=precision)


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        self.gpu = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu),
                                       '--query-gpu=' + self.QUERY, '--format=csv,noheader,nounits',
                                       '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, power, reasons = [], [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.f.read().strip().splitlines():
            parts = [x.strip() for x in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}
        loaded = [s for s, p in zip(sm, power) if p > 0.5 * max(power)] or sm
        return {'sm_mhz': statistics.median(loaded), 'sm_max_mhz': max(smax),
                'reasons': sorted(reasons), 'samples': len(sm),
                'power_w_max': max(power)}


# ----------------------------------------------------------------------------
# CPU baseline: the oracle (NumPy restatement of the reference) on samples
# ----------------------------------------------------------------------------
_SAMPLE_CACHE = {}


def _sample_operator(seed, N):
    """Ga spheres sample on the (2N-1)^3 grid: the oracle's coefficient,
    Green operator and the 3 right-hand sides (built once per process)."""
    key = (seed, N)
    if key not in _SAMPLE_CACHE:
        sys.path.insert(0, ROOT)
        import oracle
        from ffthompy_gb300.workloads import spheres_coefficient
        Nn = np.array([N] * 3)
        vals = spheres_coefficient((N,) * 3, radius=0.08, vf=0.3, contrast=100., seed=seed)
        mat = oracle.Material({'fun': lambda c, _v=vals: _v, 'Y': np.ones(3), 'order': 0,
                               'P': Nn})
        A = mat.get_A_Ga(2 * Nn - 1, 'primal')
        G, Ns = oracle.green_operator('scalar', Nn, np.ones(3), 'Ga', 1)
        Afun = lambda v, _G=G, _A=A: oracle.apply_GA(_G, _A, v)
        Bs = []
        for l in range(3):
            E = np.zeros((3,) + tuple(Ns))
            E[l] = 1.
            Bs.append(Afun(-E))
        _SAMPLE_CACHE.clear()
        _SAMPLE_CACHE[key] = (Afun, Bs, int(np.prod(Ns)))
    return _SAMPLE_CACHE[key]


def _cpu_sample(args):
    """One worker: iters CG iterations of each of the 3 loads of a Ga spheres
    sample; as_shipped adds the reference's CallBack matvec per iteration
    (ffthompy/general/solver_pp.py:13-24, installed by
    ffthompy/applications.py:71-72).  Returns (voxel-iterations, seconds)."""
    seed, N, iters, as_shipped = args
    import oracle
    Afun, Bs, M = _sample_operator(seed, N)
    t = 0.
    vox_it = 0
    for B in Bs:
        cb = None
        if as_shipped:
            log = []
            # one operator application per call, as CallBack.__call__
            cb = lambda x, _B=B, _log=log: _log.append(
                float(np.sqrt(np.sum((_B - Afun(x)) ** 2) / M)))
        t0 = time.perf_counter()
        _, info = oracle.cg(Afun, B, np.zeros_like(B), tol=0., maxiter=iters, callback=cb)
        t += time.perf_counter() - t0
        vox_it += M * info['kit']
    return vox_it, t


def _pinned_samples(jobs, core=0):
    """Run the samples in a child process pinned to one host core."""
    os.sched_setaffinity(0, {core})
    return [_cpu_sample(j) for j in jobs]


def host_cpu_model():
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith('Model name:'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open('/proc/cpuinfo'):
            if line.lower().startswith(('model name', 'cpu part')):
                return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


def cpu_baseline():
    """The oracle on one pinned host core: solver-only and as shipped (with the
    CallBack matvec) on the 61^3 and 125^3 grids of the same configuration;
    value = solver-only on 125^3 (the sample closest to the workload)."""
    import multiprocessing as mp
    jobs = [(7, 31, 4, False), (7, 31, 4, True), (7, 63, 2, False), (7, 63, 2, True)]
    core = sorted(os.sched_getaffinity(0))[0]
    with mp.get_context('spawn').Pool(1) as pool:
        res = pool.apply(_pinned_samples, (jobs, core))
    rates = {}
    for (seed, N, iters, shipped), (vox, t) in zip(jobs, res):
        rates['%s_%d^3' % ('as_shipped' if shipped else 'solver_only', 2 * N - 1)] = \
            round(vox / t / 1e6, 4)
    return {'value': rates['solver_only_125^3'], 'unit': 'Mvoxel-iter/s', 'cores': 1,
            'kind': 'port', 'cpu_model': host_cpu_model(), 'pinned_core': core,
            'variants': rates,
            'sample': 'NumPy restatement of the reference CG (rfftn G o A) pinned to one '
                      'host core: Ga spheres (r=0.08, vf=0.3, contrast 100, 3 loads) on the '
                      '61^3 grid (4 iterations per load) and the 125^3 grid (2 iterations '
                      'per load), solver-only and as shipped (the reference\'s CallBack '
                      'adds one operator application per iteration); value = solver-only '
                      'on 125^3'}


REF_SAMPLE = dict(N=63, iters=1)    # reference arm: 125^3 grid, 1 iteration per load and step


def _ref_worker(args):
    wid, seed, N, iters = args
    return _cpu_sample((seed, N, iters, False))


def run_reference(args):
    rank, world, dist = dist_init()
    if rank != 0:
        return
    import multiprocessing as mp
    cores = sorted(os.sched_getaffinity(0))
    ncores = len(cores)
    ctx = mp.get_context('spawn')
    N, iters = REF_SAMPLE['N'], REF_SAMPLE['iters']
    jobs = [(i, 100 + i, N, iters) for i in range(ncores)]
    times = []
    with ctx.Pool(ncores) as pool:
        # one sample per worker process, built once (setup not timed)
        pool.map(_ref_worker, [(i, s, n, 0) for i, s, n, _ in jobs], chunksize=1)
        for step in range(args.warmup + args.steps):
            res = pool.map(_ref_worker, jobs, chunksize=1)
            # the workers' CG phases run concurrently: aggregate over the slowest
            dt = max(r[1] for r in res)
            if step >= args.warmup:
                times.append((sum(r[0] for r in res), dt))
    vox = sum(v for v, _ in times)
    tot = sum(t for _, t in times)
    value = vox / tot / 1e6
    w = WORKLOADS[args.workload]
    out = {
        'impl': 'reference', 'metric': 'Mvoxel-iter/s', 'value': value, 'unit': 'Mvoxel-iter/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * tot / len(times), 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': '%s (sample: Ga %d^3 -> %d^3, one sample per host core)'
                               % (args.workload, N, 2 * N - 1),
                   'grid': [2 * n - 1 for n in _dims(w['N'])], 'loads': 3},
        'cpu_baseline': {'value': value, 'unit': 'Mvoxel-iter/s', 'cores': ncores, 'kind': 'port',
                         'cpu_model': host_cpu_model(),
                         'sample': '%d processes (one per host core) x (Ga %d^3 -> %d^3 spheres, '
                                   'r=0.08 vf=0.3 contrast 100, 3 loads x %d CG iteration per '
                                   'step, solver-only), NumPy restatement of the reference'
                                   % (ncores, N, 2 * N - 1, iters)},
        'e2e': {'value': value, 'unit': 'Mvoxel-iter/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------
# the GPU arm
# ----------------------------------------------------------------------------
def _ensemble_cells(count=512, sizes=(63, 127, 255, 511), seed=12):
    """The cfg4 ensemble's cells: (n, contrast, field seed) per instance."""
    rng = np.random.default_rng(seed)
    cells = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        contrast = float(np.exp(rng.uniform(np.log(2.), np.log(1000.))))
        cells.append((n, contrast, int(rng.integers(1 << 30))))
    return cells


def _ens_cpu_worker(args):
    """One host process: `iters` oracle CG iterations per load (GaNi, 2 loads,
    solver-only) of each of its cells.  Returns (voxel-iterations, seconds of
    CG)."""
    cells, iters = args
    sys.path.insert(0, ROOT)
    import oracle
    from ffthompy_gb300 import workloads
    vox, t = 0, 0.
    for n, contrast, gseed in cells:
        A = workloads.grf_phase_coefficient((n, n), ell=0.1, quantile=0.4, contrast=contrast,
                                            seed=gseed)
        G, _ = oracle.green_operator('scalar', np.array([n, n]), np.ones(2), 'GaNi', 1)
        Afun = lambda v, _G=G, _A=A: oracle.apply_GA(_G, _A, v)
        for l in range(2):
            E = np.zeros((2, n, n))
            E[l] = 1.
            B = Afun(-E)
            t0 = time.perf_counter()
            _, info = oracle.cg(Afun, B, np.zeros_like(B), tol=0., maxiter=iters)
            t += time.perf_counter() - t0
            vox += n * n * info['kit']
    return vox, t


def ensemble_cpu_baseline(iters=5):
    """The cfg4 ensemble on all host cores: the oracle (NumPy restatement of
    the reference's GaNi CG) on every one of the 512 cells for `iters`
    iterations per load, the cells dealt round-robin by size to one spawned
    process per core; aggregate Mvoxel-iter/s over the slowest process."""
    import multiprocessing as mp
    cells = sorted(_ensemble_cells(), key=lambda c: -c[0])
    ncores = len(os.sched_getaffinity(0))
    parts = [cells[i::ncores] for i in range(ncores)]
    with mp.get_context('spawn').Pool(ncores) as pool:
        res = pool.map(_ens_cpu_worker, [(p, iters) for p in parts], chunksize=1)
    vox = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return {'value': round(vox / wall / 1e6, 3), 'unit': 'Mvoxel-iter/s', 'cores': ncores,
            'kind': 'port', 'cpu_model': host_cpu_model(),
            'sample': 'all 512 cells of the ensemble, %d CG iterations per load (2 loads, '
                      'GaNi, solver-only), NumPy restatement of the reference, one spawned '
                      'process per host core' % iters}


def ensemble_measure(count=512, sizes=(63, 127, 255, 511), seed=12, tol=1e-6, workers=16,
                     precision='f64', dist=None):
    """Many independent 2D GaNi cells (thresholded Gaussian random fields,
    length 0.1, 0.4-quantile, contrast log-uniform in [2, 1000], n drawn from
    sizes, 2 loads each) solved together by homogenize_many to tol (FP64, or
    mixed: FP32 inner CG refined in FP64): aggregate Mvoxel-iter/s over all
    instances.  The cells of one size share one plan of several cells (every
    pass one launch for all of them), and the four sizes advance together in
    one graph per iteration.  Under torchrun the cells are split across the ranks
    (homogenize_many_ranks) and the time is the slowest rank's."""
    import torch
    from ffthompy_gb300 import workloads
    from ffthompy_gb300.batch import homogenize_many, homogenize_many_ranks
    coefs = [workloads.grf_phase_coefficient((n, n), ell=0.1, quantile=0.4, contrast=contrast,
                                             seed=gseed)
             for n, contrast, gseed in _ensemble_cells(count, sizes, seed)]
    # warm: the plan pool (one plan per cell), the autotuned launch shapes
    homogenize_many(coefs, tol=tol, workers=workers, precision=precision, mode='cells')
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    res = homogenize_many_ranks(coefs, tol=tol, workers=workers, precision=precision,
                                mode='cells')
    torch.cuda.synchronize()
    dt = reduce_max(dist, time.perf_counter() - t0)
    if res is None:     # not rank 0
        return None
    vox_it = sum(int(np.prod(A.shape[2:])) * sum(r['kit_primal']) for A, r in zip(coefs, res))
    return {'instances': count, 'sizes': list(sizes), 'loads': 2, 'precision': precision,
            'mode': 'cells',
            'tol': tol, 'voxels': int(sum(np.prod(A.shape[2:]) for A in coefs)),
            'ranks': 1 if dist is None else dist.get_world_size(),
            'seconds': dt, 'Mvoxel_iter_per_s': vox_it / dt / 1e6,
            'all_converged': all(r['status_primal'] == [0, 0] for r in res)}


def fibres_measure(n=127, tol=1e-6, seed=0, precisions=('f64', 'mixed')):
    """Linear elasticity with 8 parallel fibres on n^3 (Mandel 6x6 per voxel,
    phases (E, nu) = (1, 0.3) and (10, 0.2)), GaNi solve of the 6 unit strains,
    primal and dual, postprocessed with GaNi and Ga (order 0) bounds: the whole
    Problem.calculate() through the drop-in API, FP64 and mixed precision."""
    import torch
    from ffthompy_gb300 import workloads
    from ffthompy_gb300.problem import Problem
    vals = workloads.fibres_coefficient((n, n, n), seed=seed)
    N = np.array([n, n, n])
    out = {'grid': [n] * 3, 'loads': 6, 'tol': tol}
    mats = {}
    for prec in precisions:
        prob = {'name': 'fibres%d' % n, 'physics': 'elasticity',
                'material': workloads.fun_material(vals),
                'solve': {'kind': 'GaNi', 'N': N, 'primaldual': ['primal', 'dual'],
                          'precision': prec},
                'solver': {'kind': 'CG', 'tol': tol, 'maxiter': 1000},
                'postprocess': [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': 0, 'P': N}]}
        pb = Problem(prob, None)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pb.calculate()
        torch.cuda.synchronize()
        out['seconds_' + prec] = time.perf_counter() - t0
        out['kit_primal_' + prec] = [int(r['info']['kit']) for r in pb.output['res_primal']]
        out['phases_' + prec] = {pd: {k: round(v, 4) for k, v in ph.items()}
                                 for pd, ph in pb.output['time']['phases'].items()}
        mats[prec] = pb.output['mat_primal']['AH_GaNi_primal']
    if len(mats) == 2:
        out['AH_rel_diff_mixed_vs_f64'] = float(np.abs(mats['mixed'] - mats['f64']).max()
                                                / np.abs(mats['f64']).max())
    return out


def _cfg1_problem():
    """The 2D 45^2 GaNi square-inclusion problem (side 0.6, 11 I / 1 I), both
    loads, primal and dual, tol 1e-8, with GaNi and Ga (order None) bounds."""
    N = np.array([45, 45])
    mat = {'inclusions': ['square', 'otherwise'], 'positions': [np.zeros(2), ''],
           'params': [0.6 * np.ones(2), ''], 'vals': [11 * np.eye(2), np.eye(2)],
           'Y': np.ones(2), 'order': None}
    return {'name': 'square45', 'physics': 'scalar', 'material': mat,
            'solve': {'kind': 'GaNi', 'N': N, 'primaldual': ['primal', 'dual']},
            'solver': {'kind': 'CG', 'tol': 1e-8, 'maxiter': 1000},
            'postprocess': [{'kind': 'GaNi'}, {'kind': 'Ga', 'order': None}]}


def cfg1_measure(with_cpu=True, reps=5):
    """Time to solution of the 45^2 square-inclusion problem (latency-bound):
    the whole Problem.calculate() through the drop-in API in FP64 (median of
    reps after one warm run), and, on the host, the oracle (NumPy restatement
    of the reference, as shipped with its CallBack) on the same problem."""
    import torch
    from ffthompy_gb300.problem import Problem
    times = []
    for i in range(reps + 1):
        pb = Problem(_cfg1_problem(), None)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pb.calculate()
        torch.cuda.synchronize()
        if i:
            times.append(time.perf_counter() - t0)
    out = {'grid': [45, 45], 'loads': 2, 'tol': 1e-8, 'precision': 'f64',
           'seconds_median': float(np.median(times)),
           'kit_primal': [int(r['info']['kit']) for r in pb.output['res_primal']],
           'AH_GaNi_primal_00': float(pb.output['mat_primal']['AH_GaNi_primal'][0, 0]),
           'AH_Ga_primal_00': float(pb.output['mat_primal']['AH_Ga_primal'][0, 0]),
           'AH_Ga_dual_00': float(pb.output['mat_dual']['AH_Ga_dual'][0, 0])}
    if with_cpu:
        sys.path.insert(0, ROOT)
        import oracle
        t0 = time.perf_counter()
        ref = oracle.solve_problem(_cfg1_problem(), as_shipped=True)
        out['oracle_cpu_seconds'] = time.perf_counter() - t0
        a = pb.output['mat_primal']['AH_GaNi_primal']
        b = ref['mat_primal']['AH_GaNi_primal']
        out['AH_rel_diff_vs_oracle'] = float(np.abs(a - b).max() / np.abs(b).max())
    return out


def adjoint_measure(n=127, tol=1e-10):
    """dA_H/da(x) of the scalar GaNi problem with a(x) = exp(g(x)) on n^3
    (g a seeded Gaussian random field, length 0.15), 3 loads, mixed
    precision: forward solve and gradient through torch.autograd, timed
    end to end (CUDA synchronised)."""
    import torch
    from ffthompy_gb300 import workloads
    from ffthompy_gb300.adjoint import homogenized_matrix
    a_np = np.exp(workloads.gaussian_field((n,) * 3, 0.15, seed=11))
    out = {'grid': [n] * 3, 'loads': 3, 'precision': 'mixed', 'tol': tol}
    for rep in range(2):
        a = torch.tensor(a_np, device='cuda', requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        AH = homogenized_matrix(a, tol=tol, precision='mixed')
        AH[0, 0].backward()
        torch.cuda.synchronize()
        out['seconds_forward_and_gradient'] = time.perf_counter() - t0
    out['AH00'] = float(AH[0, 0])
    return out


def inverse_measure(n=253, d=6, reps=5):
    """The dual-coefficient inverse (fhp_coefficient_inverse) of a Mandel 6x6
    field on the Ga grid of the fibres problem (2*127-1)^3, CUDA events on the
    launching stream; algorithmic traffic 2 d^2 8 bytes per voxel, FP64
    operations 4 d^2 (d-1) per voxel (the elimination's products and
    differences) plus d^2 + d(d-1)/2 divisions."""
    import torch
    from ffthompy_gb300.engine import coefficient_inverse
    g = torch.Generator(device='cuda').manual_seed(1)
    R = torch.randn((d, d, n, n, n), dtype=torch.float64, device='cuda', generator=g)
    A = (R + R.transpose(0, 1)).mul_(0.5)
    A += d * torch.eye(d, dtype=torch.float64, device='cuda').reshape(d, d, 1, 1, 1)
    del R
    out = None
    for _ in range(2):
        out = coefficient_inverse(A, shift=True)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = []
    for _ in range(reps):
        del out
        torch.cuda.synchronize()
        ev[0].record(stream)
        out = coefficient_inverse(A, shift=True)
        ev[1].record(stream)
        torch.cuda.synchronize()
        ms.append(ev[0].elapsed_time(ev[1]))
    t = float(np.median(ms)) * 1e-3
    vox = n ** 3
    return {'grid': [n] * 3, 'd': d, 'ms': t * 1e3,
            'GBps': 2 * d * d * 8 * vox / t / 1e9,
            'fp64_gflops': 4 * d * d * (d - 1) * vox / t / 1e9,
            'note': 'inputs (%.1f GB) larger than L2; median of %d launches'
                    % (d * d * 8 * vox / 1e9, reps)}


def potential_measure(vals, w, tol, steps=2):
    """Time to A_H of the potential formulation (fhp_potential_*) for the
    GaNi discretisation on the image grid, 3 loads batched, FP32 with FP64
    reductions; Mvoxel-iter/s counts the image grid."""
    import torch
    from ffthompy_gb300.engine import GalerkinPlan
    N = _dims(w['N'])
    A = torch.as_tensor(vals).cuda()
    plan = GalerkinPlan(N, np.ones(3), physics='scalar', nloads=3, precision='f32')
    plan.set_coefficient(A)
    grad = GalerkinPlan(N, np.ones(3), physics='scalar', nloads=3, precision='f32')
    grad.set_coefficient(A)
    Xg, info_g = grad.cg(grad.rhs_macro(1), tol=tol, maxiter=2000)
    AHg = grad.energy(Xg)
    del grad, Xg
    # the potential CG stops on the 'r' Fourier norm of the preconditioned
    # residual, which equals the gradient residual norm of the same iterate
    run = lambda: plan.energy(plan.potential_field(
        plan.potential_cg(plan.potential_rhs(), tol=tol, maxiter=2000)[0]))
    info = plan.potential_cg(plan.potential_rhs(), tol=tol, maxiter=2000)[1]
    run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        AH = run()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    M = int(np.prod(N))
    return {'grid': list(N), 'loads': 3, 'precision': 'f32', 'time_to_AH_s': dt,
            'Mvoxel_iter_per_s': M * sum(info['kit']) / dt / 1e6, 'cg_iterations': info['kit'],
            'gradient_formulation_cg_iterations': info_g['kit'],
            'AH_rel_diff_vs_gradient_formulation': float(np.abs(AH - AHg).max()
                                                         / np.abs(AHg).max())}


def run_kernels_only(args, w, A, M, dist, world, rank):
    """The workload's steps alone (warm-up, then timed): the command line
    for profiler captures of the CG kernels."""
    import torch
    plan = make_plan(w, args.precision, args.ga_mode)
    plan.set_coefficient(A.data)
    plan.autotune()
    kits = []
    torch.cuda.synchronize()
    t0 = None
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        X, info = plan.cg(plan.rhs_macro(1), tol=w['tol'], maxiter=2000, log_rows=1)
        plan.energy(X)
        if i >= args.warmup:
            kits.append(sum(info['kit']))
    torch.cuda.synchronize()
    dt = time.perf_counter() - (t0 if t0 is not None else time.perf_counter())
    if rank == 0:
        print(json.dumps({'workload': args.workload, 'kernels_only': True,
                          'cg_iterations': info['kit'], 'seconds': dt,
                          'Mvoxel_iter_per_s': M * sum(kits) / max(dt, 1e-9) / 1e6}),
              flush=True)


def _h2d_ms(torch, h):
    """Milliseconds of one host-to-device copy of the host tensor h."""
    d = torch.empty(h.shape, dtype=h.dtype, device='cuda')
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    d.copy_(h, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    return round(e0.elapsed_time(e1), 3)


def _h2d_gbps(torch, nbytes=1 << 30):
    """Host-to-device bandwidth from a fresh pinned buffer (CUDA events)."""
    h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    h.fill_(1.0)
    d = torch.empty_like(h, device='cuda')
    d.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    d.copy_(h, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    return round(nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9, 1)


def run_gpu(args):
    import torch
    rank, world, dist = dist_init()
    torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', rank)))
    import __graft_entry__
    __graft_entry__.build()
    from ffthompy_gb300.engine import GalerkinPlan
    h2d_start = _h2d_gbps(torch)

    from ffthompy_gb300.engine import nice_size
    w = WORKLOADS[args.workload]
    N = _dims(w['N'])
    Ns = tuple(2 * n - 1 for n in N)
    M = int(np.prod(Ns))              # voxels of the reference's solve grid prod(2N-1)
    vals = image_values(w)
    cgrid = tuple(nice_size(n) for n in Ns) if args.ga_mode == 'band' else Ns
    A = ga_coefficient(vals, w, grid=cgrid)           # (3,3)+grid on the GPU, FP64
    A_iso = A.data[0, 0].contiguous()
    extras = {'coefficient_grid': list(cgrid)}

    if args.kernels_only:
        args.no_fp64 = args.no_fibres = args.no_ensemble = args.no_potential = True
        args.no_cpu_baseline = True
        return run_kernels_only(args, w, A, M, dist, world, rank)
    # FP64-refined reference A_H (mixed plan, FP64 outer residual, tight tol)
    ref = make_plan(w, 'mixed', args.ga_mode)
    ref.set_coefficient(A.data)
    t0 = time.perf_counter()
    Xr, info_r = ref.cg(ref.rhs_macro(1), tol=w['tol'] * 1e-3, maxiter=2000)
    AH_ref = ref.energy(Xr)
    extras['AH_fp64_refined'] = AH_ref.tolist()
    extras['fp64_refined_kit'] = info_r['kit']
    extras['fp64_refined_seconds'] = time.perf_counter() - t0
    del Xr, ref
    torch.cuda.empty_cache()

    plan = make_plan(w, args.precision, args.ga_mode)
    plan.set_coefficient(A.data)
    tol = w['tol']
    choice, ms_apply = plan.autotune()
    extras['autotune'] = {'choice': list(choice), 'ms_per_operator_application': ms_apply,
                          'note': 'band plans: (integration kernel 1=register lines / '
                                  '0=shared-memory cores, CTAs per SM, axis tile multiplier)'}

    def step(p=plan, t=tol):
        B = p.rhs_macro(1)
        X, info = p.cg(B, tol=t, maxiter=2000, log_rows=1)
        AH = p.energy(X)
        return AH, info

    for _ in range(args.warmup):
        AH, info = step()
    torch.cuda.synchronize()
    barrier(dist)
    # the timed region runs the shipped path: each CG iteration is one CUDA
    # graph replay, no per-kernel events
    launches0 = plan.launches()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    stream = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    kits = []
    for _ in range(args.steps):
        AH, info = step()
        kits.append(sum(info['kit']))
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(dist)
    ms = ev0.elapsed_time(ev1)
    ms = reduce_max(dist, ms)
    launches = plan.launches() - launches0
    vox_it = M * sum(kits) * world
    value = vox_it / (ms / 1e3) / 1e6
    AH_err = float(np.abs(AH - AH_ref).max() / np.abs(AH_ref).max())

    # per-kernel CUDA events: one more step of the same workload with the
    # profiler on (direct launches instead of graph replay, same kernels)
    plan.profile(True)
    torch.cuda.synchronize()
    ev2 = torch.cuda.Event(enable_timing=True)
    ev3 = torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    AHp, infop = step()
    ev3.record(stream)
    torch.cuda.synchronize()
    prof = plan.profile_read()
    plan.profile(False)
    extras['profiled_step_ms'] = ev2.elapsed_time(ev3)
    extras['profiled_step_cg_iterations'] = infop['kit']

    # roofline of the dominant kernel (largest total time in the profiled step)
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get('hbm_gbs', 6800.0))
    peak_src = 'measured' if 'hbm_gbs' in peaks else 'fallback'
    top = max(prof.items(), key=lambda kv: kv[1]['ms'])
    tname, t = top
    per_launch_s = t['ms'] / 1e3 / max(1, t['launches'])
    achieved = t['bytes_per_launch'] / per_launch_s / 1e9
    tot_ms = sum(x['ms'] for x in prof.values())
    it_max = max(infop['kit'])
    kernels = {}
    for k, v in sorted(prof.items(), key=lambda kv: -kv[1]['ms']):
        row = {'launches': v['launches'], 'ms_total': round(v['ms'], 3),
               'share': round(v['ms'] / max(1e-9, tot_ms), 4),
               'MB_per_launch': round(v['bytes_per_launch'] / 1e6, 1)}
        gbps = v['bytes_per_launch'] / (v['ms'] / 1e3 / max(1, v['launches'])) / 1e9
        # kernels launched a few times per step (set-up, final projection)
        # may run from L2: their rate is not evidence of HBM bandwidth
        if v['launches'] >= it_max:
            row['GBps'] = round(gbps, 1)
        else:
            row['GBps_not_hbm'] = round(gbps, 1)
            row['note'] = 'launched %d times per step (outside the CG loop)' % v['launches']
        kernels[k] = row
    traffic = None
    tf = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tf):
        try:
            # ncu DRAM bytes per launch of the dominant kernel, per workload
            traffic = _json.load(open(tf)).get(args.workload, {}).get(tname, {}).get(
                'bytes_per_launch')
        except (OSError, ValueError):
            traffic = None
    roofline = {'bound': 'hbm', 'achieved': round(achieved, 1), 'peak': peak, 'unit': 'GB/s',
                'frac': round(achieved / peak, 4), 'traffic': traffic, 'kernel': tname,
                'peak_source': peak_src + ' hbm_gbs',
                'timing': 'CUDA events around each launch in a profiled step of the same '
                          'workload after the timed region'}

    # the plain form: FP64 fields and FFTs, the same band operator and
    # tolerance, timed to A_H (right-hand sides, CG, energy) with CUDA events
    if not args.no_fp64:
        p64 = make_plan(w, 'f64', args.ga_mode)
        p64.set_coefficient(A.data)
        p64.cg(p64.rhs_macro(1), tol=0., maxiter=1)     # warm: graph, scratch
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        AH64, info64 = step(p64, tol)
        e1.record(stream)
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3
        extras['fp64_time_to_AH_s'] = t64
        extras['fp64_cg_iterations'] = info64['kit']
        extras['fp64_AH_rel_err_vs_fp64_refined'] = float(np.abs(AH64 - AH_ref).max()
                                                          / np.abs(AH_ref).max())
        extras['speedup_vs_fp64_gpu'] = t64 / (ms / 1e3 / args.steps)
        del p64
        torch.cuda.empty_cache()

    # end to end through the host-buffer C-ABI entry point
    # the coefficient as a user holds it: a pinned host array written by the
    # CPU; e2e_phases times torch's upload of the same buffer before and after
    # the library calls, and of fresh pinned buffers
    A_np = A_iso.cpu().numpy()
    host_A = torch.empty(tuple(A_iso.shape), dtype=torch.float64, pin_memory=True)
    A_host = host_A.numpy()
    np.copyto(A_host, A_np)
    ph = {}
    ph['torch_h2d_host_buffer_before_calls_ms'] = _h2d_ms(torch, host_A)
    e2e_plan = make_plan(w, args.precision, args.ga_mode)
    e2e_plan.set_coefficient(A.data)
    e2e_plan.autotune()     # the cached choice of the timed plan
    from ffthompy_gb300 import _lib
    from ffthompy_gb300.engine import homogenize_host_many
    e2e_steps = max(1, min(args.steps, 3))
    # one call per step (each step uploads, solves and reads A_H back)
    e2e_plan.homogenize_host(packed=A_host, kind=_lib.FHP_COEF_ISO, proj=1, tol=tol,
                             maxiter=2000)   # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kit_1 = 0
    for _ in range(e2e_steps):
        AH1, kit, _, _ = e2e_plan.homogenize_host(packed=A_host, kind=_lib.FHP_COEF_ISO, proj=1,
                                                  tol=tol, maxiter=2000)
        kit_1 += sum(kit)
    single_s = reduce_max(dist, time.perf_counter() - t0)
    # the steps as one call: the upload of step k + 1 overlaps the solve of k
    homogenize_host_many(e2e_plan, [A_host], _lib.FHP_COEF_ISO, tol=tol, maxiter=2000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    AHs, kits, _ = homogenize_host_many(e2e_plan, [A_host] * e2e_steps, _lib.FHP_COEF_ISO,
                                        tol=tol, maxiter=2000)
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    AHe = AHs[-1]
    kit_e = sum(sum(k) for k in kits)
    e2e = {'value': M * kit_e * world / e2e_s / 1e6, 'unit': 'Mvoxel-iter/s',
           'h2d_bytes_per_step': int(A_host.nbytes), 'd2h_bytes_per_step': 9 * 8,
           'seconds_per_step': e2e_s / e2e_steps,
           'api': 'fhp_homogenize_host_many over %d steps (the upload of a step overlaps the '
                  'solve of the previous one)' % e2e_steps}
    extras['e2e_single_calls'] = {'value': M * kit_1 * world / single_s / 1e6,
                                  'unit': 'Mvoxel-iter/s',
                                  'seconds_per_step': single_s / e2e_steps,
                                  'api': 'fhp_homogenize_host, one call per step'}
    extras['AH_e2e_rel_diff'] = float(np.abs(AHe - AH).max() / np.abs(AH).max())
    # the same phases through the package API, each bracketed by CUDA events
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    evs[0].record(stream)
    e2e_plan.set_coefficient_packed(A_host, _lib.FHP_COEF_ISO)
    evs[1].record(stream)
    Be = e2e_plan.rhs_macro(1)
    evs[2].record(stream)
    Xe, _ = e2e_plan.cg(Be, tol=tol, maxiter=2000, log_rows=1)
    evs[3].record(stream)
    e2e_plan.energy(Xe)
    evs[4].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    for i, name in enumerate(['coefficient_upload_ms', 'rhs_ms', 'cg_ms', 'energy_ms']):
        ph[name] = round(evs[i].elapsed_time(evs[i + 1]), 3)
    ph['wall_ms'] = round(wall * 1e3, 3)
    # the same host buffer copied by torch, for comparison with the upload,
    # and a pinned buffer filled by a device-to-host copy
    dev_A = torch.empty(tuple(A_iso.shape), dtype=torch.float64, device='cuda')
    d2h_filled = torch.empty(tuple(A_iso.shape), dtype=torch.float64, pin_memory=True)
    d2h_filled.copy_(A_iso)
    torch.cuda.synchronize()
    evs[0].record(stream)
    dev_A.copy_(d2h_filled, non_blocking=True)
    evs[1].record(stream)
    torch.cuda.synchronize()
    ph['torch_h2d_d2h_filled_buffer_ms'] = round(evs[0].elapsed_time(evs[1]), 3)
    del d2h_filled
    torch.cuda.synchronize()
    evs[0].record(stream)
    dev_A.copy_(host_A, non_blocking=True)
    evs[1].record(stream)
    torch.cuda.synchronize()
    ph['torch_h2d_same_buffer_ms'] = round(evs[0].elapsed_time(evs[1]), 3)
    del dev_A
    # a pinned buffer that does not come from torch's host-block cache
    if hasattr(torch._C, '_host_emptyCache'):
        torch._C._host_emptyCache()
    fresh = torch.empty(tuple(A_iso.shape), dtype=torch.float64, pin_memory=True)
    np.copyto(fresh.numpy(), A_np)
    ph['torch_h2d_fresh_cpu_filled_ms'] = _h2d_ms(torch, fresh)
    del fresh, A_np
    ph['h2d_fresh_pinned_GBps_at_start'] = h2d_start
    ph['h2d_fresh_pinned_GBps_here'] = _h2d_gbps(torch)
    extras['e2e_phases'] = ph
    del e2e_plan, Xe, Be
    torch.cuda.empty_cache()

    # potential formulation with the 1/|xi| preconditioner (homog_GaNi_full_
    # potential): GaNi on the image grid, all loads, FP32, against the gradient
    # formulation's A_H on the same grid and tolerance
    if not args.no_potential:
        extras['potential'] = potential_measure(vals, w, tol)
    if not args.no_fibres:
        extras['adjoint127'] = adjoint_measure()
        extras['fibres127'] = fibres_measure()
        extras['cfg1_square45'] = cfg1_measure(with_cpu=not args.no_cpu_baseline)
        extras['coefficient_inverse'] = inverse_measure()
    if not args.no_ensemble:
        extras['ensemble_grf2d'] = ensemble_measure(dist=dist)
        extras['ensemble_grf2d_mixed'] = ensemble_measure(precision='mixed', dist=dist)

    if rank != 0:
        return
    out = {
        'metric': 'Mvoxel-iter/s', 'value': round(value, 2), 'unit': 'Mvoxel-iter/s',
        'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': round(ms / args.steps, 3), 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32' if args.precision == 'f32' else 'f64+f32',
        'data': 'synthetic',
        'config': {'workload': '%s: 3D scalar Ga, spheres r=%.2f vf>=%.1f contrast %g, image '
                               '%s -> %s grid, 3 loads batched, CG tol %g (A_H within 1e-6)'
                               % (args.workload, w['radius'], w['vf'], w['contrast'],
                                  'x'.join(map(str, _dims(w['P']))), 'x'.join(map(str, Ns)),
                                  w['tol']),
                   'grid': list(Ns), 'loads': 3, 'precision': args.precision,
                   'ga_mode': args.ga_mode,
                   'voxels_counted': 'prod(2N-1) per load and iteration (the reference grid)',
                   'l2': 'inputs larger than L2 (coefficient %.2f GB, spectra %.1f GB)'
                         % (np.prod(cgrid) * (4 if args.precision == 'f32' else 8) / 1e9,
                            3 * 3 * np.prod(cgrid) * (4 if args.precision == 'f32' else 8)
                            / 1e9)},
        'time_to_AH_s': round(ms / 1e3 / args.steps, 4),
        'cg_iterations': info['kit'],
        'AH': AH.tolist(), 'AH_rel_err_vs_fp64': AH_err,
        'roofline': roofline,
        'kernels': kernels,
        'gpu_launches': int(launches),
        'clocks': clocks,
        'e2e': e2e,
    }
    out.update(extras)
    if not args.no_cpu_baseline:
        out['cpu_baseline'] = cpu_baseline()
        if not args.no_ensemble:
            out['ensemble_cpu_baseline'] = ensemble_cpu_baseline()
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.fibres_only:
        precs = ('f64', 'mixed') if args.fibres_only == 'both' else (args.fibres_only,)
        print(json.dumps({'fibres127': fibres_measure(precisions=precs)}), flush=True)
        return
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
