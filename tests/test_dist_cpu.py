"""The multi-process path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py runs one replica per GPU under torchrun (the path does not shard
within a solve): dist_init reads RANK / WORLD_SIZE / MASTER_* from the
environment, the timed region is bracketed by barriers and the step time is
the maximum over ranks; in the reference arm only rank 0 works and prints.
"""
import contextlib
import io
import os
import socket
import sys

import pytest

torch = pytest.importorskip('torch')
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, d = bench.dist_init()
    assert (r, w) == (rank, world) and d is not None
    assert d.get_backend() == 'gloo'
    bench.barrier(d)
    # the slowest rank's time is the step time
    m = bench.reduce_max(d, 10.0 * (rank + 1))
    bench.barrier(d)
    d.destroy_process_group()
    q.put((rank, m))


def test_two_gloo_ranks_barrier_and_max():
    world = 2
    port = _free_port()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 20.0), (1, 20.0)]


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, 'dist_init', lambda: (1, 2, None))

    class Args:
        steps, warmup, gpus, workload, impl = 1, 0, 2, 'spheres509', 'reference'
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert bench.run_reference(Args()) is None
    assert buf.getvalue() == ''
