"""The host line planner (csrc/fhp_lineplan.cpp) on CPU: radix factorisations
and the digit-reversed slot tables (LineDev::pos) that the pass kernels index.

The compile-time cores compute slots with p2_pos<P, K>, where K follows
p2_k_for: FP32 512-point cores run as two stages 16 * 32, all other
power-of-two cores in ceil(P/4) balanced stages.  Kernels that read the
plan's table and kernels that compute slots must agree, so the table of every
power-of-two core length, built the way an FP32 or FP64 engine builds it, must
equal that digit reversal; and 255 must factor as 3 * 5 * 17 (its
compile-time core).  A small host program linked with fhp_lineplan.cpp prints
the tables (no CUDA call runs).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'ffthompy_gb300', 'csrc')

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include "fhp_engine.h"
int main(int argc, char** argv) {
  for (int i = 1; i + 1 < argc; i += 2) {
    const int n = std::atoi(argv[i]), two = std::atoi(argv[i + 1]);
    fhp::LinePlanHost h;
    if (!fhp::build_line_plan(n, h, two)) { std::printf("fail %d\n", n); continue; }
    std::printf("%d %d %d %d", n, two, h.nf, h.blue);
    std::printf(" R");
    for (int r : h.rad) std::printf(" %d", r);
    std::printf(" P");
    for (int p : h.pos) std::printf(" %d", p);
    std::printf("\n");
  }
  return 0;
}
'''


def _p2_e(P, s, K):
    if K:
        return P // K + (1 if s >= K - P % K else 0)
    n = (P + 3) // 4
    return P // n + (1 if s < P % n else 0)


def _p2_pos(P, K, k):
    nst = K if K else (P + 3) // 4
    pos, eb = 0, 0
    for s in range(nst):
        e = _p2_e(P, s, K)
        pos |= ((k >> eb) & ((1 << e) - 1)) << (P - eb - e)
        eb += e
    return pos


def _p2_k_for(fp32, P):
    return 2 if (fp32 and P == 9) else 0


@pytest.fixture(scope='module')
def planner(tmp_path_factory):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('nvcc not found')
    d = tmp_path_factory.mktemp('lineplan')
    src = d / 'main.cpp'
    src.write_text(PROGRAM)
    exe = d / 'lineplan'
    cmd = [nvcc, '-std=c++17', '-x', 'c++', str(src), os.path.join(CSRC, 'fhp_lineplan.cpp'),
           '-I', CSRC, '-o', str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail('building the planner probe failed:\n' + r.stderr[-2000:])

    def run(pairs):
        args = [str(x) for p in pairs for x in p]
        out = subprocess.run([str(exe)] + args, capture_output=True, text=True, check=True)
        res = {}
        for line in out.stdout.splitlines():
            head, rest = line.split(' R')
            n, two, nf, blue = (int(v) for v in head.split())
            rad, pos = rest.split(' P')
            res[(n, two)] = (nf, blue, [int(v) for v in rad.split()], [int(v) for v in pos.split()])
        return res
    return run


def test_power_of_two_tables_match_the_compile_time_digit_reversal(planner):
    pairs = [(1 << P, two) for P in range(5, 11) for two in (0, 512)]
    res = planner(pairs)
    for (n, two), (nf, blue, rad, pos) in res.items():
        P = n.bit_length() - 1
        fp32 = two == 512
        K = _p2_k_for(fp32, P)
        assert nf == n and blue == 0
        nst = K if K else (P + 3) // 4
        assert rad == [1 << _p2_e(P, s, K) for s in range(nst)], (n, two, rad)
        assert pos == [_p2_pos(P, K, k) for k in range(n)], (n, two)
    # FP32 512-point lines are 16 . 32, FP64 ones 8 . 8 . 8
    assert res[(512, 512)][2] == [16, 32]
    assert res[(512, 0)][2] == [8, 8, 8]


def test_bluestein_cores_use_the_same_decomposition(planner):
    """Bluestein lines run their power-of-two cores through the same
    compile-time stages, with the filter spectrum in that digit order: 251
    (prime, 2*251-1 = 501 -> 512) gets a 16 . 32 core in FP32 and 8 . 8 . 8 in
    FP64; 127 -> 256 and 509 -> 1024; 257 -> 540 keeps a mixed-radix core."""
    res = planner([(251, 512), (251, 0), (509, 0), (509, 512), (127, 0), (127, 512),
                   (257, 512)])
    assert res[(251, 512)][:3] == (512, 1, [16, 32])
    assert res[(251, 0)][:3] == (512, 1, [8, 8, 8])
    assert res[(257, 512)][0] == 540
    for (n, two), (nf, blue, rad, pos) in res.items():
        assert blue == 1
        if nf & (nf - 1) == 0:
            P = nf.bit_length() - 1
            K = _p2_k_for(two == 512, P)
            nst = K if K else (P + 3) // 4
            assert rad == [1 << _p2_e(P, s, K) for s in range(nst)], (n, two, rad)


def test_255_factors_as_the_compile_time_core(planner):
    res = planner([(255, 0), (255, 512)])
    for (n, two), (nf, blue, rad, pos) in res.items():
        assert (nf, blue, rad) == (255, 0, [3, 5, 17])
        assert pos == [(k % 3) * 85 + ((k // 3) % 5) * 17 + k // 15 for k in range(255)]
