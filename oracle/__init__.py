"""CPU oracle for the FFTHomPy Fourier-Galerkin solve (test infrastructure).

This package is a plain NumPy restatement of the reference algorithm
(vondrejc/FFTHomPy: projections, materials, G o A operator, CG, postprocess).
It exists only to check the CUDA library: the tests under tests/, the smoke
check in __graft_entry__.smoke() and the cpu_baseline / reference arm of
bench.py use it.  The product package ffthompy_gb300 never imports it and
never falls back to it.

Pinning: tests/test_oracle_golden.py checks this restatement against the
reference's own golden pickles (test_results/python3/*, flattened into
tests/golden/ref_*.npz) and against fixtures produced by running the
reference itself (tests/golden/run_*.npz, op_*.npz; generator
tests/golden/make_golden.py).
"""
from .ffth_oracle import *  # noqa: F401,F403
