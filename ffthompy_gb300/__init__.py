"""GB300-native Fourier-Galerkin homogenisation (drop-in for FFTHomPy's
Ga / GaNi solve path).

Host layer mirroring the reference's entry points: problem.Problem,
materials.Material, projections, tensors.{Tensor, DFT, Operator},
general.solver.linear_solver, postprocess.  The hot path (G o A, CG, energy,
interpolation) runs in libffthompy_gb300.so, called through a C ABI
(include/ffthompy_gb300.h).
"""
from ._lib import FhpError, load as load_library  # noqa: F401

__version__ = '0.1.0'
