from .objects import Tensor, scalar_product, einsum
from .operators import DFT, Operator
