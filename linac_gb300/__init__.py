"""linac_gb300: dense reduced row-echelon form over F_p, the reals and the
complex numbers, plus the monomial matrix loader, on one NVIDIA GB300
(sm_103a) -- a drop-in for linac's ``cuda_row_reduce`` / ``load_matrices``.

The compute runs in hand-written CUDA (liblinac_gb300.so, C ABI in
include/linac_gb300.h) driven through ctypes; there is no CPU fallback.
"""
from .version import __version__
from ._optional import CUDA_FOUND, GALOIS_FOUND
from .row_reduce import cuda_row_reduce, row_reduce, pinned_empty
from .matrix_loader import cuda_load_matrix, load_matrices
from .timeit_decorator import timeit

__all__ = [
    "__version__",
    "CUDA_FOUND",
    "GALOIS_FOUND",
    "cuda_row_reduce",
    "cuda_load_matrix",
    "load_matrices",
    "row_reduce",
    "timeit",
    "pinned_empty",
]
