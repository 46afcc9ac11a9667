"""Drop-in ``cuda_row_reduce`` (and a GPU-backed ``row_reduce``).

``cuda_row_reduce(matrix, field_characteristic=p)`` keeps the signature,
dtype rules and return value of linac's function
(linac/pycuda_row_reduce.py:18-151):

* p > 0: residues as uint32, or uint64 when p > 2^32-1 (or ``_mod64=True``);
  the input is cast with ``astype`` exactly as the reference does.
* p == 0: float64 when every entry has zero imaginary part (or
  ``_real=True``), else complex128; rows are pre-scaled by their largest |a|
  and the head threshold is 1e-9 (linac/row_reduce.cu:55, 201-270).
* returns a new ndarray of the input's shape; the input is not modified.

Differences, all deliberate: the modulus must be prime (a non-prime raises
ZeroDivisionError instead of returning garbage); the pivot search covers every
row (the reference's windowed search can miss pivots below row 2048); an
all-zero float row stays zero instead of becoming NaN; "real" means every
imaginary part is zero (the reference tests only that the largest one is 0).
Extensions: ``return_pivots=True`` also returns the pivot columns, and ``out=``
receives the result (e.g. a pinned buffer from ``pinned_empty``).
"""
from __future__ import annotations

import ctypes
import fractions

import numpy as np

from . import _lib
from .timeit_decorator import timeit

FLOAT_TOLERANCE = 1e-9


def _is_real(matrix: np.ndarray) -> bool:
    if np.iscomplexobj(matrix):
        return not np.any(matrix.imag)
    if matrix.dtype == object:
        imag = np.vectorize(lambda x: getattr(x, "imag", 0), otypes=[object])(matrix)
        return not np.any(imag != 0)
    return True


def field_dtype(matrix: np.ndarray, field_characteristic: int, _real=None, _mod64=None) -> np.dtype:
    """The element type linac would pick (linac/pycuda_row_reduce.py:41-56)."""
    p = int(field_characteristic)
    if p > 0:
        if _mod64 or (_mod64 is None and p > 2**32 - 1):
            return np.dtype(np.uint64)
        return np.dtype(np.uint32)
    if _real or (_real is None and _is_real(matrix)):
        return np.dtype(np.float64)
    return np.dtype(np.complex128)


def _as_field_array(matrix: np.ndarray, dtype: np.dtype) -> np.ndarray:
    if dtype == np.float64 and np.iscomplexobj(matrix):
        host = matrix.real.astype(np.float64)
    elif dtype == np.float64 and matrix.dtype == object:
        host = np.vectorize(lambda x: float(getattr(x, "real", x)), otypes=[np.float64])(matrix)
    elif dtype == np.complex128 and matrix.dtype == object:
        host = np.vectorize(complex, otypes=[np.complex128])(matrix)
    else:
        host = matrix.astype(dtype, copy=False)
    if host.ndim != 2:
        raise ValueError("cuda_row_reduce expects a 2-D matrix")
    if not (host.flags.c_contiguous or (host.strides[1] == host.itemsize and host.strides[0] % host.itemsize == 0
                                        and host.strides[0] >= host.shape[1] * host.itemsize)):
        host = np.ascontiguousarray(host)
    return host


def rref_host_call(host: np.ndarray, p: int, out: np.ndarray, flags: int = 0,
                   tol: float = FLOAT_TOLERANCE):
    """One synchronous lnc_rref_host call; returns (pivot_columns, rank)."""
    code = _lib.DTYPE_CODE[host.dtype]
    m, n = host.shape
    ld_in = host.strides[0] // host.itemsize if m > 0 else n
    ld_out = out.strides[0] // out.itemsize if m > 0 else n
    kmax = min(m, n)
    piv = np.empty(max(kmax, 1), dtype=np.int64)
    rank = ctypes.c_int64(0)
    rc = _lib.lib().lnc_rref_host(code, m, n, int(p), float(tol), host.ctypes.data, ld_in,
                                  out.ctypes.data, ld_out, piv.ctypes.data, ctypes.byref(rank), int(flags))
    _lib.check(rc, "cuda_row_reduce")
    r = int(rank.value)
    return [int(x) for x in piv[:r]], r


@timeit
def cuda_row_reduce(matrix, field_characteristic=0, verbose=False, _real=None, _mod64=None,
                    return_pivots=False, out=None, mixed=False):
    r"""Reduced row-echelon form on the GPU.

    Args:
        matrix (2D numpy.ndarray): the matrix to reduce.
        field_characteristic (int, optional, default: 0): the characteristic p
            of the field, or 0 for real and complex matrices.
        verbose (bool, optional, default: False): print timing information.
        return_pivots (bool): also return the list of pivot columns.
        out (ndarray, optional): destination of the result (shape of matrix,
            dtype of the field).
        mixed (bool): real / complex matrices only -- trailing updates on the
            tensor cores in 31-bit fixed point, FP64 panels, FP64 refinement
            of the result (``linac_gb300._lib.mixed_report()`` describes it).
    """
    matrix = np.asarray(matrix)
    if matrix.ndim != 2:
        raise ValueError("cuda_row_reduce expects a 2-D matrix")
    p = int(field_characteristic)
    dtype = field_dtype(matrix, p, _real, _mod64)
    host = _as_field_array(matrix, dtype)
    if out is None:
        out = np.empty(host.shape, dtype=dtype)
    elif out.shape != host.shape or out.dtype != dtype:
        raise ValueError(f"out must have shape {host.shape} and dtype {dtype}")
    if verbose:
        _lib.kernel_timing(True)
    flags = 0
    if mixed:
        if p != 0:
            raise ValueError("mixed precision applies to real / complex matrices (field_characteristic=0)")
        flags |= _lib.LNC_FLAG_MIXED
    pivots, rank = rref_host_call(host, p, out, flags=flags)
    if verbose:
        for name, kc in (("panel", _lib.KC_PANEL), ("trailing update", _lib.KC_TRAILING),
                         ("gather", _lib.KC_GATHER)):
            cnt, ms = _lib.kernel_timing_read(kc)
            print(f"time_{name.replace(' ', '_')}: {ms / 1000.0:.6f} s over {cnt} launches")
        print(f"rank {rank} of a {host.shape[0]} x {host.shape[1]} matrix")
        _lib.kernel_timing(False)
    if return_pivots:
        return out, pivots
    return out


def row_reduce(matrix, pivoting=1, scaling=True, reduced_echelon=True, threshold=10 ** -9, prime=None,
               verbose=False):
    """GPU-backed counterpart of linac's CPU ``row_reduce`` (linac/row_reduce.py:16).

    Returns ``(matrix, variable_order)``.  Only Gauss-Jordan to the reduced
    echelon form with row pivoting is provided (pivoting 0 or 1; the pivot row
    is searched over every remaining row, which always yields the RREF);
    column-permuting rook / total pivoting and ``reduced_echelon=False`` raise
    NotImplementedError.  With a prime the matrix is reduced over F_prime (the
    scaling flag is ignored there: scaling a residue matrix by real row maxima
    is meaningless); without, over float64 / complex128 with ``threshold``.
    """
    if pivoting not in [0, 1, 2, 3]:
        raise ValueError("Invalid pivoting.")
    if pivoting > 1:
        raise NotImplementedError("rook / total pivoting (column permutations) is not provided on the GPU")
    if not reduced_echelon:
        raise NotImplementedError("only the reduced row-echelon form is provided on the GPU")
    matrix = np.asarray(matrix)
    variable_order = list(range(matrix.shape[1]))
    if prime:
        p = int(prime)
        if matrix.dtype == object:
            def conv(x):
                if isinstance(x, fractions.Fraction):
                    return x.numerator * pow(x.denominator, -1, p) % p
                return int(x) % p
            matrix = np.vectorize(conv, otypes=[object])(matrix)
        dtype = np.uint64 if p > 2**32 - 1 else np.uint32
        host = np.ascontiguousarray((matrix.astype(object) % p).astype(dtype)) if matrix.dtype == object \
            else np.ascontiguousarray(np.mod(matrix.astype(np.int64) if matrix.dtype.kind == "i" else matrix, p)
                                      .astype(dtype))
        out = np.empty_like(host)
        rref_host_call(host, p, out)
        return out.astype(np.int64) if dtype == np.uint32 else out, variable_order
    dtype = field_dtype(matrix, 0)
    host = _as_field_array(matrix, dtype)
    out = np.empty(host.shape, dtype=dtype)
    rref_host_call(host, 0, out, flags=0 if scaling else _lib.LNC_FLAG_NO_SCALING, tol=float(threshold))
    return out, variable_order


def pinned_empty(shape, dtype) -> np.ndarray:
    """An ndarray in pinned host memory (fast host<->device copies); the
    allocation is released when the array is garbage-collected."""
    return np.asarray(_lib.PinnedArray(shape, dtype))
