"""Drop-in ``load_matrices`` and ``cuda_load_matrix``.

Both keep linac's signatures and return values
(linac/pycuda_matrix_loader.py:27-124 and :127-230):

* ``load_matrices(prefactors, ansatze, points, use_cuda=True)`` builds, per
  system, the ``bases`` (points x [variables..., prefactor]) and ``lindices``
  (monomials x (degree + 1), the last index selecting the prefactor) arrays on
  the host and evaluates every entry ``prefactor(point) * prod(variables)`` on
  the GPU.  Points are a dict (``points['field']``, ``points[name]`` -> values)
  or a list of callables with a ``.field`` attribute, as in the reference.
* ``cuda_load_matrix(bases, lindices, ...)`` evaluates one matrix: uint32
  residues for p <= 2^31-1, uint64 above (the loader's own threshold,
  pycuda_matrix_loader.py:63), float64 / complex128 for p = 0.

There is no CPU path in this package: ``use_cuda=False`` raises
NotImplementedError.  Variables are numbered in a deterministic order (by
length, then name); the reference orders same-length names by set iteration,
so its index arrays can differ from run to run while the matrices are equal.
"""
from __future__ import annotations

from copy import deepcopy

import numpy as np

from . import _lib
from .timeit_decorator import timeit


def _flatten(x):
    if isinstance(x, (str, bytes)):
        return [x]
    out = []
    try:
        items = list(x)
    except TypeError:
        return [x]
    for it in items:
        out.extend(_flatten(it))
    return out


def loader_dtype(field_characteristic: int, bases=None, _real=None, _mod64=None) -> np.dtype:
    p = int(field_characteristic)
    if p > 0:
        if _mod64 or (_mod64 is None and p > 2**31 - 1):
            return np.dtype(np.uint64)
        return np.dtype(np.uint32)
    if _real:
        return np.dtype(np.float64)
    if _real is None and bases is not None:
        b0 = np.asarray(bases)[0] if len(bases) else np.zeros(0)
        imag = np.vectorize(lambda x: getattr(x, "imag", 0), otypes=[object])(b0) if b0.dtype == object \
            else np.imag(b0)
        if not np.any(np.asarray(imag, dtype=complex if np.iscomplexobj(imag) else float) != 0):
            return np.dtype(np.float64)
    return np.dtype(np.complex128)


def _to_field_array(bases, dtype: np.dtype) -> np.ndarray:
    bases = np.asarray(bases)
    if dtype == np.float64 and (np.iscomplexobj(bases) or bases.dtype == object):
        if bases.dtype == object:
            return np.vectorize(lambda x: float(getattr(x, "real", x)), otypes=[np.float64])(bases)
        return np.ascontiguousarray(bases.real, dtype=np.float64)
    if dtype == np.complex128 and bases.dtype == object:
        return np.vectorize(complex, otypes=[np.complex128])(bases)
    if dtype.kind == "u" and bases.dtype == object:
        return np.ascontiguousarray(np.array([[int(v) for v in row] for row in bases], dtype=dtype)
                                    .reshape(bases.shape))
    return np.ascontiguousarray(bases.astype(dtype))


@timeit
def cuda_load_matrix(bases, lindices, shape=None, field_characteristic=0, _real=None, _mod64=None,
                     verbose=False):
    """Evaluate monomials as products of precomputed base values on the GPU.

    bases: (n_rows, basis_length); lindices: (n_cols, degree) uint32 indices
    into a bases row.  Returns the (n_rows, n_cols) matrix.
    """
    bases = np.atleast_2d(np.asarray(bases))
    lindices = np.asarray(lindices)
    n_rows, n_cols = bases.shape[0], lindices.shape[0]
    if shape is not None:
        assert tuple(shape) == (n_rows, n_cols), (
            f"Shape mismatch: provided {shape}, inferred {(n_rows, n_cols)}")
    p = int(field_characteristic)
    dtype = loader_dtype(p, bases, _real, _mod64)
    b = _to_field_array(bases, dtype)
    lind = np.ascontiguousarray(lindices, dtype=np.uint32)
    if lind.ndim != 2:
        raise ValueError("lindices must be 2-D (n_cols, degree)")
    degree = lind.shape[1]
    out = np.zeros((n_rows, n_cols), dtype=dtype)
    if n_rows == 0 or n_cols == 0:
        return out
    if degree == 0:
        raise ValueError("lindices needs at least one index per column")
    if lind.size and int(lind.max()) >= b.shape[1]:
        raise ValueError("lindices refers past the end of a bases row")
    if verbose:
        _lib.kernel_timing(True)
    rc = _lib.lib().lnc_load_matrix_host(_lib.DTYPE_CODE[dtype], n_rows, n_cols, b.shape[1], degree, p,
                                         b.ctypes.data, lind.ctypes.data, out.ctypes.data)
    _lib.check(rc, "cuda_load_matrix")
    if verbose:
        cnt, ms = _lib.kernel_timing_read(_lib.KC_LOADER)
        print(f"time loading: {ms / 1000.0:.6f} s ({cnt} launch)")
        _lib.kernel_timing(False)
    return out


def _field_of(points):
    return points["field"] if isinstance(points, dict) else points[0].field


def _native_converter(field):
    p = int(field.characteristic)
    if p == 0:
        return (float, float) if field.name in ("mpf", "R") else (complex, complex)
    if field.name in ("padic", "Qp"):
        try:
            from pyadic import ModP  # optional: reduces p-adic numbers to their residue
        except ImportError:  # plain integers: the residue is n mod p
            ModP = None

        def to_native(x):
            if ModP is not None:
                return int(ModP(x) if x in field else ModP(x, p))
            return int(x) % p
        return to_native, int
    return int, int


def build_bases_and_indices(prefactors, ansatze, points):
    """Host half of load_matrices: per system, the bases array (object dtype
    of native numbers) and the uint32 lindices array.  Returns
    (bases_list, lindices_list); a system with no monomials gets an index
    array with zero rows."""
    field = _field_of(points)
    to_native, _ = _native_converter(field)
    ansatze = deepcopy(ansatze)
    for i, ansatz in enumerate(ansatze):
        L = max((len(mono) for mono in ansatz), default=0)
        ansatze[i] = [list(mono) + ["1"] * (L - len(mono)) for mono in ansatz]
    names = sorted(set(_flatten(ansatze)) - {"1"}, key=lambda s: (len(s), s))
    variables = ["1"] + names
    index = {v: k for k, v in enumerate(variables)}
    if isinstance(points, dict):
        cols = [np.asarray(points[v], dtype=object).ravel() for v in variables]
        n_pts = len(cols[0]) if cols else 0
        mono = np.empty((n_pts, len(variables)), dtype=object)
        for k, col in enumerate(cols):
            mono[:, k] = [to_native(x) for x in col]
    else:
        mono = np.array([[to_native(pt(v)) for v in variables] for pt in points], dtype=object)
        n_pts = len(points)
    bases_list, lind_list = [], []
    p = int(field.characteristic)
    for i, prefactor in enumerate(prefactors):
        if isinstance(points, dict):
            pref = np.array([to_native(x) for x in np.asarray(points[prefactor], dtype=object).ravel()],
                            dtype=object)
        else:
            vals = []
            for pt in points:
                if isinstance(prefactor, str):
                    vals.append(to_native(pt(prefactor)))
                else:
                    v = prefactor(pt)
                    vals.append(1 if v == 1 else to_native(v))
            pref = np.array(vals, dtype=object)
        bases = np.empty((n_pts, len(variables) + 1), dtype=object)
        bases[:, :len(variables)] = mono
        bases[:, -1] = pref
        if field.name in ("padic", "Qp"):
            bases = bases % p
        ansatz = ansatze[i]
        width = (len(ansatz[0]) if len(ansatz) > 0 else 0) + 1
        lind = np.zeros((len(ansatz), width), dtype=np.uint32)
        for j, monomial in enumerate(ansatz):
            for k, var in enumerate(monomial):
                lind[j, k] = index[var]
            lind[j, width - 1] = bases.shape[1] - 1
        bases_list.append(bases)
        lind_list.append(lind)
    return bases_list, lind_list


def load_matrices(prefactors, ansatze, points, use_cuda=True, _use_galois=True, verbose=False):
    """One matrix per (prefactor, ansatz) system, rows = points, columns =
    monomials (linac/pycuda_matrix_loader.py:127-230)."""
    if not use_cuda:
        raise NotImplementedError("linac_gb300 evaluates the loader on the GPU only (use_cuda=False)")
    field = _field_of(points)
    p = int(field.characteristic)
    bases_list, lind_list = build_bases_and_indices(prefactors, ansatze, points)
    real = None
    if p == 0:
        real = field.name in ("mpf", "R")
    As = []
    for bases, lind in zip(bases_list, lind_list):
        if lind.shape[0] > 0:
            As.append(cuda_load_matrix(bases, lind, (bases.shape[0], lind.shape[0]), field_characteristic=p,
                                       _real=real, verbose=verbose))
        else:
            As.append(np.empty((bases.shape[0], 0), dtype="uint32"))
    if _single_point(points, ansatze):
        # one point given as scalars: the reference's bases are 1-D and it returns the
        # matrices' only rows (linac/pycuda_matrix_loader.py:191,228-229)
        return [A[0] for A in As]
    return As


def _single_point(points, ansatze) -> bool:
    """True for dict-form points whose variables hold scalars (one point)."""
    if not isinstance(points, dict):
        return False
    names = {"1"} | set(_flatten(ansatze))
    return all(np.ndim(points[v]) == 0 for v in names if v in points)
