"""Pivots and null spaces of row-reduced matrices (GPU-backed counterparts of
linac/linear_algebra_tools.py:10-63).

* ``canonical_kernel_from_row_reduced_echelon_form(rref)`` -- same result as
  linac's host function (an RREF with zero rows dropped -> its canonical
  null-space basis, one column per non-pivot column with -1 in that column's
  row), built on the device.  Dtypes follow numpy's promotion of the RREF's
  dtype with int, as in linac (uint32 -> int64, uint64 -> float64, float and
  complex unchanged).
* ``null_space(matrix, field_characteristic)`` -- RREF and basis without the
  RREF leaving the device; over F_p the basis is in residues (-1 is p - 1).
* ``rref_append(rref, pivots, new_rows, p)`` -- the RREF of the stacked rows
  from the RREF of the old ones (the grow-and-retry pattern of
  linac/vector_spaces/over_function_fields.py:74-101 without re-reducing).
* ``pivot_columns_from_row_reduced_echelon_form``,
  ``non_pivot_columns_from_row_reduced_echelon_form``,
  ``drop_bottom_zero_rows``, ``row_reduced_echelon_form_from_canonical_kernel``:
  host helpers with linac's semantics.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .row_reduce import _as_field_array, field_dtype


def _is_one(row) -> np.ndarray:
    row = np.asarray(row)
    if row.dtype.kind in "fc" or row.dtype == object:
        try:
            return np.isclose(row.astype(complex), 1)
        except TypeError:
            return row == 1
    return row == 1


def pivot_columns_from_row_reduced_echelon_form(rref) -> list[int]:
    """First entry equal to 1 in every row (rows are the non-zero RREF rows)."""
    rref = np.asarray(rref)
    return [int(np.flatnonzero(_is_one(rref[i]))[0]) for i in range(rref.shape[0])]


def non_pivot_columns_from_row_reduced_echelon_form(rref) -> list[int]:
    piv = set(pivot_columns_from_row_reduced_echelon_form(rref))
    return [c for c in range(np.asarray(rref).shape[1]) if c not in piv]


def drop_bottom_zero_rows(rref):
    """Remove trailing rows whose largest |entry| is below 1 (zero rows of an RREF)."""
    rref = np.asarray(rref)
    r = rref.shape[0]
    while r > 0:
        mx = float(np.abs(rref[r - 1]).max()) if rref.shape[1] else 0.0
        if mx > 1 or np.isclose(mx, 1):
            break
        r -= 1
    return rref[:r]


def row_reduced_echelon_form_from_canonical_kernel(kernel):
    """Inverse of canonical_kernel_from_row_reduced_echelon_form: the RREF whose
    null space the canonical basis spans."""
    K = np.asarray(kernel)
    n, q = K.shape
    nonpiv = []
    for j in range(q):
        col = K[:, j]
        hits = np.flatnonzero(np.isclose(col.astype(complex), -1)) if col.dtype.kind in "fc" else np.flatnonzero(col == -1)
        nonpiv.append(int(hits[-1]))
    piv = [c for c in range(n) if c not in set(nonpiv)]
    out = np.zeros((n - q, n), dtype=np.result_type(K.dtype, int))
    out[np.arange(n - q), piv] = 1
    out[:, nonpiv] = K[piv, :]
    return out


def _kernel_device(dR, r: int, n: int, code: int, p: int, pivots, dt, stream) -> np.ndarray:
    q = n - r
    K = np.empty((n, max(q, 0)), dtype=dt)
    if q <= 0:
        return K
    d_piv = _lib.DeviceBuffer(8 * max(r, 1))
    if r:
        d_piv.upload(np.asarray(pivots, dtype=np.int64), stream.handle)
    dK = _lib.DeviceBuffer(K.nbytes)
    _lib.check(_lib.lib().lnc_canonical_kernel_device(code, r, n, p, dR.ptr, n, d_piv.ptr, dK.ptr, q, stream.handle),
               "lnc_canonical_kernel_device")
    dK.download(K, stream.handle)
    stream.synchronize()
    return K


def canonical_kernel_from_row_reduced_echelon_form(row_reduced_echelon_form):
    """Canonical null-space basis of an RREF without zero rows (linac's function, on the device)."""
    R = np.asarray(row_reduced_echelon_form)
    r, n = R.shape
    pivots = pivot_columns_from_row_reduced_echelon_form(R)
    out_dtype = np.result_type(R.dtype, int)
    if R.dtype.kind == "u":
        dt = np.uint64 if R.dtype.itemsize > 4 else np.uint32
        code, marker_p = (_lib.LNC_U64, 0) if dt == np.uint64 else (_lib.LNC_U32, 2**32)
    elif R.dtype.kind == "c" or R.dtype == object:
        return _host_kernel(R, pivots)
    else:
        dt, code, marker_p = np.float64, _lib.LNC_F64, 0
        if R.dtype != np.float64:
            return _host_kernel(R, pivots)
    host = np.ascontiguousarray(R, dtype=dt)
    stream = _lib.Stream()
    dR = _lib.DeviceBuffer(max(host.nbytes, 1))
    if host.size:
        dR.upload(host, stream.handle)
    K = _kernel_device(dR, r, n, code, marker_p, pivots, dt, stream)
    if dt == np.float64:
        return K
    marker = np.iinfo(dt).max
    out = K.astype(out_dtype)
    out[K == marker] = -1
    return out


def _host_kernel(R, pivots):
    """Complex / object RREFs: the same construction on the host."""
    r, n = R.shape
    nonpiv = [c for c in range(n) if c not in set(pivots)]
    K = np.zeros((n, n - r), dtype=np.result_type(R.dtype, int))
    K[pivots, :] = R[:, nonpiv]
    K[nonpiv, np.arange(n - r)] = -1
    return K


def null_space(matrix, field_characteristic: int = 0, return_pivots: bool = False):
    """Canonical null-space basis of `matrix` over F_p (p > 0) or the reals /
    complex numbers (p = 0): RREF and basis on the device, one download."""
    A = np.asarray(matrix)
    p = int(field_characteristic)
    dt = field_dtype(A, p)
    host = np.ascontiguousarray(_as_field_array(A, dt))
    m, n = host.shape
    code = _lib.DTYPE_CODE[np.dtype(dt)]
    stream = _lib.Stream()
    nbytes = max(host.nbytes, 1)
    d_in, d_R = _lib.DeviceBuffer(nbytes), _lib.DeviceBuffer(nbytes)
    kmax = max(min(m, n), 1)
    d_piv, d_rank = _lib.DeviceBuffer(8 * kmax), _lib.DeviceBuffer(8)
    if host.size:
        d_in.upload(host, stream.handle)
    _lib.check(_lib.lib().lnc_rref_device(code, m, n, p, 1e-9, d_in.ptr, n, d_R.ptr, n, d_piv.ptr, d_rank.ptr,
                                          stream.handle, 0), "lnc_rref_device")
    rank = np.zeros(1, dtype=np.int64)
    piv = np.empty(kmax, dtype=np.int64)
    d_rank.download(rank, stream.handle)
    d_piv.download(piv, stream.handle)
    stream.synchronize()
    r = int(rank[0])
    q = n - r
    K = np.empty((n, q), dtype=dt)
    if q > 0:
        dK = _lib.DeviceBuffer(K.nbytes)
        _lib.check(_lib.lib().lnc_canonical_kernel_device(code, r, n, p, d_R.ptr, n, d_piv.ptr, dK.ptr, q,
                                                          stream.handle), "lnc_canonical_kernel_device")
        dK.download(K, stream.handle)
        stream.synchronize()
    if return_pivots:
        return K, [int(x) for x in piv[:r]]
    return K


def rref_append(rref, pivots, new_rows, field_characteristic: int, return_pivots: bool = False):
    """RREF over F_p (p < 2^32) of the rows behind `rref` (its non-zero rows,
    pivot columns `pivots`) stacked with `new_rows`, computed from `rref`:
    the new rows are reduced by the old pivots, row-reduced among themselves,
    and the old rows are cleared in the new pivot columns (two tensor-core
    products and a k-row RREF).  Returns an (r + k) x n uint32 array."""
    p = int(field_characteristic)
    R = np.ascontiguousarray(np.asarray(rref, dtype=np.uint32))
    N = np.ascontiguousarray(np.asarray(new_rows).astype(np.uint64) % np.uint64(p)).astype(np.uint32)
    pv = [int(x) for x in pivots]
    r = len(pv)
    R = R[:r]
    k, n = N.shape
    if R.shape[1] != n and r:
        raise ValueError("old and new rows differ in width")
    stream = _lib.Stream()
    dR = _lib.DeviceBuffer(max(R.nbytes, 1))
    dN = _lib.DeviceBuffer(max(N.nbytes, 1))
    dP = _lib.DeviceBuffer(8 * max(r, 1))
    dO = _lib.DeviceBuffer(4 * max((r + k) * n, 1))
    dOP = _lib.DeviceBuffer(8 * max(r + k, 1))
    dRk = _lib.DeviceBuffer(8)
    if R.size:
        dR.upload(R, stream.handle)
    if N.size:
        dN.upload(N, stream.handle)
    if r:
        dP.upload(np.asarray(pv, dtype=np.int64), stream.handle)
    _lib.check(_lib.lib().lnc_rref_append_device(_lib.LNC_U32, r, k, n, p, dR.ptr, n, dP.ptr, dN.ptr, n, dO.ptr, n,
                                                 dOP.ptr, dRk.ptr, stream.handle), "lnc_rref_append_device")
    out = np.empty((r + k, n), dtype=np.uint32)
    rank = np.zeros(1, dtype=np.int64)
    piv = np.empty(max(r + k, 1), dtype=np.int64)
    if out.size:
        dO.download(out, stream.handle)
    dRk.download(rank, stream.handle)
    dOP.download(piv, stream.handle)
    stream.synchronize()
    if return_pivots:
        return out, [int(x) for x in piv[:int(rank[0])]]
    return out
