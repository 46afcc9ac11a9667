"""The no-allocation RREF entry point, lnc_rref_device_noalloc.

Callers that cannot allocate device memory when they need an RREF -- a host
framework that reserved all of HBM for its own pool allocator, or a
latency-critical thread that must not wait on an allocator -- use this entry
point: its scratch is a fixed 16 MiB array inside the library, not
stream-ordered allocations.  These tests check, through the C ABI, that it
returns exactly what the allocating entry point (lnc_rref_device) returns, on
two calls in a row (the second call reuses the array the first one left
dirty), that both agree with the CPU oracle (so a scratch-layout fault the two
entry points share would not pass), and that a request too large for the
fixed array, or with overlapping input and output, is refused.

This file is named so that pytest collects it last; it is self-contained and
passes on its own in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu

_i64, _u64, _vp, _int, _dbl = ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int, ctypes.c_double


def _noalloc():
    return _lib.bind("lnc_rref_device_noalloc",
                     [_int, _i64, _i64, _u64, _dbl, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _int])


def _run(entry, dtype_code, A, p, tol, stream):
    """Upload A, run one device RREF entry point, return (R, pivots, rank)."""
    m, n = A.shape
    d_work = _lib.DeviceBuffer(A.nbytes)
    d_out = _lib.DeviceBuffer(A.nbytes)
    d_piv = _lib.DeviceBuffer(8 * min(m, n))
    d_rank = _lib.DeviceBuffer(8)
    d_work.upload(A, stream.handle)
    rc = entry(dtype_code, m, n, p, tol, d_work.ptr, n, d_out.ptr, n, d_piv.ptr, d_rank.ptr, stream.handle, 0)
    _lib.check(rc, "rref")
    stream.synchronize()
    _lib.device_status()
    R = np.empty_like(A)
    d_out.download(R, stream.handle)
    piv = np.empty(min(m, n), dtype=np.int64)
    d_piv.download(piv, stream.handle)
    rank = np.empty(1, dtype=np.int64)
    d_rank.download(rank, stream.handle)
    return R, piv, int(rank[0])


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    if _lib.device_count() < 1:
        pytest.skip("no CUDA device")
    noalloc = _noalloc()
    alloc = _lib.lib().lnc_rref_device
    stream = _lib.Stream()
    p = 2**31 - 1
    rng = np.random.default_rng(2024)
    inputs = [workloads.rank_deficient_modp(700, 900, 611, p, rng).astype(np.uint32),
              rng.integers(0, p, size=(1000, 1030), dtype=np.uint32)]
    for A in inputs:  # two calls in a row on the shared array
        R_ref, piv_ref, rank_ref = _run(alloc, _lib.LNC_U32, A, p, 0.0, stream)
        R, piv, rank = _run(noalloc, _lib.LNC_U32, A, p, 0.0, stream)
        # residues mod p: the tolerance is zero, results must be identical
        assert rank == rank_ref
        assert np.array_equal(piv, piv_ref)
        assert np.array_equal(R, R_ref)
        R_o, piv_o, rank_o = oracle.rref_modp(A, p)
        assert rank == rank_o and list(piv[:rank]) == list(piv_o)
        assert np.array_equal(R.astype(np.uint64), R_o)


def test_noalloc_float_matches_allocating_entry_point():
    if _lib.device_count() < 1:
        pytest.skip("no CUDA device")
    noalloc = _noalloc()
    alloc = _lib.lib().lnc_rref_device
    stream = _lib.Stream()
    rng = np.random.default_rng(7)
    A = np.hstack([workloads.conditioned_matrix(300, rng, 1e3), rng.standard_normal((300, 8))])
    A = np.ascontiguousarray(A)
    R_ref, piv_ref, rank_ref = _run(alloc, _lib.LNC_F64, A, 0, 1e-9, stream)
    R, piv, rank = _run(noalloc, _lib.LNC_F64, A, 0, 1e-9, stream)
    assert rank == rank_ref and np.array_equal(piv, piv_ref)
    # same kernels on the same inputs: agreement to 1e-12 (the float tests' bar is 1e-9)
    assert np.allclose(R, R_ref, rtol=0, atol=1e-12)
    # and the FP64 oracle (linac's CPU row_reduce, pivoting=1, scaling=True): the float tests' 1e-9
    R_o, piv_o, rank_o = oracle.rref_f64(A)
    assert rank == rank_o and list(piv[:rank]) == list(piv_o)
    assert np.allclose(R, R_o, rtol=1e-9, atol=1e-9)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    if _lib.device_count() < 1:
        pytest.skip("no CUDA device")
    noalloc = _noalloc()
    dummy = _lib.DeviceBuffer(16)
    rc = noalloc(_lib.LNC_U32, 40000, 40000, 2**31 - 1, 0.0, dummy.ptr, 40000, dummy.ptr + 8, 40000,
                 None, None, None, 0)
    assert rc == _lib.LNC_ERR_INVALID
    assert "no-allocation scratch" in _lib.last_error()
    rc = noalloc(_lib.LNC_U32, 10, 10, 2**31 - 1, 0.0, dummy.ptr, 10, dummy.ptr, 10, None, None, None, 0)
    assert rc == _lib.LNC_ERR_INVALID  # in place is refused: output must be a separate buffer
    assert "do not overlap" in _lib.last_error()
    # a partial overlap (the output starts inside the input) is refused as well
    rc = noalloc(_lib.LNC_U32, 2, 2, 2**31 - 1, 0.0, dummy.ptr, 2, dummy.ptr + 8, 2, None, None, None, 0)
    assert rc == _lib.LNC_ERR_INVALID and "do not overlap" in _lib.last_error()
