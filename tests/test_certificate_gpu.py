"""Exact certificates of large solves, where an oracle elimination would take
too long on the CPU.

An augmented system [A | B] with A square and non-singular over F_p has the
RREF [I | X] with X = A^-1 B, so `A X = B (mod p)` certifies every entry of X
exactly.  The product is formed twice: on the CPU by the oracle's exact
matrix product (all rows), and on the device by lnc_matmul_modp_device.  This
is the check the reference applies to its own large case, a 4096 x 4097
augmented matrix whose last column is compared with a stored vector
(tests/test_row_reduce_random_cuda.py:52-63); here the sizes run all panels
of the look-ahead schedule (two streams) and its 64-bit counterpart.
"""
import hashlib

import numpy as np
import pytest

import oracle
from linac_gb300 import _lib
from linac_gb300.row_reduce import rref_host_call

pytestmark = pytest.mark.gpu


def _augmented(m, q, p, seed):
    rng = np.random.default_rng(seed)
    dt = np.uint64 if p > 2**32 else np.uint32
    return (rng.integers(0, 2**63, size=(m, m + q), dtype=np.uint64) % np.uint64(p)).astype(dt)


def _device_product(code, A_host, X_host, p):
    """A X mod p through the C ABI (device buffers, library matmul)."""
    L = _lib.lib()
    m, k = A_host.shape
    q = X_host.shape[1]
    elt = A_host.dtype.itemsize
    s = _lib.Stream()
    dA, dX, dC = _lib.DeviceBuffer(A_host.nbytes), _lib.DeviceBuffer(X_host.nbytes), _lib.DeviceBuffer(elt * m * q)
    dA.upload(A_host, s.handle)
    dX.upload(X_host, s.handle)
    _lib.check(L.lnc_matmul_modp_device(code, m, k, q, p, dA.ptr, k, dX.ptr, q, dC.ptr, q, s.handle))
    C = np.empty((m, q), dtype=A_host.dtype)
    dC.download(C, s.handle)
    return C


def _certify(M, p, flags):
    m = M.shape[0]
    q = M.shape[1] - m
    out = np.empty_like(M)
    piv, rank = rref_host_call(M, p, out, flags=flags)
    assert rank == m and piv == list(range(m))
    left = out[:, :m]
    assert np.all(np.diagonal(left) == 1) and int(np.count_nonzero(left)) == m
    A, B, X = M[:, :m], M[:, m:], np.ascontiguousarray(out[:, m:])
    AX = oracle.matmul_modp(A, X, p)
    assert np.array_equal(AX, B.astype(np.uint64)), "A X != B (mod p) on the CPU"
    code = _lib.LNC_U64 if M.dtype == np.uint64 else _lib.LNC_U32
    AXd = _device_product(code, np.ascontiguousarray(A), X, p)
    assert np.array_equal(AXd, B), "A X != B (mod p) on the device"
    return hashlib.sha256(X.tobytes()).hexdigest()


def test_u32_8192_augmented_lookahead():
    """8192 x 8208 mod 2^31-1: 65 panels, look-ahead on (it is the default at
    this size; the flag makes it explicit), certificate over all rows, and the
    same X on a second solve."""
    p = 2**31 - 1
    M = _augmented(8192, 16, p, seed=8192)
    h1 = _certify(M, p, _lib.LNC_FLAG_LOOKAHEAD)
    h2 = _certify(M, p, _lib.LNC_FLAG_LOOKAHEAD)
    assert h1 == h2


def test_u32_8192_augmented_one_stream_matches():
    """The one-stream schedule gives the same X as the look-ahead."""
    p = 2**31 - 1
    M = _augmented(8192, 16, p, seed=8192)
    assert _certify(M, p, _lib.LNC_FLAG_NO_LOOKAHEAD) == _certify(M, p, _lib.LNC_FLAG_LOOKAHEAD)


def test_u64_4096_augmented_lookahead():
    """4096 x 4112 mod 2^61-1 on the eight-digit limb contraction with the
    64-column cluster panels and the look-ahead."""
    p = 2**61 - 1
    M = _augmented(4096, 16, p, seed=4096)
    h1 = _certify(M, p, _lib.LNC_FLAG_LOOKAHEAD)
    h2 = _certify(M, p, _lib.LNC_FLAG_LOOKAHEAD)
    assert h1 == h2


@pytest.mark.parametrize("m,k,n,p", [(37, 300, 5, 2**61 - 1), (300, 17, 40, 2**64 - 59), (64, 64, 64, 4294967311)])
def test_u64_device_matmul_vs_oracle(m, k, n, p):
    rng = np.random.default_rng(m + k + n)
    A = rng.integers(0, 2**63, size=(m, k), dtype=np.uint64) % np.uint64(p)
    B = rng.integers(0, 2**63, size=(k, n), dtype=np.uint64) % np.uint64(p)
    assert np.array_equal(_device_product(_lib.LNC_U64, A, B, p), oracle.matmul_modp(A, B, p))
