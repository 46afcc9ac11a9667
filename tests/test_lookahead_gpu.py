"""Look-ahead of the candidate-panel path: the next panel runs on a second
stream while the caller's stream applies the current panel to the columns
beyond it.  Forced on small shapes (LNC_FLAG_LOOKAHEAD) the results must stay
bit-identical to the oracle, including panels the candidate block misses
(their exhaustive redo corrects the near columns before the fork and the far
columns after it) and rank-deficient inputs; at sizes where it is on by
default it must agree bit for bit with the single-stream schedule."""
import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads
from linac_gb300.row_reduce import rref_host_call

pytestmark = pytest.mark.gpu

LA = _lib.LNC_FLAG_LOOKAHEAD


def _check(A, p, flags):
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=flags)
    R_ref, piv_ref, rank_ref = oracle.rref_modp(A, p)
    assert np.array_equal(out.astype(np.uint64), R_ref)
    assert piv == list(piv_ref) and rank == rank_ref


@pytest.mark.parametrize("m,n,p", [(700, 900, 2**31 - 1), (900, 700, 4294967291), (520, 400, 2)])
def test_u32_random(m, n, p):
    rng = np.random.default_rng(m + 3 * n)
    A = (rng.integers(0, p, size=(m, n), dtype=np.uint64)).astype(np.uint32)
    _check(A, p, LA)


@pytest.mark.parametrize("m,n,r,p", [(900, 700, None, 2**31 - 1), (1100, 1300, 777, 4294967291),
                                     (800, 1000, 300, 2**31 - 19)])
def test_u32_missed_pivots_and_rank_deficiency(m, n, r, p):
    """Leading rows zero in the leading columns make the candidate block miss
    pivots; zero columns and a low rank exercise empty and partial panels."""
    rng = np.random.default_rng(m * n)
    if r is None:
        A = rng.integers(0, p, size=(m, n), dtype=np.uint64)
    else:
        A = workloads.rank_deficient_modp(m, n, r, p, rng)
    A[: m // 2, :60] = 0
    A[:, 200:205] = 0
    A[: m // 3, 300:420] = 0
    _check(A.astype(np.uint32), p, LA)


@pytest.mark.parametrize("m,n,p", [(700, 900, 2**61 - 1), (600, 500, 2**64 - 59)])
def test_u64_random_and_missed(m, n, p):
    rng = np.random.default_rng(m * 5 + n)
    A = rng.integers(0, 2**63, size=(m, n), dtype=np.uint64) % np.uint64(p)
    _check(A.copy(), p, LA)
    A[: m // 2, :80] = 0
    A[:, 200:205] = 0
    A[: m // 3, 260:330] = 0
    _check(A, p, LA)


@pytest.mark.parametrize("m,n,p", [(40, 2000, 2**31 - 1), (3000, 300, 4294967291), (161, 700, 2**61 - 1),
                                   (7, 1300, 2)])
def test_extreme_aspect_ratios(m, n, p):
    """Short-wide (fewer rows than a candidate block: the block holds every
    remaining row) and tall-skinny inputs, and a ragged last panel."""
    rng = np.random.default_rng(m + n)
    dt = np.uint64 if p > 2**32 else np.uint32
    A = (rng.integers(0, 2**62, size=(m, n), dtype=np.uint64) % np.uint64(p)).astype(dt)
    A[:, 130:140] = 0
    _check(A, p, LA)


def test_deferred_fallback_reports_a_miss_with_lookahead():
    p = 2**31 - 1
    rng = np.random.default_rng(5)
    A = rng.integers(0, p, size=(900, 700), dtype=np.uint64).astype(np.uint32)
    _check(A, p, LA | _lib.LNC_FLAG_DEFER_FALLBACK)  # no miss: exact result
    A[:450, :60] = 0
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=LA | _lib.LNC_FLAG_DEFER_FALLBACK)
    assert rank == -1


@pytest.mark.parametrize("dtype,p", [(np.uint32, 2**31 - 1), (np.uint64, 2**61 - 1)])
def test_default_lookahead_matches_single_stream(dtype, p):
    """2048 x 2304 (on by default there): identical outputs with and without
    the look-ahead, identity in the pivot block, and a checksum of the
    non-pivot block that the oracle reproduces from a few rows."""
    m, n = 2048, 2304
    rng = np.random.default_rng(11)
    A = (rng.integers(0, 2**63, size=(m, n), dtype=np.uint64) % np.uint64(p)).astype(dtype)
    out_la = np.empty_like(A)
    out_1s = np.empty_like(A)
    piv_la, rank_la = rref_host_call(A, p, out_la, flags=0)
    piv_1s, rank_1s = rref_host_call(A, p, out_1s, flags=_lib.LNC_FLAG_NO_LOOKAHEAD)
    assert rank_la == rank_1s == m and piv_la == piv_1s == list(range(m))
    assert np.array_equal(out_la, out_1s)
    assert np.array_equal(out_la[:, :m], np.eye(m, dtype=dtype))
    # row i of the RREF solves A[:, :m] X = A[:, m:]: check A[:8] @ X == A[:8, m:] mod p
    X = out_la[:, m:].astype(np.uint64)
    lhs = oracle.matmul_modp(A[:8, :m].astype(np.uint64), X, p)
    assert np.array_equal(lhs, A[:8, m:].astype(np.uint64))
