"""Null spaces on the device (csrc/kernel_space.cu, linac_gb300/linear_algebra.py),
after tests/test_null_space.py of the reference: RREF -> canonical kernel
shapes, pivots and the kernel -> RREF round trip on the reference's own
fixture matrices, plus R K = 0 / A K = 0 on random rank-deficient input."""
import numpy as np
import pytest

import oracle
import fixtures
from linac_gb300 import workloads
from linac_gb300.linear_algebra import (canonical_kernel_from_row_reduced_echelon_form, drop_bottom_zero_rows,
                                        non_pivot_columns_from_row_reduced_echelon_form, null_space,
                                        pivot_columns_from_row_reduced_echelon_form,
                                        row_reduced_echelon_form_from_canonical_kernel)
from linac_gb300.row_reduce import cuda_row_reduce

pytestmark = pytest.mark.gpu


def _host_canonical_kernel(R):
    """The construction of linac/linear_algebra_tools.py:54-63, restated."""
    piv = pivot_columns_from_row_reduced_echelon_form(R)
    non = non_pivot_columns_from_row_reduced_echelon_form(R)
    K = np.zeros((R.shape[1], R.shape[1] - R.shape[0]), dtype=np.result_type(R.dtype, int))
    K[piv, :] = R[:, non]
    K[non, np.arange(len(non))] = -1
    return K


@pytest.mark.parametrize("size,rref_shape,ck_shape", [("small", (6, 7), (7, 1)), ("medium", (31, 86), (86, 55))])
def test_reference_fixture_kernels(size, rref_shape, ck_shape):
    fx = fixtures.nullspace(size)
    p = int(fx["p"][0])
    R = drop_bottom_zero_rows(cuda_row_reduce(fx["A"], p))
    K = canonical_kernel_from_row_reduced_echelon_form(R)
    assert R.shape == rref_shape and K.shape == ck_shape
    assert K.dtype == np.result_type(R.dtype, int)
    assert np.array_equal(K, _host_canonical_kernel(R))
    assert np.array_equal(row_reduced_echelon_form_from_canonical_kernel(K).astype(np.int64), R.astype(np.int64))
    assert pivot_columns_from_row_reduced_echelon_form(R) == [int(x) for x in fx["known_pivots"]]


@pytest.mark.parametrize("m,n,r,p", [(300, 420, 250, 2**31 - 1), (200, 200, 150, 65521), (150, 260, 90, 2**61 - 1)])
def test_null_space_annihilates_matrix(m, n, r, p):
    rng = np.random.default_rng(m + n + r)
    B = rng.integers(0, 2**62, size=(m, r), dtype=np.uint64) % np.uint64(p)
    C = rng.integers(0, 2**62, size=(r, n), dtype=np.uint64) % np.uint64(p)
    A = oracle.matmul_modp(B, C, p)
    if p < 2**32:
        A = A.astype(np.uint32)
    K, piv = null_space(A, p, return_pivots=True)
    assert K.shape == (n, n - r) and len(piv) == r
    AK = oracle.matmul_modp(A.astype(np.uint64), K.astype(np.uint64), p)
    assert not AK.any()
    R_o, piv_o, _ = oracle.rref_modp(A, p)
    assert piv == list(piv_o)
    K_host = _host_canonical_kernel(R_o[:r].astype(object)) % p  # exact integers (no float64 promotion)
    assert np.array_equal(K.astype(object), K_host)


def test_float_null_space_and_kernel():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((120, 40)) @ rng.standard_normal((40, 170))
    K = null_space(A, 0)
    assert K.shape == (170, 130)
    assert np.abs(A @ K).max() <= 1e-8 * np.abs(A).max() * np.abs(K).max() * 170
    R = drop_bottom_zero_rows(cuda_row_reduce(A, 0))
    assert np.array_equal(canonical_kernel_from_row_reduced_echelon_form(R), _host_canonical_kernel(R))


def test_full_rank_and_zero_matrix():
    p = 2**31 - 1
    rng = np.random.default_rng(4)
    A = rng.integers(0, p, size=(50, 50), dtype=np.uint64).astype(np.uint32)
    assert null_space(A, p).shape == (50, 0)
    Z = null_space(np.zeros((5, 7), dtype=np.uint32), p)
    assert np.array_equal(Z, (np.eye(7, dtype=np.uint64) * (p - 1)).astype(np.uint32))


@pytest.mark.parametrize("m,k,n,p", [(300, 80, 400, 2**31 - 1), (0, 50, 70, 65521), (120, 0, 90, 2**31 - 19),
                                     (200, 60, 500, 4294967291)])
def test_rref_append_equals_full_reduction(m, k, n, p):
    from linac_gb300.linear_algebra import rref_append
    rng = np.random.default_rng(m + k + n)
    A = (workloads.rank_deficient_modp(m, n, max(min(m, n) - 20, 0), p, rng) if m else
         np.zeros((0, n), dtype=np.uint64)).astype(np.uint64)
    B = rng.integers(0, p, size=(k, n), dtype=np.uint64)
    if k > 10 and m > 0:
        B[:5] = A[:5]            # dependent new rows
        B[5:10, :30] = 0         # and rows whose pivots come late
    R_A, piv_A, rank_A = oracle.rref_modp(A, p) if m else (np.zeros((0, n), dtype=np.uint64), [], 0)
    out, piv = rref_append(R_A[:rank_A], piv_A, B, p, return_pivots=True)
    R_full, piv_full, rank_full = oracle.rref_modp(np.vstack([A, B]), p)
    assert piv == list(piv_full)
    assert out.shape == (rank_A + k, n)  # the old matrix's zero rows are not carried
    assert np.array_equal(out[:rank_full].astype(np.uint64), R_full[:rank_full]) and not out[rank_full:].any()
