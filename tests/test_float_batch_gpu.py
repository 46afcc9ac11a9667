"""Batched float64 / complex128 RREF (lnc_rref_float_batch): uneven matrices
solved concurrently by host workers on their own streams.  Every result must
equal, bit for bit, the single-matrix call on the same input (the same
kernels run; concurrency changes only their order on the GPU), be within the
float bound of the FP64-accurate reference solution, and carry its own
mixed-precision report."""
import numpy as np
import pytest

import oracle
from linac_gb300 import cuda_row_reduce, workloads
from linac_gb300.batch import rref_float_batch

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _systems(ns, cplx, seed, q=8):
    rng = np.random.default_rng(seed)
    mats, parts = [], []
    for n in ns:
        A = workloads.conditioned_matrix(n, rng, cond=1e5, complex_=cplx)
        B = rng.standard_normal((n, q)) + (1j * rng.standard_normal((n, q)) if cplx else 0)
        mats.append(np.hstack([A, B]))
        parts.append((A, B))
    return mats, parts


@pytest.mark.parametrize("cplx", [False, True])
def test_mixed_batch_equals_single_calls_and_meets_bound(cplx):
    ns = [130, 700, 257, 64, 512, 390, 1000, 33] if not cplx else [130, 400, 257, 64, 300]
    mats, parts = _systems(ns, cplx, seed=17 + cplx)
    res, pivs, reps = rref_float_batch(mats, mixed=True, workers=4, return_pivots=True, return_reports=True)
    for M, R, piv, rep, (A, B) in zip(mats, res, pivs, reps, parts):
        n = A.shape[0]
        R1, piv1 = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
        assert piv == piv1 == list(range(n))
        assert np.array_equal(R, R1)
        assert np.array_equal(R[:, :n], np.eye(n))
        assert _rel(R[:, n:], oracle.reference_solution(A, B)) <= TOL
        assert not rep["redone_fp64"] and rep["error_estimate"] is not None and rep["error_estimate"] <= 4 * TOL


def test_fp64_batch_equals_single_calls():
    rng = np.random.default_rng(5)
    mats = [rng.standard_normal((m, n)) for m, n in ((300, 320), (50, 900), (700, 200), (128, 128))]
    res, pivs = rref_float_batch(mats, mixed=False, workers=3, return_pivots=True)
    for M, R, piv in zip(mats, res, pivs):
        R1, piv1 = cuda_row_reduce(M, 0, return_pivots=True)
        assert piv == piv1 and np.array_equal(R, R1)
        R_o, piv_o, _ = oracle.rref_f64(M)
        assert piv == list(piv_o)
        assert np.allclose(R, R_o, rtol=1e-9, atol=1e-9)


def test_rank_deficient_member_is_redone_in_fp64():
    rng = np.random.default_rng(9)
    low = rng.standard_normal((300, 120)) @ rng.standard_normal((120, 280))
    mats = [rng.standard_normal((200, 210)), low, rng.standard_normal((90, 95))]
    res, pivs, reps = rref_float_batch(mats, mixed=True, workers=2, return_pivots=True, return_reports=True)
    assert reps[1]["redone_fp64"] and reps[1]["error_estimate"] is None
    assert len(pivs[1]) == 120
    R1, piv1 = cuda_row_reduce(low, 0, return_pivots=True)
    assert np.array_equal(res[1], R1) and pivs[1] == piv1
