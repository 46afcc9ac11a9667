"""Mixed-precision float RREF (LNC_FLAG_MIXED): fixed-point tensor-core
trailing updates, FP64 panels, FP64 refinement.

The bound is 1e-10 in the max norm relative to the result's largest entry.
Small systems are held to it against the FP64 oracle (linac's row_reduce
restated in C, pivoting=1, scaling=True, threshold 1e-9), with the same pivot
columns.  At the benchmark's sizes (2,000 and 5,000 unknowns, condition 1e6)
the FP64 oracle is itself about cond * eps ~ 1e-10 away from the exact
solution, so no result more accurate than the oracle can be within 1e-10 of
it; there the bound is held against the FP64-accurate reference solution of
the stored system (LAPACK refined with double-double residuals,
oracle.reference_solution), and the result's own error estimate
(mixed_report()["error_estimate"]) must be within it as well."""
import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads
from linac_gb300.row_reduce import cuda_row_reduce

pytestmark = pytest.mark.gpu

TOL = 1e-10  # max-norm error relative to the largest entry of the result


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _truth(A, B):
    """A^-1 B to FP64 accuracy (refined with double-double residuals)."""
    return oracle.reference_solution(A, B)


@pytest.mark.parametrize("n,cplx", [(300, False), (700, False), (257, True), (500, True)])
def test_conditioned_system_matches_fp64_oracle(n, cplx):
    rng = np.random.default_rng(n)
    A = workloads.conditioned_matrix(n, rng, cond=1e6, complex_=cplx)
    B = rng.standard_normal((n, 16)) + (1j * rng.standard_normal((n, 16)) if cplx else 0)
    M = np.hstack([A, B])
    R, piv = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
    rep = _lib.mixed_report()
    R_o, piv_o, rank_o = (oracle.rref_c128 if cplx else oracle.rref_f64)(M)
    assert piv == list(piv_o) == list(range(n))
    assert not rep["redone_fp64"] and rep["iterations"] >= 1
    assert _rel(R, R_o) <= TOL, (_rel(R, R_o), rep)
    X = _truth(A, B)
    assert _rel(R[:, n:], X) <= max(2.0 * _rel(R_o[:, n:], X), 1e-12)
    assert np.array_equal(R[:, :n], np.eye(n))


def test_wide_matrix_many_nonpivot_columns():
    rng = np.random.default_rng(7)
    M = rng.standard_normal((300, 900))
    R, piv = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
    R_o, piv_o, _ = oracle.rref_f64(M)
    assert piv == list(piv_o)
    assert _rel(R, R_o) <= TOL
    assert _lib.mixed_report()["iterations"] >= 1


def test_full_rank_square_and_tall_need_no_refinement():
    rng = np.random.default_rng(8)
    for shape in ((400, 400), (600, 350)):
        M = rng.standard_normal(shape)
        R, piv = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
        k = min(shape)
        assert piv == list(range(k))
        assert np.array_equal(R[:k], np.eye(*R[:k].shape)) and not R[k:].any()
        assert _lib.mixed_report()["iterations"] == 0


def test_rank_deficient_is_redone_in_fp64():
    """Dependent rows leave entries near the threshold after reduced-precision
    updates: the solve is redone in FP64 and equals the FP64 path exactly."""
    rng = np.random.default_rng(9)
    Bm = rng.standard_normal((400, 250))
    Cm = rng.standard_normal((250, 380))
    M = Bm @ Cm
    R_mixed, piv_mixed = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
    assert _lib.mixed_report()["redone_fp64"]
    R_fp64, piv_fp64 = cuda_row_reduce(M, 0, return_pivots=True)
    assert np.array_equal(R_mixed, R_fp64) and piv_mixed == piv_fp64
    R_o, piv_o, rank_o = oracle.rref_f64(M)
    assert rank_o == 250 and piv_fp64 == list(piv_o)


def test_mixed_rejects_prime_fields():
    with pytest.raises(ValueError):
        cuda_row_reduce(np.eye(3, dtype=np.uint32), 7, mixed=True)


@pytest.mark.parametrize("n,cplx", [(2000, False), (2000, True), (5000, False), (5000, True)])
def test_benchmark_sizes_within_bound_of_reference_solution(n, cplx):
    """[A | B] with A = U diag(s) V^H (cond 1e6) and 16 right-hand sides, as
    the float benchmark: the solution block within 1e-10 of the reference
    solution, the pivot block exactly I, the per-result error estimate within
    the bound and of the order of the measured error."""
    rng = np.random.default_rng(5000 + n + cplx)
    A = workloads.conditioned_matrix(n, rng, cond=1e6, complex_=cplx)
    B = rng.standard_normal((n, 16)) + (1j * rng.standard_normal((n, 16)) if cplx else 0)
    M = np.hstack([A, B])
    R, piv = cuda_row_reduce(M, 0, return_pivots=True, mixed=True)
    rep = _lib.mixed_report()
    assert piv == list(range(n)) and not rep["redone_fp64"]
    assert np.array_equal(R[:, :n], np.eye(n))
    X = _truth(A, B)
    err = _rel(R[:, n:], X)
    assert err <= TOL, (err, rep)
    # the estimate (one further FP64-residual correction) is of the order of the error: at
    # condition 1e6 both sit at the FP64 floor cond * eps, the estimate somewhat above
    est = rep["error_estimate"]
    assert est is not None and est / 4.0 <= err + 1e-15 and err <= 4.0 * est, (err, est)
