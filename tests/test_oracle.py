"""Pin the CPU oracle (oracle/rref_oracle.c) against the reference.

Every case here compares the oracle with outputs of linac's own CPU code
(committed fixtures from tests/golden/make_golden.py) or with the reference's
stored golden vector (tests/test_row_reduce_random_cuda.py:52-63).  When the
reference checkout is present, a few extra cases run the reference live.
"""
import hashlib

import numpy as np
import pytest

import fixtures
import oracle
from linac_gb300 import workloads


@pytest.mark.parametrize("case", fixtures.modp_cases(), ids=lambda c: c[0])
def test_oracle_modp_matches_reference_fixture(case):
    name, A, p, R_ref, piv_ref = case
    R, piv, rank = oracle.rref_modp(A, p)
    assert np.array_equal(R, R_ref), name
    assert piv == piv_ref
    assert rank == len(piv_ref)


@pytest.mark.parametrize("case", fixtures.float_cases(), ids=lambda c: c[0])
def test_oracle_float_matches_reference_fixture(case):
    name, A, R_ref = case
    if np.iscomplexobj(A):
        R, _, _ = oracle.rref_c128(A)
    else:
        R, _, _ = oracle.rref_f64(A)
    # same operations in the same order: agreement to the last few ulps
    assert np.allclose(R, R_ref, rtol=0, atol=1e-12), name


def test_oracle_config1_matches_reference_hash():
    meta = fixtures.config1()
    A, p = workloads.config1()
    assert hashlib.sha256(A.tobytes()).hexdigest() == meta["input_sha256_u32"]
    R, piv, rank = oracle.rref_modp(A, p)
    R32 = R.astype(np.uint32)
    assert hashlib.sha256(R32.tobytes()).hexdigest() == meta["rref_sha256_u32"]
    assert piv == meta["pivots"] and rank == meta["rank"] == 384


def test_oracle_known_result_4096():
    """The reference's stored golden vector: last RREF column of the seed-0
    4096 x 4097 matrix mod 2^31-19."""
    A, p = fixtures.golden_4096_input()
    R, piv, rank = oracle.rref_modp(A, p)
    known = fixtures.known_result_4096()
    assert rank == 4096
    assert np.array_equal(R[:, -1].astype(np.uint32), known)


@pytest.mark.parametrize("size", ["small", "medium"])
def test_oracle_nullspace_fixtures_pivots(size):
    fx = fixtures.nullspace(size)
    R, piv, rank = oracle.rref_modp(fx["A"], int(fx["p"][0]))
    assert piv == [int(x) for x in fx["known_pivots"]]
    assert (rank, R.shape[1]) == tuple(int(x) for x in fx["rref_shape"])
    assert np.array_equal(R.astype(np.uint32), fx["R"])


def test_oracle_nonprime_raises():
    A = np.array([[2, 1], [1, 1]], dtype=np.uint64)
    with pytest.raises(ZeroDivisionError):
        oracle.rref_modp(A, 4)


def test_oracle_loader_matches_reference_fixture():
    prefactors, ansatze, cases = fixtures.loader_cases()
    from linac_gb300 import matrix_loader
    for fname, p, pts, As_ref in cases:
        bases, lind_list = matrix_loader.build_bases_and_indices(prefactors, ansatze, pts)
        for t, (A_ref, lind) in enumerate(zip(As_ref, lind_list)):
            if lind.shape[0] == 0:
                continue
            if p > 0:
                b = np.array([[int(v) for v in row] for row in bases[t]], dtype=np.uint64)
                out = oracle.load_modp(b, lind, p)
                assert np.array_equal(out, A_ref.astype(np.uint64)), (fname, t)
            else:
                out = oracle.load_float(np.asarray(bases[t], dtype=complex if fname == "mpc" else float), lind)
                assert np.array_equal(out, A_ref), (fname, t)


def test_oracle_matmul_modp_matches_numpy_split():
    rng = np.random.default_rng(3)
    p = 2**31 - 1
    B = rng.integers(0, p, size=(37, 19), dtype=np.uint64)
    C = rng.integers(0, p, size=(19, 23), dtype=np.uint64)
    assert np.array_equal(oracle.matmul_modp(B, C, p), workloads.matmul_modp(B, C, p).astype(np.uint64))


def test_reference_live_small_cases():
    """Cross-check with the reference itself when its checkout is present."""
    import reference_import as ri
    if not ri.reference_available():
        pytest.skip("reference checkout not present")
    row_reduce = ri.reference_row_reduce()
    rng = np.random.default_rng(99)
    for p in (2**31 - 1, 65521, 3):
        for shape in ((13, 13), (9, 21), (21, 9)):
            A = rng.integers(0, p, size=shape, dtype=np.int64)
            Rr, _ = row_reduce(A.copy(), pivoting=1, scaling=False, threshold=0, prime=p)
            Ro, _, _ = oracle.rref_modp(A, p)
            assert np.array_equal(Rr.astype(np.uint64), Ro)
        # pivoting=0 (the reference GPU tests' CPU call) agrees on generic input
        A = rng.integers(0, p, size=(15, 15), dtype=np.int64)
        R0, _ = row_reduce(A.copy(), pivoting=0, scaling=False, threshold=0, prime=p)
        Ro, _, _ = oracle.rref_modp(A, p)
        if p > 1000:
            assert np.array_equal(R0.astype(np.uint64), Ro)
