"""GPU parity of the RREF against the oracle and the reference's fixtures.

Mirrors linac's tests/test_row_reduce_random_cuda.py (identity checks,
the stored 4096 x 4097 golden vector) and tests/test_null_space.py (known
pivots), plus bit-exact comparison with the C oracle on rank-deficient,
ragged and edge-case inputs.  F_p results must be bit-identical; float
results are compared with the tolerance stated in each test.
"""
import ctypes
import hashlib

import numpy as np
import pytest

import fixtures
import oracle
from linac_gb300 import _lib, cuda_row_reduce, workloads
from linac_gb300.row_reduce import rref_host_call

pytestmark = pytest.mark.gpu


def _modp_ids(c):
    return c[0]


@pytest.mark.parametrize("case", fixtures.modp_cases(), ids=_modp_ids)
def test_modp_fixture_cases(case):
    name, A, p, R_ref, piv_ref = case
    R, piv = cuda_row_reduce(A, field_characteristic=p, return_pivots=True)
    assert R.dtype == (np.uint64 if p > 2**32 - 1 else np.uint32)
    assert np.array_equal(R.astype(np.uint64), R_ref), name
    assert piv == piv_ref


@pytest.mark.parametrize("case", [c for c in fixtures.modp_cases() if c[2] < 2**32][::3], ids=_modp_ids)
def test_modp_fixture_cases_simt_trailing(case):
    name, A, p, R_ref, piv_ref = case
    host = np.ascontiguousarray(A.astype(np.uint32))
    out = np.empty_like(host)
    piv, rank = rref_host_call(host, p, out, flags=_lib.LNC_FLAG_SIMT_TRAILING)
    assert np.array_equal(out.astype(np.uint64), R_ref)
    assert piv == piv_ref


def test_config1_hash_and_pivots():
    meta = fixtures.config1()
    A, p = workloads.config1()
    R, piv = cuda_row_reduce(A, field_characteristic=p, return_pivots=True)
    assert hashlib.sha256(R.tobytes()).hexdigest() == meta["rref_sha256_u32"]
    assert piv == meta["pivots"]


def test_known_result_4096():
    """tests/test_row_reduce_random_cuda.py:52-63 of the reference."""
    A, p = fixtures.golden_4096_input()
    R = cuda_row_reduce(A, p)
    assert np.array_equal(R[:, -1], fixtures.known_result_4096())
    assert np.array_equal(R[:, :-1], np.eye(4096, dtype=np.uint32))


@pytest.mark.parametrize("p,n", [(2**31 - 1, 1024), (2**31 - 1, 2048), (2**31 - 1, 3072),
                                 (2**31 + 11, 3072), (2**61 - 1, 2048)])
def test_random_square_is_identity(p, n):
    """tests/test_row_reduce_random_cuda.py:23-49 of the reference (F_p)."""
    rng = np.random.default_rng(n + p % 1000)
    A = rng.integers(0, p, size=(n, n), dtype=np.uint64)
    R = cuda_row_reduce(A, p)
    assert np.array_equal(R, np.identity(n, dtype=R.dtype))


@pytest.mark.parametrize("n", [1024, 2048])
def test_random_complex_is_identity(n):
    """tests/test_row_reduce_random_cuda.py:23-49 of the reference (complex)."""
    rng = np.random.default_rng(n)
    A = rng.random((n, n)) + 1j * rng.random((n, n))
    R = cuda_row_reduce(A, 0)
    assert R.dtype == np.complex128
    # same criterion as the reference test: numpy.isclose to the identity
    assert np.all(np.isclose(R - np.identity(n), 0))


@pytest.mark.parametrize("m,n,r,p", [(300, 400, 250, 2**31 - 1), (400, 300, 123, 2**31 - 19),
                                     (257, 513, 257, 2**31 + 11), (700, 700, 650, 65521),
                                     (129, 1100, 100, 2**31 - 1), (1100, 129, 90, 2**31 - 1),
                                     (50, 50, 0, 2**31 - 1), (33, 2000, 33, 3)])
def test_rank_deficient_vs_oracle(m, n, r, p):
    rng = np.random.default_rng(m * 7 + n)
    if r == 0:
        A = np.zeros((m, n), dtype=np.uint64)
    else:
        A = workloads.rank_deficient_modp(m, n, r, p, rng)
    R, piv = cuda_row_reduce(A, p, return_pivots=True)
    R_ref, piv_ref, rank_ref = oracle.rref_modp(A, p)
    if p > 2**16:  # over a small field B.C loses rank with noticeable probability
        assert rank_ref == min(r, m, n)
    assert np.array_equal(R.astype(np.uint64), R_ref)
    assert piv == piv_ref


@pytest.mark.parametrize("m,n,p", [(200, 260, 2**61 - 1), (260, 200, 2**61 + 15),
                                   (150, 150, 18446744073709551557)])
def test_u64_vs_oracle(m, n, p):
    rng = np.random.default_rng(m + n)
    A = rng.integers(0, 2**62, size=(m, n), dtype=np.uint64) % np.uint64(p)
    A[:, 3] = 0
    A[17] = A[5]
    R, piv = cuda_row_reduce(A, p, return_pivots=True)
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert R.dtype == np.uint64
    assert np.array_equal(R, R_ref)
    assert piv == piv_ref


def test_entries_above_p_are_reduced():
    p = 2**31 - 1
    rng = np.random.default_rng(5)
    A = rng.integers(0, 2**32, size=(40, 50), dtype=np.uint64)
    R = cuda_row_reduce(A.astype(np.uint32), p)
    R_ref, _, _ = oracle.rref_modp(A % p, p)
    assert np.array_equal(R.astype(np.uint64), R_ref)


@pytest.mark.parametrize("case", fixtures.float_cases(), ids=lambda c: c[0])
def test_float_fixture_cases(case):
    name, A, R_ref = case
    R = cuda_row_reduce(A, 0)
    # FP64 Gauss-Jordan on the GPU vs numpy's: 1e-9 absolute on entries of
    # magnitude <= ~1e3 (condition numbers of these fixtures are <= 1e3)
    assert np.allclose(R, R_ref, rtol=1e-9, atol=1e-9), name


@pytest.mark.parametrize("size", ["small", "medium"])
def test_nullspace_fixture_pivots(size):
    """tests/test_null_space.py:30-62 of the reference (F_p, use_cuda)."""
    fx = fixtures.nullspace(size)
    R, piv = cuda_row_reduce(fx["A"], int(fx["p"][0]), return_pivots=True)
    assert piv == [int(x) for x in fx["known_pivots"]]
    assert np.array_equal(R, fx["R"])


def test_device_api_in_and_out_of_place():
    p = 2**31 - 1
    rng = np.random.default_rng(11)
    A = workloads.rank_deficient_modp(333, 444, 200, p, rng).astype(np.uint32)
    R_ref, piv_ref, rank_ref = oracle.rref_modp(A, p)
    L = _lib.lib()
    nbytes = A.nbytes
    d_in = _lib.DeviceBuffer(nbytes)
    d_out = _lib.DeviceBuffer(nbytes)
    d_piv = _lib.DeviceBuffer(8 * 333)
    d_rank = _lib.DeviceBuffer(8)
    s = _lib.Stream()
    for in_place in (False, True):
        d_in.upload(A, s.handle)
        out_ptr = d_in.ptr if in_place else d_out.ptr
        rc = L.lnc_rref_device(_lib.LNC_U32, 333, 444, p, 0.0, d_in.ptr, 444, out_ptr, 444, d_piv.ptr,
                               d_rank.ptr, s.handle, 0)
        _lib.check(rc)
        s.synchronize()
        _lib.device_status()
        R = np.empty_like(A)
        (d_in if in_place else d_out).download(R, s.handle)
        piv = np.empty(333, dtype=np.int64)
        d_piv.download(piv, s.handle)
        rank = np.empty(1, dtype=np.int64)
        d_rank.download(rank, s.handle)
        assert np.array_equal(R.astype(np.uint64), R_ref)
        assert int(rank[0]) == rank_ref == 200
        assert list(piv[:rank_ref]) == piv_ref and np.all(piv[rank_ref:] == -1)


def test_launch_counter_moves():
    before = _lib.launch_count()
    cuda_row_reduce(np.eye(5, dtype=np.uint32) * 3, 7)
    assert _lib.launch_count() > before


def test_strided_input_and_input_not_modified():
    p = 2**31 - 1
    rng = np.random.default_rng(3)
    big = rng.integers(0, p, size=(64, 100), dtype=np.uint32)
    view = big[:, 10:90]
    keep = big.copy()
    R = cuda_row_reduce(view, p)
    R_ref, _, _ = oracle.rref_modp(np.ascontiguousarray(view), p)
    assert np.array_equal(R.astype(np.uint64), R_ref)
    assert np.array_equal(big, keep)


def _extreme_digit_matrix(p, m=384, n=400, seed=0):
    """First panel = identity on 128 pivot rows; the other rows' panel part and
    the pivot rows' trailing part are residues whose balanced base-256 digits are
    (-128, -128, -128, -63), so the limb products summed over the 128-deep
    contraction exceed 2^22 and the tensor-core epilogue must take its exact
    float-to-int fallback."""
    rng = np.random.default_rng(seed)
    x = -128 * (1 + 256 + 65536) - 63 * 2**24  # centred value with extreme digits
    xr = x % p
    A = rng.integers(0, p, size=(m, n), dtype=np.uint64)
    A[:128, :128] = np.eye(128, dtype=np.uint64)
    A[:128, 128:] = xr
    A[128:, :128] = (p - xr) % p
    return A.astype(np.uint32)


@pytest.mark.parametrize("flags", [0, _lib.LNC_FLAG_ROBUST_PANEL])
def test_limb_gemm_extreme_digits_exact(flags):
    p = 2**31 - 1
    A = _extreme_digit_matrix(p)
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=flags)
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert np.array_equal(out.astype(np.uint64), R_ref)
    assert piv == piv_ref


@pytest.mark.parametrize("flags", [0, _lib.LNC_FLAG_ROBUST_PANEL, _lib.LNC_FLAG_SIMT_TRAILING])
@pytest.mark.parametrize("m,n,r,p", [(900, 700, None, 2**31 - 1), (600, 600, None, 2**31 - 19),
                                     (1100, 1300, 777, 4294967291)])
def test_panel_paths_agree_on_adversarial_inputs(flags, m, n, r, p):
    """Leading rows zero in the leading columns: the candidate-block panel misses
    pivots there and the exhaustive panel redoes those panels."""
    rng = np.random.default_rng(m + n)
    if r is None:
        A = rng.integers(0, p, size=(m, n), dtype=np.uint64)
    else:
        A = workloads.rank_deficient_modp(m, n, r, p, rng)
    A[: m // 2, :60] = 0
    A[:, 200:205] = 0
    A = A.astype(np.uint32)
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=flags)
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert np.array_equal(out.astype(np.uint64), R_ref)
    assert piv == piv_ref


@pytest.mark.parametrize("flags", [0, _lib.LNC_FLAG_SIMT_TRAILING, _lib.LNC_FLAG_ROBUST_PANEL,
                                   _lib.LNC_FLAG_DEFER_FALLBACK])
@pytest.mark.parametrize("m,n,p", [(700, 900, 2**61 - 1), (900, 600, 2**32 + 15), (520, 520, 2**64 - 59)])
def test_u64_tensor_core_update_vs_oracle(flags, m, n, p):
    """64-bit residues: eight-digit limb contraction (default) and the SIMT
    update agree with the oracle, including entries at the digit extremes
    (p - 1, (p - 1) / 2, (p + 1) / 2) and rank deficiency."""
    rng = np.random.default_rng(m * 7 + n)
    r = min(m, n) - 37
    Bf = rng.integers(0, 2**63, size=(m, r), dtype=np.uint64) % np.uint64(p)
    Cf = rng.integers(0, 2**63, size=(r, n), dtype=np.uint64) % np.uint64(p)
    A = oracle.matmul_modp(Bf, Cf, p)
    A[:40, 100:300] = np.uint64(p - 1)
    A[40:80, 300:500] = np.uint64((p - 1) // 2)
    A[80:90] = np.uint64((p + 1) // 2)
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=flags)
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert np.array_equal(out, R_ref)
    assert piv == piv_ref


@pytest.mark.parametrize("flags", [0, _lib.LNC_FLAG_ROBUST_PANEL])
def test_u64_candidate_panel_misses_are_redone(flags):
    """64-bit residues, leading rows zero in the leading columns: the candidate
    block misses pivots there and the exhaustive panel redoes those panels."""
    p = 2**61 - 1
    rng = np.random.default_rng(77)
    A = rng.integers(0, 2**62, size=(900, 700), dtype=np.uint64) % np.uint64(p)
    A[:450, :80] = 0
    A[:, 200:205] = 0
    out = np.empty_like(A)
    piv, rank = rref_host_call(A, p, out, flags=flags)
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert np.array_equal(out, R_ref)
    assert piv == piv_ref


def test_large_host_outputs_fresh_strided_and_in_place():
    """Pageable host outputs of 64 MB and more are mapped by host threads while
    the GPU solves: the default fresh output, a strided output (the columns
    between its rows stay untouched) and an in-place call (the input is read
    before anything is written) all hold the exact result."""
    p = 2**31 - 1
    m = 4200  # 4200 x 4200 uint32: 70.6 MB; full rank with overwhelming probability, so the RREF is I
    rng = np.random.default_rng(11)
    A = rng.integers(0, p, size=(m, m), dtype=np.uint64).astype(np.uint32)
    eye = np.eye(m, dtype=np.uint32)
    R, piv = cuda_row_reduce(A, p, return_pivots=True)
    assert piv == list(range(m)) and np.array_equal(R, eye)
    big = np.full((m, m + 5), 7, dtype=np.uint32)
    out = big[:, :m]
    cuda_row_reduce(A, p, out=out)
    assert np.array_equal(out, eye) and np.all(big[:, m:] == 7)
    B = A.copy()
    cuda_row_reduce(B, p, out=B)
    assert np.array_equal(B, eye)
