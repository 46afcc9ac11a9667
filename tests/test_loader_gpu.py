"""GPU parity of the monomial loader.

Mirrors linac's tests/test_matrix_loader.py: the GPU matrices must equal the
reference's CPU ``load_matrices`` output exactly (fixtures produced by the
reference), and solving the system recovers the known coefficients of
f(x, y, z).  Points are dict-form with synthetic values (syngular's
RingPoint is not available).
"""
import numpy as np
import pytest

import fixtures
import oracle
from linac_gb300 import cuda_load_matrix, cuda_row_reduce, load_matrices

pytestmark = pytest.mark.gpu

KAT = [1, 2, 3, 0, 0, 0, 0, 0, 5, 0, 0, 0, 1, 7, 0, 0, 11, 0]

PREFACTORS, ANSATZE, CASES = fixtures.loader_cases()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_load_matrices_matches_reference_cpu(case):
    fname, p, pts, As_ref = case
    As = load_matrices(PREFACTORS, ANSATZE, pts)
    assert len(As) == len(As_ref)
    for A, A_ref in zip(As, As_ref):
        assert A.shape == A_ref.shape
        if A.shape[1] == 0:
            continue
        if p > 0:
            assert A.dtype == (np.uint64 if p > 2**31 - 1 else np.uint32)
            assert np.array_equal(A.astype(np.uint64), A_ref.astype(np.uint64))
        else:
            # the same IEEE products in the same order: bit-identical
            assert np.array_equal(A, A_ref.astype(A.dtype))


def _f_values(pts, p):
    x, y, z = pts["x"], pts["y"], pts["z"]
    if p > 0:
        out = []
        for a, b, c in zip(x, y, z):
            a, b, c = int(a), int(b), int(c)
            t1 = a * (a + 2 * b + 3 * c + 5 * a * b * c) * pow(a * a + b + c, -1, p)
            t2 = b * (a * a + 7 * a * b + 11 * b * c) * pow(a + b + c * c, -1, p)
            out.append((t1 + t2) % p)
        return np.array(out, dtype=np.uint64)
    return (x * (x + 2 * y + 3 * z + 5 * x * y * z)) / (x ** 2 + y + z) + \
        (y * (x ** 2 + 7 * x * y + 11 * y * z)) / (x + y + z ** 2)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_known_coefficients(case):
    """Solve [A | b] for the coefficients of f (reference test :44-57)."""
    fname, p, pts, _ = case
    As = load_matrices(PREFACTORS, ANSATZE, pts)
    b = _f_values(pts, p if fname != "padic" else p)
    if p > 0:
        A = np.hstack([a.astype(np.uint64) for a in As if a.shape[1] > 0])
        Ab = np.hstack([A, b[:, None]])
        rref = cuda_row_reduce(Ab, field_characteristic=p)
        assert np.array_equal(rref[:, :-1], np.identity(Ab.shape[0], dtype=rref.dtype))
        assert rref[:, -1].tolist() == KAT
    else:
        A = np.hstack([a for a in As if a.shape[1] > 0])
        Ab = np.hstack([A, np.asarray(b)[:, None]])
        rref = cuda_row_reduce(Ab, field_characteristic=0)
        assert np.allclose(rref[:, :-1], np.identity(Ab.shape[0]))
        assert np.allclose(rref[:, -1], KAT, atol=1e-7)


@pytest.mark.parametrize("p,dtype", [(2**31 - 1, np.uint32), (2**31 - 19, np.uint32), (2, np.uint32),
                                     (2**31 + 11, np.uint64), (2**61 - 1, np.uint64),
                                     (18446744073709551557, np.uint64)])
def test_cuda_load_matrix_vs_oracle(p, dtype):
    rng = np.random.default_rng(p % 997)
    n_rows, L, n_cols, D = 1000, 12, 3001, 9
    hi = min(p, 2**63)
    bases = rng.integers(0, hi, size=(n_rows, L), dtype=np.uint64)
    if dtype == np.uint32:
        bases = bases.astype(np.uint32)
    lind = rng.integers(0, L, size=(n_cols, D)).astype(np.uint32)
    out = cuda_load_matrix(bases, lind, field_characteristic=p)
    assert out.dtype == dtype
    assert np.array_equal(out.astype(np.uint64), oracle.load_modp(bases.astype(np.uint64), lind, p))


def test_cuda_load_matrix_unreduced_inputs_and_single_factor():
    p = 2**31 - 1
    rng = np.random.default_rng(9)
    bases = rng.integers(0, 2**32, size=(20, 5), dtype=np.uint64).astype(np.uint32)
    lind2 = rng.integers(0, 5, size=(33, 3)).astype(np.uint32)
    out = cuda_load_matrix(bases, lind2, field_characteristic=p)
    assert np.array_equal(out.astype(np.uint64), oracle.load_modp(bases, lind2, p))
    lind1 = rng.integers(0, 5, size=(33, 1)).astype(np.uint32)
    out1 = cuda_load_matrix(bases, lind1, field_characteristic=p)
    # one factor: copied as given, as the reference does
    assert np.array_equal(out1, bases[:, lind1[:, 0]])


@pytest.mark.parametrize("complex_", [False, True])
def test_cuda_load_matrix_float_bit_exact(complex_):
    rng = np.random.default_rng(4)
    bases = rng.standard_normal((500, 7))
    if complex_:
        bases = bases + 1j * rng.standard_normal((500, 7))
    lind = rng.integers(0, 7, size=(700, 6)).astype(np.uint32)
    out = cuda_load_matrix(bases, lind, field_characteristic=0)
    assert out.dtype == (np.complex128 if complex_ else np.float64)
    assert np.array_equal(out, oracle.load_float(bases, lind))


@pytest.mark.parametrize("p,L,D", [(2**30 + 3, 12, 9), (2**31 - 1, 12, 2), (2**31 - 1, 7, 3), (1000003, 12, 4),
                                   (2, 5, 8), (2**31 - 1, 40, 5), (2**31 - 1, 100, 6)])
def test_pair_products_and_fallback_vs_oracle(p, L, D):
    """p < 2^31: pair products with lazy Shoup multiplies (odd and even
    degrees); a long basis row (L = 100: the pair table does not fit shared
    memory) takes the factor-by-factor path.  Ragged row bands (1000 rows, 32
    per band) and column strips (3001 columns, 8 blocks of 256 per CTA)."""
    rng = np.random.default_rng(p % 1009 + L + D)
    n_rows, n_cols = 1000, 3001
    bases = rng.integers(0, 2**32, size=(n_rows, L), dtype=np.uint64).astype(np.uint32)  # unreduced
    lind = rng.integers(0, L, size=(n_cols, D)).astype(np.uint32)
    out = cuda_load_matrix(bases, lind, field_characteristic=p)
    assert np.array_equal(out.astype(np.uint64), oracle.load_modp(bases, lind, p))


def test_u32_modulus_above_2_31_through_the_c_abi():
    """2^31 <= p < 2^32 with 32-bit residues (Barrett path; linac itself
    switches to 64-bit words there, so only the C entry reaches it)."""
    from linac_gb300 import _lib
    p = 4294967291
    rng = np.random.default_rng(3)
    bases = rng.integers(0, p, size=(77, 12), dtype=np.uint64).astype(np.uint32)
    lind = rng.integers(0, 12, size=(600, 9)).astype(np.uint32)
    out = np.empty((77, 600), dtype=np.uint32)
    _lib.check(_lib.lib().lnc_load_matrix_host(_lib.LNC_U32, 77, 600, 12, 9, p, bases.ctypes.data, lind.ctypes.data,
                                               out.ctypes.data))
    assert np.array_equal(out.astype(np.uint64), oracle.load_modp(bases, lind, p))


@pytest.mark.parametrize("p,dtype", [(2**31 - 1, np.uint32), (2**61 - 1, np.uint64)])
def test_device_entry_flags_out_of_range_index(p, dtype):
    """The device entry cannot validate host-side: a column whose index list
    refers past the end of a bases row is written as zeros, every other column
    is exact, and lnc_device_status reports LNC_ERR_INVALID once."""
    from linac_gb300 import _lib
    L_ = _lib.lib()
    rng = np.random.default_rng(11)
    n_rows, basis_len, n_cols, D = 70, 6, 300, 4
    bases = rng.integers(0, p, size=(n_rows, basis_len), dtype=np.uint64).astype(dtype)
    lind = rng.integers(0, basis_len, size=(n_cols, D)).astype(np.uint32)
    lind[17, 2] = basis_len  # one past the end
    s = _lib.Stream()
    db, dl = _lib.DeviceBuffer(bases.nbytes), _lib.DeviceBuffer(lind.nbytes)
    dout = _lib.DeviceBuffer(np.dtype(dtype).itemsize * n_rows * n_cols)
    db.upload(bases, s.handle)
    dl.upload(lind, s.handle)
    code = _lib.LNC_U64 if dtype == np.uint64 else _lib.LNC_U32
    _lib.device_status()  # clear
    _lib.check(L_.lnc_load_matrix_device(code, n_rows, n_cols, basis_len, D, p, db.ptr, dl.ptr, dout.ptr, n_cols,
                                         s.handle))
    out = np.empty((n_rows, n_cols), dtype=dtype)
    dout.download(out, s.handle)
    assert L_.lnc_device_status() == _lib.LNC_ERR_INVALID
    assert L_.lnc_device_status() == _lib.LNC_OK  # read and cleared
    good = np.ones(n_cols, dtype=bool)
    good[17] = False
    ref = oracle.load_modp(bases, np.where(good[:, None], lind, 0).astype(np.uint32), p)
    assert np.array_equal(out[:, good].astype(np.uint64), ref[:, good])
    assert not np.any(out[:, 17])


@pytest.mark.parametrize("case", CASES[:4], ids=lambda c: f"{c[0]}-{c[1]}")
def test_single_point_returns_vectors(case):
    """Dict-form points holding scalars (one point): the reference's bases are
    1-D and load_matrices returns each matrix's only row as a vector
    (linac/pycuda_matrix_loader.py:191,228-229)."""
    fname, p, pts, As_ref = case
    for i in (0, 3):
        one = {k: (v if k == "field" else v[i]) for k, v in pts.items()}
        vecs = load_matrices(PREFACTORS, ANSATZE, one)
        assert len(vecs) == len(As_ref)
        for v, A_ref in zip(vecs, As_ref):
            assert v.ndim == 1 and v.shape == (A_ref.shape[1],)
            if A_ref.shape[1]:
                if p > 0:
                    assert np.array_equal(v.astype(np.uint64), A_ref[i].astype(np.uint64))
                else:
                    assert np.array_equal(v, A_ref[i].astype(v.dtype))
