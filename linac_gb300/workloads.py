"""Seeded synthetic inputs with the shapes of the RREF / loader workloads.

linac ships no benchmark data; every workload here is generated from a fixed
seed with ``numpy.random.default_rng`` so that tests and the benchmark see the
same matrices on every machine.

* ``rank_deficient_modp(m, n, r, p, rng)`` -- A = B.C mod p with B (m x r) and
  C (r x n) uniform in [0, p): rank r with overwhelming probability.  The
  product is computed exactly on the host by splitting C into 16-bit halves so
  that every int64 partial sum stays below 2^63.
* ``uniform_modp(m, n, p, rng)`` -- entries uniform in [0, p).
* ``config1()`` -- the 512 x 640, rank-384 matrix mod 2^31-1 (seed 0).
* ``batch_shapes(count, rng)`` -- uneven batch shapes: m ~ U[64, 2048],
  n = round(m * U[0.8, 1.25]), rank deficit ~ U[0, 10%] of min(m, n), and a
  prime per matrix from the 64 largest primes below 2^31.
* ``haar_orthogonal`` / ``conditioned_matrix`` -- U diag(s) V^T test matrices
  with log-spaced singular values for the float / complex path.
* ``serve_load_request(rng, d, p)`` -- one served load+RREF request: all
  monomials of total degree <= d in 10 variables (truncated to 8000), rows =
  columns + 16 points uniform in F_p^10 with non-zero uniform prefactors, as
  loader inputs (bases = [1, x_1..x_10, prefactor] per point, lindices = the
  monomial's d basis columns + the prefactor column).
"""
from __future__ import annotations

import itertools
from functools import lru_cache

import numpy as np

from .primes import is_prime, largest_primes_below

P31 = 2**31 - 1
P61 = 2**61 - 1


def matmul_modp(B: np.ndarray, C: np.ndarray, p: int) -> np.ndarray:
    """Exact (B @ C) mod p for p < 2^32 and inner dimension <= 2^14."""
    p = int(p)
    if p >= 2**32:
        raise ValueError("matmul_modp handles p < 2^32")
    B = np.asarray(B, dtype=np.int64) % p
    C = np.asarray(C, dtype=np.int64) % p
    k = B.shape[1]
    if k > 2**14:
        raise ValueError("inner dimension too large for the exact int64 split")
    lo = C & 0xFFFF
    hi = C >> 16
    # B < 2^32, lo/hi < 2^16: each product < 2^48, k <= 2^14 terms < 2^62
    r_lo = (B @ lo) % p
    r_hi = (B @ hi) % p
    return ((r_hi * 65536) % p + r_lo) % p


def uniform_modp(m: int, n: int, p: int, rng: np.random.Generator) -> np.ndarray:
    return rng.integers(0, int(p), size=(m, n), dtype=np.uint64)


def rank_deficient_modp(m: int, n: int, r: int, p: int, rng: np.random.Generator) -> np.ndarray:
    B = rng.integers(0, int(p), size=(m, r), dtype=np.int64)
    C = rng.integers(0, int(p), size=(r, n), dtype=np.int64)
    return matmul_modp(B, C, p).astype(np.uint64)


def config1() -> tuple[np.ndarray, int]:
    """512 x 640 matrix of rank 384 over F_p, p = 2^31-1, built as B.C with
    B (512 x 384) and C (384 x 640) uniform in [0, p) from seed 0."""
    rng = np.random.default_rng(0)
    p = P31
    B = rng.integers(0, p, size=(512, 384), dtype=np.int64)
    C = rng.integers(0, p, size=(384, 640), dtype=np.int64)
    return matmul_modp(B, C, p).astype(np.uint32), p


def batch_primes() -> list[int]:
    return largest_primes_below(2**31, 64)


def batch_shapes(count: int, rng: np.random.Generator, m_lo: int = 64, m_hi: int = 2048):
    """Shapes, ranks and primes of an uneven batch (see module docstring)."""
    primes = batch_primes()
    out = []
    for _ in range(count):
        m = int(rng.integers(m_lo, m_hi + 1))
        n = max(1, int(round(m * rng.uniform(0.8, 1.25))))
        deficit = int(np.floor(rng.uniform(0.0, 0.10) * min(m, n)))
        r = min(m, n) - deficit
        p = int(primes[int(rng.integers(0, len(primes)))])
        out.append((m, n, r, p))
    return out


def haar_orthogonal(n: int, rng: np.random.Generator, complex_: bool = False) -> np.ndarray:
    """Haar-random orthogonal (unitary) matrix: QR of a Gaussian with the
    signs of R's diagonal folded into Q."""
    if complex_:
        Z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2.0)
    else:
        Z = rng.standard_normal((n, n))
    Q, R = np.linalg.qr(Z)
    d = np.diag(R)
    ph = d / np.abs(d)
    return Q * ph[None, :]


def conditioned_matrix(n: int, rng: np.random.Generator, cond: float = 1e6,
                       complex_: bool = False) -> np.ndarray:
    """U diag(s) V^H with s log-spaced over [1, cond]."""
    U = haar_orthogonal(n, rng, complex_)
    V = haar_orthogonal(n, rng, complex_)
    s = np.logspace(0.0, np.log10(cond), n)
    return (U * s[None, :]) @ V.conj().T


def random_prime_below(bound: int, rng: np.random.Generator, lo: int | None = None) -> int:
    """A prime drawn uniformly-ish from [lo, bound) (default lo = bound / 2)."""
    lo = bound // 2 if lo is None else lo
    while True:
        c = int(rng.integers(lo, bound)) | 1
        if c < bound and is_prime(c):
            return c


@lru_cache(maxsize=16)
def monomial_indices(n_vars: int, d: int, max_cols: int = 8000) -> np.ndarray:
    """Basis columns of every monomial of total degree <= d in n_vars variables
    (column 0 is the constant 1, column v the variable v): one row of d indices
    per monomial, multisets in lexicographic order (so a truncation keeps the
    lower degrees first), at most max_cols rows."""
    rows = list(itertools.islice(itertools.combinations_with_replacement(range(n_vars + 1), d), max_cols))
    out = np.array(rows, dtype=np.uint32).reshape(len(rows), d)
    out.flags.writeable = False
    return out


def serve_load_request(rng: np.random.Generator, d: int, p: int, n_vars: int = 10, max_cols: int = 8000,
                       extra_rows: int = 16):
    """(bases, lindices) of one load+RREF request (see module docstring)."""
    mono = monomial_indices(n_vars, d, max_cols)
    n_cols = mono.shape[0]
    n_rows = n_cols + extra_rows
    bases = np.empty((n_rows, n_vars + 2), dtype=np.uint32)
    bases[:, 0] = 1
    bases[:, 1:n_vars + 1] = rng.integers(0, p, size=(n_rows, n_vars), dtype=np.uint64)
    bases[:, n_vars + 1] = rng.integers(1, p, size=n_rows, dtype=np.uint64)
    lind = np.empty((n_cols, d + 1), dtype=np.uint32)
    lind[:, :d] = mono
    lind[:, d] = n_vars + 1
    return bases, lind
