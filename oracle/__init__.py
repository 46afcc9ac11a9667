"""CPU oracle for the RREF / monomial-loader path.

TEST INFRASTRUCTURE ONLY.  This package is the checker: tests/, the smoke
check in __graft_entry__.py and bench.py (its cpu_baseline leg and its
``--impl reference`` arm) are the only code allowed to import it.  The
linac_gb300 product path never imports it and has no CPU fallback.

The numerics live in ``rref_oracle.c`` (a C restatement of linac's CPU
``row_reduce``, linac/row_reduce.py:16-78, and of the CPU branch of
``load_matrices``, linac/pycuda_matrix_loader.py:220-225).  ``build()``
compiles it with gcc into ``oracle/_build/liboracle.so``.  Parity of this
restatement with the reference is pinned by the fixtures in tests/golden/,
produced from the reference's own Python code and its stored golden vector.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "rref_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the C oracle (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", _SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            # OpenMP threads sleep as soon as a parallel region ends instead of spinning, so that
            # an oracle check does not take host cores from the timed GPU work that follows it
            os.environ.setdefault("OMP_WAIT_POLICY", "passive")
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            i64, u64, dbl, vp, cint = (ctypes.c_int64, ctypes.c_uint64, ctypes.c_double,
                                       ctypes.c_void_p, ctypes.c_int)
            lib.oracle_rref_modp.argtypes = [vp, i64, i64, i64, u64, vp, vp, cint]
            lib.oracle_rref_modp.restype = cint
            lib.oracle_rref_modp_partial.argtypes = [vp, i64, i64, i64, u64, i64, cint]
            lib.oracle_rref_modp_partial.restype = i64
            lib.oracle_rref_f64.argtypes = [vp, i64, i64, i64, dbl, cint, vp, vp]
            lib.oracle_rref_f64.restype = cint
            lib.oracle_rref_c128.argtypes = [vp, i64, i64, i64, dbl, cint, vp, vp]
            lib.oracle_rref_c128.restype = cint
            lib.oracle_load_modp.argtypes = [vp, i64, i64, vp, i64, i64, u64, vp]
            lib.oracle_load_f64.argtypes = [vp, i64, i64, vp, i64, i64, vp]
            lib.oracle_load_c128.argtypes = [vp, i64, i64, vp, i64, i64, vp]
            lib.oracle_matmul_modp.argtypes = [vp, vp, i64, i64, i64, u64, vp, cint]
            lib.oracle_residual_f64.argtypes = [vp, vp, vp, i64, i64, i64, vp, cint]
            lib.oracle_residual_c128.argtypes = [vp, vp, vp, i64, i64, i64, vp, cint]
            _lib = lib
    return _lib


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def rref_modp(A, p: int, nthreads: int | None = None):
    """RREF of A over F_p.  Returns (R, pivot_columns, rank); R has A's shape,
    dtype uint64.  Raises ZeroDivisionError for a non-invertible pivot (p not
    prime), as linac/row_reduce.py:63-64 does."""
    lib = _load()
    A = np.array(A, dtype=np.uint64, order="C", copy=True)
    if A.ndim != 2:
        raise ValueError("expected a 2-D matrix")
    m, n = A.shape
    piv = np.zeros(max(1, min(m, n)), dtype=np.int64)
    rank = np.zeros(1, dtype=np.int64)
    rc = lib.oracle_rref_modp(A.ctypes.data, m, n, n, int(p), piv.ctypes.data, rank.ctypes.data,
                              nthreads or default_threads())
    if rc == -2:
        raise ZeroDivisionError(f"an inverse mod {p} does not exist; is {p} prime?")
    if rc != 0:
        raise ValueError(f"oracle_rref_modp failed ({rc})")
    r = int(rank[0])
    return A, [int(x) for x in piv[:r]], r


def rref_modp_partial(A, p: int, max_pivots: int, nthreads: int | None = None) -> int:
    """Run the first `max_pivots` pivot steps in place (timing samples)."""
    lib = _load()
    assert A.dtype == np.uint64 and A.flags.c_contiguous
    m, n = A.shape
    return int(lib.oracle_rref_modp_partial(A.ctypes.data, m, n, n, int(p), int(max_pivots),
                                            nthreads or default_threads()))


def rref_f64(A, threshold: float = 1e-9, scaling: bool = True):
    lib = _load()
    A = np.array(A, dtype=np.float64, order="C", copy=True)
    m, n = A.shape
    piv = np.zeros(max(1, min(m, n)), dtype=np.int64)
    rank = np.zeros(1, dtype=np.int64)
    lib.oracle_rref_f64(A.ctypes.data, m, n, n, float(threshold), int(bool(scaling)),
                        piv.ctypes.data, rank.ctypes.data)
    r = int(rank[0])
    return A, [int(x) for x in piv[:r]], r


def rref_c128(A, threshold: float = 1e-9, scaling: bool = True):
    lib = _load()
    A = np.array(A, dtype=np.complex128, order="C", copy=True)
    m, n = A.shape
    piv = np.zeros(max(1, min(m, n)), dtype=np.int64)
    rank = np.zeros(1, dtype=np.int64)
    lib.oracle_rref_c128(A.ctypes.data, m, n, n, float(threshold), int(bool(scaling)),
                         piv.ctypes.data, rank.ctypes.data)
    r = int(rank[0])
    return A, [int(x) for x in piv[:r]], r


def load_modp(bases, lindices, p: int):
    lib = _load()
    bases = np.ascontiguousarray(bases, dtype=np.uint64)
    lind = np.ascontiguousarray(lindices, dtype=np.uint32)
    out = np.zeros((bases.shape[0], lind.shape[0]), dtype=np.uint64)
    lib.oracle_load_modp(bases.ctypes.data, bases.shape[0], bases.shape[1], lind.ctypes.data,
                         lind.shape[0], lind.shape[1], int(p), out.ctypes.data)
    return out


def load_float(bases, lindices):
    lib = _load()
    lind = np.ascontiguousarray(lindices, dtype=np.uint32)
    if np.iscomplexobj(bases):
        bases = np.ascontiguousarray(bases, dtype=np.complex128)
        out = np.zeros((bases.shape[0], lind.shape[0]), dtype=np.complex128)
        lib.oracle_load_c128(bases.ctypes.data, bases.shape[0], bases.shape[1], lind.ctypes.data,
                             lind.shape[0], lind.shape[1], out.ctypes.data)
    else:
        bases = np.ascontiguousarray(bases, dtype=np.float64)
        out = np.zeros((bases.shape[0], lind.shape[0]), dtype=np.float64)
        lib.oracle_load_f64(bases.ctypes.data, bases.shape[0], bases.shape[1], lind.ctypes.data,
                            lind.shape[0], lind.shape[1], out.ctypes.data)
    return out


def matmul_modp(B, C, p: int, nthreads: int | None = None):
    lib = _load()
    B = np.ascontiguousarray(B, dtype=np.uint64)
    C = np.ascontiguousarray(C, dtype=np.uint64)
    m, k = B.shape
    k2, n = C.shape
    assert k == k2
    out = np.zeros((m, n), dtype=np.uint64)
    lib.oracle_matmul_modp(B.ctypes.data, C.ctypes.data, m, k, n, int(p), out.ctypes.data,
                           nthreads or default_threads())
    return out


def residual_dd(A, X, B, nthreads: int | None = None):
    """B - A X with double-double accumulation, rounded once (float64 or
    complex128 operands)."""
    lib = _load()
    cplx = np.iscomplexobj(A) or np.iscomplexobj(X) or np.iscomplexobj(B)
    dt = np.complex128 if cplx else np.float64
    A = np.ascontiguousarray(A, dtype=dt)
    X = np.ascontiguousarray(X, dtype=dt)
    B = np.ascontiguousarray(B, dtype=dt)
    m, k = A.shape
    q = X.shape[1]
    assert X.shape[0] == k and B.shape == (m, q)
    out = np.empty((m, q), dtype=dt)
    f = lib.oracle_residual_c128 if cplx else lib.oracle_residual_f64
    f(A.ctypes.data, X.ctypes.data, B.ctypes.data, m, k, q, out.ctypes.data, nthreads or default_threads())
    return out


def reference_solution(A, B, iterations: int = 3):
    """Solution of A X = B to FP64 accuracy: LAPACK's solve refined with
    double-double residuals (the exact solution of the stored system, rounded;
    cond(A) * eps^2 below FP64's own rounding for cond(A) << 1/eps)."""
    try:
        from scipy.linalg import lu_factor, lu_solve
    except ImportError:  # one factorisation per solve without scipy
        def solve(rhs):
            return np.linalg.solve(A, rhs)
    else:
        lu = lu_factor(A)

        def solve(rhs):
            return lu_solve(lu, rhs)
    X = solve(B)
    for _ in range(iterations):
        X = X + solve(residual_dd(A, X, B))
    return X
