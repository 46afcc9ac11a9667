"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Run from the repository root in a container that has the reference checkout
(``LINAC_REFERENCE``, default: a directory ``reference`` beside the
repository root):

    python tests/golden/make_golden.py

What it writes (all small, committed):

* ``modp_cases.npz`` -- small F_p matrices and their RREF + pivot columns as
  computed by the reference's ``row_reduce(A, pivoting=1, scaling=False,
  threshold=0, prime=p)`` (linac/row_reduce.py:16).  For p >= 2^31.5 the
  reference's int64 path overflows, so those cases run the same reference
  function on an object array of exact residues (``ModP`` stand-in).
* ``float_cases.npz`` -- float64 / complex128 matrices and the reference's
  ``row_reduce(A, pivoting=1, scaling=True, threshold=1e-9)``.
* ``config1.json`` -- SHA-256, pivots, rank and last column of the RREF of the
  512 x 640 rank-384 matrix (linac_gb300.workloads.config1) by the reference.
* ``known_result_4096_4097_2to32m19.npy`` -- the reference's own stored golden
  vector (tests/test_data/, used by tests/test_row_reduce_random_cuda.py:52-63),
  copied byte for byte.
* ``nullspace_{small,medium}_2147483647.npz`` -- the reference's pickled
  ModP fixtures (tests/test_data/*_kernel_test_matrix_2147483647.npy) decoded
  with a restricted unpickler into plain uint32 arrays, with the known pivots
  and RREF shapes of tests/test_null_space.py:26-41.
* ``loader_cases.npz`` / ``loader_cases.json`` -- ``load_matrices(...,
  use_cuda=False, _use_galois=False)`` (linac/pycuda_matrix_loader.py:127) on
  dict-form points over several fields, with the produced matrices.
"""
from __future__ import annotations

import hashlib
import io
import json
import os
import pickle
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

import reference_import as ri  # noqa: E402
from linac_gb300 import workloads  # noqa: E402
from linac_gb300.primes import is_prime  # noqa: E402

INT64_SAFE = int(3.0e9)  # p*p < 2^63 keeps the reference's int64 path exact


def ref_rref_modp(A: np.ndarray, p: int):
    row_reduce = ri.reference_row_reduce()
    if p < INT64_SAFE:
        R, _ = row_reduce(A.astype(np.int64), pivoting=1, scaling=False, threshold=0, prime=p)
        R = R.astype(np.uint64)
    else:
        obj = np.empty(A.shape, dtype=object)
        for idx, v in np.ndenumerate(A):
            obj[idx] = ri.ModP(int(v), p)
        R, _ = row_reduce(obj, pivoting=1, scaling=False, threshold=0, prime=None)
        R = np.vectorize(lambda x: int(x) if isinstance(x, ri.ModP) else int(x) % p,
                         otypes=[object])(R).astype(np.uint64)
    piv = []
    for r in range(R.shape[0]):
        nz = np.nonzero(R[r])[0]
        if len(nz) == 0:
            break
        piv.append(int(nz[0]))
    return R, piv


def modp_cases():
    rng = np.random.default_rng(12345)
    primes = [2, 3, 5, 65521, 2**31 - 1, 2**31 - 19, 2**31 + 11, 4294967291,
              2**61 - 1, 2**61 + 15, 2**63 - 25, 18446744073709551557]
    for p in primes:
        assert is_prime(p), p
    cases = []

    def add(name, A, p):
        cases.append((name, np.asarray(A, dtype=np.uint64) % np.uint64(p), p))

    for p in primes:
        add(f"rand8x8_p{p}", rng.integers(0, p, size=(8, 8), dtype=np.uint64), p)
        add(f"rand16x24_p{p}", rng.integers(0, p, size=(16, 24), dtype=np.uint64), p)
        add(f"rand24x16_p{p}", rng.integers(0, p, size=(24, 16), dtype=np.uint64), p)
    P = 2**31 - 1
    for p in (P, 2**31 + 11, 2**61 - 1):
        add(f"zero5x7_p{p}", np.zeros((5, 7)), p)
        add(f"one1x1_p{p}", np.array([[rng.integers(1, min(p, 2**62))]]), p)
        add(f"zero1x1_p{p}", np.zeros((1, 1)), p)
        add(f"row1x9_p{p}", rng.integers(0, min(p, 2**62), size=(1, 9), dtype=np.uint64), p)
        add(f"col9x1_p{p}", rng.integers(0, min(p, 2**62), size=(9, 1), dtype=np.uint64), p)
    for p in (P, 2**31 - 19, 2**31 + 11):
        add(f"rank40_64x80_p{p}", workloads.rank_deficient_modp(64, 80, 40, p, rng), p)
        add(f"rank50_80x64_p{p}", workloads.rank_deficient_modp(80, 64, 50, p, rng), p)
        add(f"rank1_40x40_p{p}", workloads.rank_deficient_modp(40, 40, 1, p, rng), p)
        add(f"rank3_33x47_p{p}", workloads.rank_deficient_modp(33, 47, 3, p, rng), p)
        A = rng.integers(0, p, size=(20, 26), dtype=np.uint64)
        A[:, :3] = 0
        A[:, 7] = 0
        add(f"zerocols_20x26_p{p}", A, p)
        A = rng.integers(0, p, size=(17, 17), dtype=np.uint64)
        np.fill_diagonal(A, 0)
        add(f"zerodiag_17x17_p{p}", A, p)
        A = rng.integers(0, p, size=(12, 15), dtype=np.uint64)
        A[5] = A[2]
        A[9] = (A[1] * np.uint64(3)) % np.uint64(p)
        add(f"duprows_12x15_p{p}", A, p)
        add(f"rand70x70_p{p}", rng.integers(0, p, size=(70, 70), dtype=np.uint64), p)
        add(f"rand45x130_p{p}", rng.integers(0, p, size=(45, 130), dtype=np.uint64), p)
        add(f"rand130x45_p{p}", rng.integers(0, p, size=(130, 45), dtype=np.uint64), p)
    # sparse 0/1 pattern: many zero pivots candidates
    A = (rng.random((30, 40)) < 0.1).astype(np.uint64)
    add("sparse01_30x40_p2147483647", A, P)
    A = (rng.random((30, 40)) < 0.3).astype(np.uint64)
    add("sparse01_30x40_p2", A, 2)
    for p in (2**61 - 1, 2**61 + 15):
        B = rng.integers(0, p, size=(24, 6), dtype=np.uint64)
        C = rng.integers(0, p, size=(6, 30), dtype=np.uint64)
        BC = np.zeros((24, 30), dtype=np.uint64)
        for i in range(24):
            for j in range(30):
                BC[i, j] = sum(int(B[i, t]) * int(C[t, j]) for t in range(6)) % p
        add(f"rank6_24x30_p{p}", BC, p)

    out = {}
    names = []
    for k, (name, A, p) in enumerate(cases):
        R, piv = ref_rref_modp(A, p)
        out[f"{name}__A"] = A
        out[f"{name}__R"] = R
        out[f"{name}__p"] = np.array([p], dtype=np.uint64)
        out[f"{name}__piv"] = np.array(piv, dtype=np.int64)
        names.append(name)
    out["__names__"] = np.array(names)
    np.savez_compressed(HERE / "modp_cases.npz", **out)
    print(f"modp_cases.npz: {len(names)} cases")


def float_cases():
    row_reduce = ri.reference_row_reduce()
    rng = np.random.default_rng(777)
    cases = []
    cases.append(("f64_rand8x8", rng.standard_normal((8, 8))))
    cases.append(("f64_rand12x20", rng.standard_normal((12, 20))))
    cases.append(("f64_rand20x12", rng.standard_normal((20, 12))))
    A = rng.standard_normal((10, 14))
    A[4] = 2.0 * A[1]
    A[7] = A[2] + A[3]
    cases.append(("f64_rankdef10x14", A))
    cases.append(("f64_cond_40x44", np.hstack([workloads.conditioned_matrix(40, rng, 1e3),
                                                rng.standard_normal((40, 4))])))
    cases.append(("c128_rand8x8", rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))))
    cases.append(("c128_rand12x20", rng.standard_normal((12, 20)) + 1j * rng.standard_normal((12, 20))))
    B = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    B[5] = (1 + 2j) * B[0]
    cases.append(("c128_rankdef16x16", B))
    cases.append(("c128_cond_40x44", np.hstack([workloads.conditioned_matrix(40, rng, 1e3, True),
                                                 rng.standard_normal((40, 4)) + 0j])))
    out = {}
    names = []
    for name, A in cases:
        R, _ = row_reduce(A.copy(), pivoting=1, scaling=True, threshold=1e-9)
        out[f"{name}__A"] = A
        out[f"{name}__R"] = np.asarray(R)
        names.append(name)
    out["__names__"] = np.array(names)
    np.savez_compressed(HERE / "float_cases.npz", **out)
    print(f"float_cases.npz: {len(names)} cases")


def config1_fixture():
    A, p = workloads.config1()
    R, piv = ref_rref_modp(A.astype(np.uint64), p)
    R32 = R.astype(np.uint32)
    digest = hashlib.sha256(np.ascontiguousarray(R32).tobytes()).hexdigest()
    input_digest = hashlib.sha256(np.ascontiguousarray(A).tobytes()).hexdigest()
    data = {"shape": list(A.shape), "p": p, "rank": len(piv), "pivots": piv,
            "rref_sha256_u32": digest, "input_sha256_u32": input_digest,
            "last_column": [int(x) for x in R32[:, -1]],
            "row0": [int(x) for x in R32[0]]}
    (HERE / "config1.json").write_text(json.dumps(data))
    print("config1.json:", len(piv), digest[:16])


def known_result_copy():
    src = ri.REFERENCE_ROOT / "tests" / "test_data" / "known_result_4096_4097_2to32m19.npy"
    shutil.copyfile(src, HERE / "known_result_4096_4097_2to32m19.npy")
    print("known_result copied")


class _RestrictedUnpickler(pickle.Unpickler):
    """Maps the pickled pyadic ModP class to the local stand-in; refuses
    every other global except numpy's array reconstruction helpers."""

    ALLOWED = {("numpy.core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "_reconstruct"),
               ("numpy", "ndarray"), ("numpy", "dtype"), ("numpy.core.multiarray", "scalar"),
               ("numpy._core.multiarray", "scalar")}

    def find_class(self, module, name):
        if name == "ModP" or name == "ModPArray" or module.startswith("pyadic"):
            return _ModPState
        if (module, name) in self.ALLOWED:
            import importlib
            return getattr(importlib.import_module(module), name)
        raise pickle.UnpicklingError(f"refused global {module}.{name}")


class _ModPState:
    def __init__(self, *args, **kwargs):
        self.n, self.p = None, None

    def __setstate__(self, state):
        if isinstance(state, tuple) and len(state) == 2:
            self.n, self.p = int(state[0]), int(state[1])
        elif isinstance(state, dict):
            self.n, self.p = int(state.get("n")), int(state.get("p"))
        else:
            raise pickle.UnpicklingError(f"unexpected ModP state {state!r}")

    def __reduce__(self):
        raise TypeError


def _load_modp_npy(path: Path) -> tuple[np.ndarray, int]:
    raw = path.read_bytes()
    f = io.BytesIO(raw)
    version = np.lib.format.read_magic(f)
    if version == (1, 0):
        shape, fortran, dtype = np.lib.format.read_array_header_1_0(f)
    else:
        shape, fortran, dtype = np.lib.format.read_array_header_2_0(f)
    assert dtype == np.dtype(object)
    arr = _RestrictedUnpickler(f).load()
    flat = arr.ravel(order="F" if fortran else "C")
    vals = np.array([x.n for x in flat], dtype=np.uint64).reshape(shape, order="F" if fortran else "C")
    ps = {x.p for x in flat}
    assert len(ps) == 1
    return np.ascontiguousarray(vals), ps.pop()


def nullspace_fixtures():
    for size, piv, shape, ck in (
            ("small", [0, 1, 2, 3, 4, 5], (6, 7), (7, 1)),
            ("medium", [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23,
                        24, 25, 26, 27, 38, 39, 40, 41, 59], (31, 86), (86, 55))):
        src = ri.REFERENCE_ROOT / "tests" / "test_data" / f"{size}_kernel_test_matrix_2147483647.npy"
        vals, p = _load_modp_npy(src)
        R, rpiv = ref_rref_modp(vals, p)
        assert rpiv == piv, (rpiv, piv)
        np.savez_compressed(HERE / f"nullspace_{size}_2147483647.npz", A=vals.astype(np.uint32),
                            p=np.array([p], dtype=np.uint64), known_pivots=np.array(piv),
                            rref_shape=np.array(shape), kernel_shape=np.array(ck),
                            R=R.astype(np.uint32))
        print(f"nullspace_{size}: {vals.shape} pivots ok")


class _Field:
    def __init__(self, name, characteristic):
        self.name = name
        self.characteristic = characteristic

    def __contains__(self, x):
        return False


LOADER_PREFACTORS = ['(x)/(x^2+y+z)', '(y)/(x+y+z^2)', '(z)/(x+y^2+z)']
LOADER_ANSATZE = [
    [['x'], ['y'], ['z'], ['x', 'x'], ['x', 'y'], ['x', 'z'], ['y', 'y'], ['y', 'z'], ['x', 'y', 'z']],
    [['x'], ['y'], ['z'], ['x', 'x'], ['x', 'y'], ['x', 'z'], ['y', 'y'], ['y', 'z'], ['x', 'y', 'z']],
    [],
]


def loader_points(field_name: str, p: int, n_pts: int, seed: int):
    """Dict-form points over a field: values of x, y, z, '1' and of each
    prefactor (x/(x^2+y+z) etc.) computed exactly in the field."""
    rng = np.random.default_rng(seed)
    pts = {"field": _Field(field_name, p)}
    if p > 0:
        xs = [int(v) for v in rng.integers(1, p if p < 2**62 else 2**62, size=n_pts)]
        ys = [int(v) for v in rng.integers(1, p if p < 2**62 else 2**62, size=n_pts)]
        zs = [int(v) for v in rng.integers(1, p if p < 2**62 else 2**62, size=n_pts)]
        inv = lambda a: pow(int(a) % p, -1, p)  # noqa: E731
        pts["1"] = np.array([1] * n_pts, dtype=object)
        pts["x"] = np.array(xs, dtype=object)
        pts["y"] = np.array(ys, dtype=object)
        pts["z"] = np.array(zs, dtype=object)
        pts[LOADER_PREFACTORS[0]] = np.array([x * inv(x * x + y + z) % p for x, y, z in zip(xs, ys, zs)], dtype=object)
        pts[LOADER_PREFACTORS[1]] = np.array([y * inv(x + y + z * z) % p for x, y, z in zip(xs, ys, zs)], dtype=object)
        pts[LOADER_PREFACTORS[2]] = np.array([z * inv(x + y * y + z) % p for x, y, z in zip(xs, ys, zs)], dtype=object)
    else:
        cplx = field_name not in ("mpf", "R")
        def draw():
            v = rng.uniform(0.5, 2.0, size=n_pts)
            if cplx:
                v = v + 1j * rng.uniform(-1.0, 1.0, size=n_pts)
            return v
        xs, ys, zs = draw(), draw(), draw()
        pts["1"] = np.ones(n_pts, dtype=complex if cplx else float)
        pts["x"], pts["y"], pts["z"] = xs, ys, zs
        pts[LOADER_PREFACTORS[0]] = xs / (xs ** 2 + ys + zs)
        pts[LOADER_PREFACTORS[1]] = ys / (xs + ys + zs ** 2)
        pts[LOADER_PREFACTORS[2]] = zs / (xs + ys ** 2 + zs)
    return pts


LOADER_FIELDS = [("finite field", 2**31 - 1), ("finite field", 2**31 - 19), ("finite field", 2**31 + 11),
                 ("finite field", 2**61 - 1), ("finite field", 2**61 + 15), ("padic", 2**31 - 1),
                 ("mpf", 0), ("mpc", 0)]


def loader_fixtures():
    load_matrices = ri.reference_load_matrices()
    out = {}
    meta = []
    n_pts = sum(map(len, LOADER_ANSATZE))
    for k, (fname, p) in enumerate(LOADER_FIELDS):
        pts = loader_points(fname, p, n_pts, seed=100 + k)
        As = load_matrices(LOADER_PREFACTORS, LOADER_ANSATZE, pts, use_cuda=False, _use_galois=False)
        for t, A in enumerate(As):
            out[f"f{k}_A{t}"] = np.asarray(A)
        for key, vals in pts.items():
            if key == "field":
                continue
            arr = np.asarray(vals)
            if p > 0:
                arr = np.array([int(v) for v in vals], dtype=np.uint64)
            out[f"f{k}_pt_{key}"] = arr
        meta.append({"index": k, "field": fname, "p": p, "n_matrices": len(As)})
    np.savez_compressed(HERE / "loader_cases.npz", **out)
    (HERE / "loader_cases.json").write_text(json.dumps(
        {"fields": meta, "prefactors": LOADER_PREFACTORS, "ansatze": LOADER_ANSATZE,
         "point_keys": ["1", "x", "y", "z"] + LOADER_PREFACTORS}, indent=1))
    print(f"loader fixtures: {len(meta)} fields")


def main():
    if not ri.reference_available():
        raise SystemExit(f"reference checkout not found at {ri.REFERENCE_ROOT}")
    known_result_copy()
    nullspace_fixtures()
    modp_cases()
    float_cases()
    config1_fixture()
    loader_fixtures()


if __name__ == "__main__":
    main()
