"""Import linac's own CPU code (``row_reduce`` and the CPU loader) unmodified
from a reference checkout, for generating the golden fixtures in this folder
and for the CPU cross-checks in tests/ that skip when no checkout is present.

linac's package ``__init__`` pulls in syngular / pycoretools / pyadic, which
are not installed, so the two modules are loaded directly with importlib and
three tiny stand-ins are registered first:

* ``pyadic.finite_field.extended_euclidean_algorithm`` -- the textbook
  extended Euclid, returning (s, t, gcd) with a*s + b*t = gcd;
* ``pyadic.ModP`` -- an integer residue class with the handful of operators
  ``row_reduce`` uses on object arrays (used to run the reference's
  elimination exactly for 64-bit primes, where its int64 path overflows);
* ``pycoretools.flatten`` -- recursive flatten treating strings as atoms.

Nothing here runs on the GPU host: the reference checkout is absent there.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types
from pathlib import Path

# the reference checkout: $LINAC_REFERENCE, else a sibling directory named
# "reference" next to this repository's root
REFERENCE_ROOT = Path(os.environ.get("LINAC_REFERENCE",
                                     Path(__file__).resolve().parents[3] / "reference"))


def reference_available() -> bool:
    return (REFERENCE_ROOT / "linac" / "row_reduce.py").exists()


def extended_euclidean_algorithm(a, b):
    a, b = int(a), int(b)
    old_r, r = a, b
    old_s, s = 1, 0
    old_t, t = 0, 1
    while r != 0:
        q = old_r // r
        old_r, r = r, old_r - q * r
        old_s, s = s, old_s - q * s
        old_t, t = t, old_t - q * t
    return old_s, old_t, old_r


class ModP:
    """Residue class n mod p (stand-in for pyadic.ModP)."""

    __slots__ = ("n", "p")

    def __init__(self, n, p=None):
        if isinstance(n, ModP):
            p = n.p if p is None else p
            n = n.n
        if p is None:
            raise ValueError("ModP needs a modulus")
        self.p = int(p)
        self.n = int(n) % self.p

    def _v(self, other):
        return other.n if isinstance(other, ModP) else int(other) % self.p

    def __add__(self, o): return ModP(self.n + self._v(o), self.p)
    __radd__ = __add__
    def __sub__(self, o): return ModP(self.n - self._v(o), self.p)
    def __rsub__(self, o): return ModP(self._v(o) - self.n, self.p)
    def __mul__(self, o): return ModP(self.n * self._v(o), self.p)
    __rmul__ = __mul__
    def __neg__(self): return ModP(-self.n, self.p)

    def __truediv__(self, o):
        d = self._v(o)
        s, _, g = extended_euclidean_algorithm(d, self.p)
        if g != 1:
            raise ZeroDivisionError
        return ModP(self.n * s, self.p)

    def __abs__(self): return self
    def __int__(self): return self.n
    def __index__(self): return self.n
    def __eq__(self, o): return self.n == self._v(o)
    def __hash__(self): return hash((self.n, self.p))
    def __gt__(self, o): return self.n > (o.n if isinstance(o, ModP) else o)
    def __lt__(self, o): return self.n < (o.n if isinstance(o, ModP) else o)
    def __ge__(self, o): return self.n >= (o.n if isinstance(o, ModP) else o)
    def __le__(self, o): return self.n <= (o.n if isinstance(o, ModP) else o)
    def __repr__(self): return f"{self.n} % {self.p}"


def _flatten(x):
    out = []
    if isinstance(x, (str, bytes)):
        return [x]
    try:
        items = list(x)
    except TypeError:
        return [x]
    for it in items:
        out.extend(_flatten(it))
    return out


def _install_stubs():
    if "pyadic" not in sys.modules:
        pyadic = types.ModuleType("pyadic")
        ff = types.ModuleType("pyadic.finite_field")
        ff.extended_euclidean_algorithm = extended_euclidean_algorithm
        ff.ModP = ModP
        pyadic.finite_field = ff
        pyadic.ModP = ModP
        sys.modules["pyadic"] = pyadic
        sys.modules["pyadic.finite_field"] = ff
    if "pycoretools" not in sys.modules:
        pct = types.ModuleType("pycoretools")
        pct.flatten = _flatten
        sys.modules["pycoretools"] = pct


_cache = {}


def _load_module(name: str):
    if name in _cache:
        return _cache[name]
    _install_stubs()
    pkg_name = "_linac_reference"
    if pkg_name not in sys.modules:
        pkg = types.ModuleType(pkg_name)
        pkg.__path__ = [str(REFERENCE_ROOT / "linac")]
        sys.modules[pkg_name] = pkg
    full = f"{pkg_name}.{name}"
    spec = importlib.util.spec_from_file_location(full, REFERENCE_ROOT / "linac" / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[full] = mod
    spec.loader.exec_module(mod)
    _cache[name] = mod
    return mod


def reference_row_reduce():
    """linac.row_reduce.row_reduce, loaded unmodified."""
    return _load_module("row_reduce").row_reduce


def reference_load_matrices():
    """linac.pycuda_matrix_loader.load_matrices, loaded unmodified (CPU path)."""
    _load_module("timeit_decorator")
    _load_module("_optional")
    return _load_module("pycuda_matrix_loader").load_matrices


def reference_linear_algebra_tools():
    return _load_module("linear_algebra_tools")
