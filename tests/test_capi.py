"""CPU-side checks of the C ABI: the library loads without a GPU, exports
every function include/linac_gb300.h declares, and rejects bad arguments on
the host before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

from linac_gb300 import _lib, cuda_row_reduce

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(lnc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_loads_and_exports_all_declared_symbols():
    L = _lib.lib()
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    bound = set(_lib.declared_symbols())
    for n in header_functions():
        assert n in bound or n.startswith(("lnc_batch", "lnc_server", "lnc_serve", "lnc_tc", "lnc_autotune",
                                           "lnc_graph", "lnc_load_rref", "lnc_rref_batch", "lnc_matmul",
                                           "lnc_rref_device_noalloc", "lnc_rref_refine", "lnc_rref_float_batch")), n


def test_header_constants_match_the_python_binding():
    """Every status, dtype and flag #define of the header has the same value in
    linac_gb300._lib (the ctypes layer passes them through unchanged)."""
    text = open(os.path.join(ROOT, "include", "linac_gb300.h")).read()
    defines = dict(re.findall(r"#define\s+(LNC_(?:OK|ERR_[A-Z_]+|U32|U64|F64|C128|FLAG_[A-Z_]+))\s+\(?(-?\d+)\)?",
                              text))
    assert len(defines) >= 20
    for name, value in defines.items():
        assert getattr(_lib, name) == int(value), name


def test_version_and_device_count():
    assert b"sm_103a" in _lib.lib().lnc_version()
    assert _lib.device_count() >= 0


def test_nonprime_modulus_rejected_on_host():
    A = np.array([[2, 1], [1, 1]], dtype=np.uint32)
    with pytest.raises(ZeroDivisionError):
        cuda_row_reduce(A, field_characteristic=4)
    with pytest.raises(ZeroDivisionError):
        cuda_row_reduce(A, field_characteristic=2**61)


def test_bad_arguments_rejected():
    L = _lib.lib()
    buf = np.zeros((2, 3), dtype=np.uint32)
    piv = np.zeros(2, dtype=np.int64)
    rank = ctypes.c_int64()
    rc = L.lnc_rref_host(99, 2, 3, 7, 0.0, buf.ctypes.data, 3, buf.ctypes.data, 3, piv.ctypes.data,
                         ctypes.byref(rank), 0)
    assert rc == _lib.LNC_ERR_INVALID
    rc = L.lnc_rref_host(_lib.LNC_U32, 2, 3, 7, 0.0, buf.ctypes.data, 2, buf.ctypes.data, 3, piv.ctypes.data,
                         ctypes.byref(rank), 0)
    assert rc == _lib.LNC_ERR_INVALID
    assert "leading dimension" in _lib.last_error()
    rc = L.lnc_rref_host(_lib.LNC_U32, 2, 3, 2**33 + 1, 0.0, buf.ctypes.data, 3, buf.ctypes.data, 3,
                         piv.ctypes.data, ctypes.byref(rank), 0)
    assert rc == _lib.LNC_ERR_INVALID


def test_loader_host_entry_rejects_out_of_range_index():
    """Checked on the host before any device work (no GPU needed)."""
    L = _lib.lib()
    bases = np.ones((4, 3), dtype=np.uint32)
    lind = np.array([[0, 1], [2, 3]], dtype=np.uint32)  # 3 is one past a row of 3
    out = np.zeros((4, 2), dtype=np.uint32)
    rc = L.lnc_load_matrix_host(_lib.LNC_U32, 4, 2, 3, 2, 2**31 - 1, bases.ctypes.data, lind.ctypes.data,
                                out.ctypes.data)
    assert rc == _lib.LNC_ERR_INVALID
    assert "lindices[1, 1]" in _lib.last_error()


def test_empty_shapes_need_no_device():
    for shape in ((0, 5), (5, 0), (0, 0)):
        out = cuda_row_reduce(np.zeros(shape, dtype=np.uint32), 2**31 - 1)
        assert out.shape == shape and out.dtype == np.uint32


def test_dtype_dispatch_rules():
    from linac_gb300.row_reduce import field_dtype
    from linac_gb300.matrix_loader import loader_dtype
    A = np.zeros((2, 2))
    assert field_dtype(A, 2**31 - 1) == np.uint32
    assert field_dtype(A, 2**32 - 5) == np.uint32
    assert field_dtype(A, 2**32 + 15) == np.uint64
    assert field_dtype(A, 7, _mod64=True) == np.uint64
    assert field_dtype(A, 0) == np.float64
    assert field_dtype(A + 1j, 0) == np.complex128
    assert field_dtype(A + 0j, 0) == np.float64
    assert loader_dtype(2**31 - 1) == np.uint32
    assert loader_dtype(2**31 + 11) == np.uint64


def test_load_matrices_host_logic():
    """bases / lindices construction (pycuda_matrix_loader.py:165-202)."""
    import fixtures
    from linac_gb300.matrix_loader import build_bases_and_indices
    prefactors, ansatze, cases = fixtures.loader_cases()
    fname, p, pts, As_ref = cases[0]
    bases, linds = build_bases_and_indices(prefactors, ansatze, pts)
    assert len(bases) == 3 and len(linds) == 3
    assert linds[0].shape == (9, 4) and linds[2].shape == (0, 1)
    # last index selects the prefactor column
    assert np.all(linds[0][:, -1] == bases[0].shape[1] - 1)
    # a host-side product of the selected bases reproduces the reference matrix
    b = bases[0]
    prod = np.array([[int(np.prod([int(b[r, i]) for i in ix], dtype=object) % p) for ix in linds[0]]
                     for r in range(b.shape[0])], dtype=np.uint64)
    assert np.array_equal(prod, As_ref[0].astype(np.uint64))


def test_use_cuda_false_is_explicitly_unsupported():
    from linac_gb300 import load_matrices
    import fixtures
    prefactors, ansatze, cases = fixtures.loader_cases()
    with pytest.raises(NotImplementedError):
        load_matrices(prefactors, ansatze, cases[0][2], use_cuda=False)
