"""ctypes binding of liblinac_gb300.so (the C ABI in include/linac_gb300.h).

The shared library is built in-tree by ``python -m linac_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is missing
or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblinac_gb300.so")

LNC_OK = 0
LNC_ERR_INVALID = -1
LNC_ERR_NOT_PRIME = -2
LNC_ERR_CUDA = -3
LNC_ERR_OOM = -4
LNC_ERR_TIMEOUT = -5
LNC_ERR_ADMISSION = -6
LNC_ERR_NO_DEVICE = -7
LNC_ERR_UNSUPPORTED = -8

LNC_U32, LNC_U64, LNC_F64, LNC_C128 = 1, 2, 3, 4
DTYPE_CODE = {np.dtype(np.uint32): LNC_U32, np.dtype(np.uint64): LNC_U64,
              np.dtype(np.float64): LNC_F64, np.dtype(np.complex128): LNC_C128}

LNC_FLAG_NONE = 0
LNC_FLAG_NO_SCALING = 1
LNC_FLAG_SIMT_TRAILING = 2
LNC_FLAG_ROBUST_PANEL = 4
LNC_FLAG_DEFER_FALLBACK = 8
LNC_FLAG_MIXED = 16
LNC_FLAG_NO_LOOKAHEAD = 32
LNC_FLAG_LOOKAHEAD = 64

KC_PANEL, KC_TRAILING, KC_LOADER, KC_GATHER, KC_BATCH = 0, 1, 2, 3, 4


class LinacGpuError(RuntimeError):
    """A CUDA-side failure reported by liblinac_gb300."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class AdmissionError(LinacGpuError):
    """A request was rejected by device-memory admission control."""


class DeviceTimeoutError(LinacGpuError):
    """A bounded device-side wait ran out."""


_lock = threading.Lock()
_lib = None

_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p
_int = ctypes.c_int
_dbl = ctypes.c_double
_sz = ctypes.c_size_t

_SIGNATURES = {
    "lnc_version": ([], ctypes.c_char_p),
    "lnc_last_error": ([], ctypes.c_char_p),
    "lnc_device_count": ([], _int),
    "lnc_set_device": ([_int], _int),
    "lnc_device_info": ([_vp, _vp, _vp], _int),
    "lnc_launch_count": ([], _i64),
    "lnc_malloc": ([_vp, _sz], _int),
    "lnc_free": ([_vp], _int),
    "lnc_malloc_host": ([_vp, _sz], _int),
    "lnc_free_host": ([_vp], _int),
    "lnc_memcpy_h2d": ([_vp, _vp, _sz, _vp], _int),
    "lnc_memcpy_d2h": ([_vp, _vp, _sz, _vp], _int),
    "lnc_memcpy_d2d": ([_vp, _vp, _sz, _vp], _int),
    "lnc_memset": ([_vp, _int, _sz, _vp], _int),
    "lnc_stream_create": ([_vp], _int),
    "lnc_stream_destroy": ([_vp], _int),
    "lnc_stream_synchronize": ([_vp], _int),
    "lnc_device_synchronize": ([], _int),
    "lnc_event_create": ([_vp], _int),
    "lnc_event_destroy": ([_vp], _int),
    "lnc_event_record": ([_vp, _vp], _int),
    "lnc_event_elapsed_ms": ([_vp, _vp, _vp], _int),
    "lnc_stream_wait_event": ([_vp, _vp], _int),
    "lnc_device_status": ([], _int),
    "lnc_kernel_timing_enable": ([_int], _int),
    "lnc_kernel_timing_reset": ([], _int),
    "lnc_kernel_timing_read": ([_int, _vp, _vp], _int),
    "lnc_kernel_timing_work": ([_int, _vp], _int),
    "lnc_rref_host": ([_int, _i64, _i64, _u64, _dbl, _vp, _i64, _vp, _i64, _vp, _vp, _int], _int),
    "lnc_rref_device": ([_int, _i64, _i64, _u64, _dbl, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _int], _int),
    "lnc_load_matrix_host": ([_int, _i64, _i64, _i64, _i64, _u64, _vp, _vp, _vp], _int),
    "lnc_load_matrix_device": ([_int, _i64, _i64, _i64, _i64, _u64, _vp, _vp, _vp, _i64, _vp], _int),
    "lnc_fill_uniform_modp": ([_vp, _i64, _u64, _u64, _int, _vp], _int),
    "lnc_mixed_report": ([_vp, _vp, _vp], _int),
    "lnc_mixed_error_estimate": ([_vp], _int),
    "lnc_canonical_kernel_device": ([_int, _i64, _i64, _u64, _vp, _i64, _vp, _vp, _i64, _vp], _int),
    "lnc_rref_append_device": ([_int, _i64, _i64, _i64, _u64, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _vp],
                               _int),
    "lnc_matmul_modp_device": ([_int, _i64, _i64, _i64, _u64, _vp, _i64, _vp, _i64, _vp, _i64, _vp], _int),
}


def declared_symbols():
    """Names of the entry points the Python layer binds."""
    return list(_SIGNATURES)


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise ImportError(
                        f"{LIB_PATH} is missing: build it with `python -m linac_gb300.build`")
                L = ctypes.CDLL(LIB_PATH)
                for name, (argt, rest) in _SIGNATURES.items():
                    fn = getattr(L, name, None)
                    if fn is None:
                        continue
                    fn.argtypes = argt
                    fn.restype = rest
                _lib = L
    return _lib


def bind(name: str, argtypes, restype=_int):
    """Bind an extra entry point (used by modules that add their own)."""
    fn = getattr(lib(), name)
    fn.argtypes = argtypes
    fn.restype = restype
    return fn


def last_error() -> str:
    return lib().lnc_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc == LNC_OK:
        return
    msg = last_error()
    if what:
        msg = f"{what}: {msg}"
    if rc == LNC_ERR_NOT_PRIME:
        raise ZeroDivisionError(msg)
    if rc == LNC_ERR_OOM:
        raise MemoryError(msg)
    if rc == LNC_ERR_INVALID:
        raise ValueError(msg)
    if rc == LNC_ERR_ADMISSION:
        raise AdmissionError(rc, msg)
    if rc == LNC_ERR_TIMEOUT:
        raise DeviceTimeoutError(rc, msg)
    raise LinacGpuError(rc, msg)


def device_count() -> int:
    try:
        return int(lib().lnc_device_count())
    except (ImportError, OSError):
        return 0


def launch_count() -> int:
    return int(lib().lnc_launch_count())


def ptr(a) -> int:
    """Address of a numpy array's data (None-safe)."""
    if a is None:
        return None
    return a.ctypes.data


# ---- device memory helpers ---------------------------------------------------

class DeviceBuffer:
    """A cudaMalloc'd buffer owned by Python (freed on close / GC)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(lib().lnc_malloc(ctypes.byref(p), max(self.nbytes, 1)), "lnc_malloc")
        self.ptr = p.value

    def close(self):
        if self.ptr:
            lib().lnc_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, arr: np.ndarray, stream=None):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        check(lib().lnc_memcpy_h2d(self.ptr, arr.ctypes.data, arr.nbytes, stream), "h2d")

    def download(self, out: np.ndarray, stream=None, offset: int = 0):
        assert out.flags.c_contiguous
        check(lib().lnc_memcpy_d2h(out.ctypes.data, self.ptr + offset, out.nbytes, stream), "d2h")
        if stream is not None:
            check(lib().lnc_stream_synchronize(stream))
        else:
            check(lib().lnc_device_synchronize())
        return out


class PinnedArray:
    """Owner of a pinned (page-locked) host allocation.  ``np.asarray(obj)``
    gives an ndarray over it whose ``.base`` keeps the allocation alive."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        self.shape = tuple(int(s) for s in shape)
        self.dtype = dtype
        n = int(np.prod(self.shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        check(lib().lnc_malloc_host(ctypes.byref(p), max(n, 1)), "lnc_malloc_host")
        self._ptr = p.value
        self.__array_interface__ = {"shape": self.shape, "typestr": dtype.str,
                                    "data": (self._ptr, False), "version": 3}

    @property
    def array(self) -> np.ndarray:
        return np.asarray(self)

    def __del__(self):
        try:
            if self._ptr:
                lib().lnc_free_host(self._ptr)
                self._ptr = None
        except Exception:
            pass


class Stream:
    def __init__(self):
        p = ctypes.c_void_p()
        check(lib().lnc_stream_create(ctypes.byref(p)), "stream")
        self.handle = p.value

    def synchronize(self):
        check(lib().lnc_stream_synchronize(self.handle), "stream sync")

    def close(self):
        if self.handle:
            lib().lnc_stream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Event:
    def __init__(self):
        p = ctypes.c_void_p()
        check(lib().lnc_event_create(ctypes.byref(p)), "event")
        self.handle = p.value

    def record(self, stream=None):
        check(lib().lnc_event_record(self.handle, stream.handle if isinstance(stream, Stream) else stream))

    def wait_on(self, stream):
        """Make later work on `stream` wait for this event."""
        check(lib().lnc_stream_wait_event(stream.handle if isinstance(stream, Stream) else stream, self.handle))

    def elapsed_ms(self, end: "Event") -> float:
        ms = ctypes.c_float()
        check(lib().lnc_event_elapsed_ms(self.handle, end.handle, ctypes.byref(ms)))
        return float(ms.value)

    def __del__(self):
        try:
            if self.handle:
                lib().lnc_event_destroy(self.handle)
        except Exception:
            pass


def kernel_timing(enable: bool):
    check(lib().lnc_kernel_timing_enable(int(bool(enable))))
    check(lib().lnc_kernel_timing_reset())


def kernel_timing_read(kclass: int):
    n = ctypes.c_int64()
    ms = ctypes.c_double()
    check(lib().lnc_kernel_timing_read(int(kclass), ctypes.byref(n), ctypes.byref(ms)))
    return int(n.value), float(ms.value)


def kernel_timing_work(kclass: int) -> float:
    w = ctypes.c_double()
    check(lib().lnc_kernel_timing_work(int(kclass), ctypes.byref(w)))
    return float(w.value)


def device_info():
    sms = ctypes.c_int()
    free = ctypes.c_size_t()
    total = ctypes.c_size_t()
    check(lib().lnc_device_info(ctypes.byref(sms), ctypes.byref(free), ctypes.byref(total)))
    return {"sms": sms.value, "free_bytes": free.value, "total_bytes": total.value}


def device_status():
    check(lib().lnc_device_status(), "device status")


def mixed_report() -> dict:
    """Outcome of this thread's last mixed-precision float solve."""
    it, corr, redone = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_int(0)
    check(lib().lnc_mixed_report(ctypes.byref(it), ctypes.byref(corr), ctypes.byref(redone)), "lnc_mixed_report")
    est = ctypes.c_double(0)
    check(lib().lnc_mixed_error_estimate(ctypes.byref(est)), "lnc_mixed_error_estimate")
    return {"iterations": it.value, "last_correction": corr.value, "redone_fp64": bool(redone.value),
            "error_estimate": None if est.value < 0 else est.value}
