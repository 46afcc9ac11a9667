"""Serving loop: RREF and load+RREF requests of mixed size and prime.

linac's callers make one synchronous ``cuda_row_reduce`` (and, for loaded
systems, ``load_matrices``) call per system
(linac/pycuda_row_reduce.py:18-151, linac/pycuda_matrix_loader.py:127-230).
``Server`` keeps a native scheduler (csrc/serve.cu) that admits requests by
device memory as they arrive, keeps each admitted matrix resident from its
load to its result, and runs the requests in flight concurrently on their own
streams; p50 / p99 latency (submit -> result on the host) and throughput are
read from ``Server.stats()``.

    with Server() as srv:
        t1 = srv.submit(A, p)                       # RREF of a host matrix
        t2 = srv.submit_load(bases, lindices, p)    # monomial load, then RREF
        R, pivots, rank = t1.result()

Results land in page-locked host buffers owned by the server's pool; a
ticket's ``result()`` copies them out (``copy=False`` returns views that stay
valid until ``release()``).
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _lib
from .matrix_loader import loader_dtype
from .row_reduce import _as_field_array, field_dtype


class lnc_serve_request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dtype", ctypes.c_int), ("p", ctypes.c_uint64), ("tol", ctypes.c_double),
                ("m", ctypes.c_int64), ("n", ctypes.c_int64),
                ("host_in", ctypes.c_void_p), ("ld_in", ctypes.c_int64),
                ("host_bases", ctypes.c_void_p), ("basis_len", ctypes.c_int64),
                ("host_lindices", ctypes.c_void_p), ("degree", ctypes.c_int64),
                ("host_out", ctypes.c_void_p), ("ld_out", ctypes.c_int64),
                ("host_pivot_cols", ctypes.c_void_p), ("host_rank", ctypes.c_void_p),
                ("flags", ctypes.c_int)]


class lnc_serve_stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "completed", "failed", "redone", "queued", "inflight",
                                              "bytes_in_use", "peak_bytes", "budget_bytes")] + \
               [(k, ctypes.c_double) for k in ("p50_ms", "p99_ms", "mean_ms", "max_ms")]


SERVE_RREF = 1
SERVE_LOAD_RREF = 2

_bound = False


def _bind():
    global _bound
    if _bound:
        return
    vp, i64, ci, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
    _lib.bind("lnc_server_create", [i64, ci, vp])
    _lib.bind("lnc_server_destroy", [vp])
    _lib.bind("lnc_serve_request_bytes", [vp], i64)
    _lib.bind("lnc_serve_submit", [vp, vp, vp])
    _lib.bind("lnc_serve_poll", [vp, i64, vp, vp])
    _lib.bind("lnc_serve_wait", [vp, i64, dbl, vp])
    _lib.bind("lnc_serve_latency", [vp, i64, vp, vp])
    _lib.bind("lnc_serve_release", [vp, i64])
    _lib.bind("lnc_serve_stats_read", [vp, vp])
    _lib.bind("lnc_serve_stats_reset", [vp])
    _bound = True


class _PinnedPool:
    """Page-locked host buffers, reused by size class (powers of two >= 1 MiB)."""

    def __init__(self):
        self._free: dict[int, list] = {}
        self._lock = threading.Lock()

    @staticmethod
    def _cls(nbytes: int) -> int:
        c = 1 << 20
        while c < nbytes:
            c <<= 1
        return c

    def take(self, nbytes: int) -> _lib.PinnedArray:
        c = self._cls(max(int(nbytes), 1))
        with self._lock:
            lst = self._free.get(c)
            if lst:
                return lst.pop()
        return _lib.PinnedArray((c,), np.uint8)

    def give(self, buf: _lib.PinnedArray):
        with self._lock:
            self._free.setdefault(buf.shape[0], []).append(buf)

    def clear(self):
        with self._lock:
            self._free.clear()


def _status_error(status: int, what: str):
    cls = {-2: ZeroDivisionError, -4: MemoryError, -5: _lib.DeviceTimeoutError,
           -6: _lib.AdmissionError}.get(status)
    msg = f"{what}: request failed with status {status}"
    if cls in (_lib.DeviceTimeoutError, _lib.AdmissionError):
        return cls(status, msg)
    if cls is not None:
        return cls(msg)
    return _lib.LinacGpuError(status, msg)


class Ticket:
    """One submitted request."""

    def __init__(self, server: "Server", tid: int, shape, dtype, bufs, out, piv, rank, keep):
        self.server = server
        self.id = tid
        self.shape = shape
        self.dtype = dtype
        self._bufs = bufs
        self._out = out
        self._piv = piv
        self._rank = rank
        self._keep = keep
        self._status = None

    def done(self) -> bool:
        d, s = ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(_lib.lib().lnc_serve_poll(self.server._h, self.id, ctypes.byref(d), ctypes.byref(s)),
                   "lnc_serve_poll")
        if d.value:
            self._status = s.value
        return bool(d.value)

    def wait(self, timeout: float | None = None) -> int:
        if self._status is None:
            s = ctypes.c_int(0)
            _lib.check(_lib.lib().lnc_serve_wait(self.server._h, self.id, -1.0 if timeout is None else float(timeout),
                                                 ctypes.byref(s)), "lnc_serve_wait")
            self._status = s.value
        return self._status

    def latency(self):
        """(queue_ms, total_ms): submit -> admission, submit -> result on the host."""
        self.wait()
        q, t = ctypes.c_double(0), ctypes.c_double(0)
        _lib.check(_lib.lib().lnc_serve_latency(self.server._h, self.id, ctypes.byref(q), ctypes.byref(t)),
                   "lnc_serve_latency")
        return q.value, t.value

    def result(self, copy: bool = True, timeout: float | None = None):
        """(RREF, pivot columns, rank); raises if the request failed."""
        st = self.wait(timeout)
        if st != 0:
            raise _status_error(st, "serve")
        rank = int(self._rank[0])
        R = self._out.copy() if copy else self._out
        return R, [int(x) for x in self._piv[:rank]], rank

    def release(self):
        if self._bufs is None:
            return
        self.wait()
        _lib.check(_lib.lib().lnc_serve_release(self.server._h, self.id), "lnc_serve_release")
        for b in self._bufs:
            self.server._pool.give(b)
        self._bufs = self._out = self._piv = self._rank = self._keep = None

    def __del__(self):
        try:  # the buffers must outlive the device's copies into them
            if self._bufs is not None and getattr(self.server, "_h", None):
                self.release()
        except Exception:
            pass


class Server:
    """Native serving loop on the current device (see module docstring)."""

    def __init__(self, budget_bytes: int = 0, max_inflight: int = 16):
        _bind()
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().lnc_server_create(int(budget_bytes), int(max_inflight), ctypes.byref(h)),
                   "lnc_server_create")
        self._h = h.value
        self._pool = _PinnedPool()

    # -- submission ---------------------------------------------------------------------
    def _outputs(self, m: int, n: int, dtype: np.dtype):
        kmax = max(min(m, n), 1)
        out_b = self._pool.take(m * n * dtype.itemsize)
        piv_b = self._pool.take(8 * kmax + 8)
        out = np.asarray(out_b)[:m * n * dtype.itemsize].view(dtype).reshape(m, n)
        pv = np.asarray(piv_b)[:8 * kmax + 8].view(np.int64)
        return [out_b, piv_b], out, pv[:kmax], pv[kmax:kmax + 1]

    def _submit(self, req: lnc_serve_request) -> int:
        t = ctypes.c_int64(0)
        _lib.check(_lib.lib().lnc_serve_submit(self._h, ctypes.byref(req), ctypes.byref(t)), "lnc_serve_submit")
        return t.value

    def request_bytes(self, req: lnc_serve_request) -> int:
        return int(_lib.lib().lnc_serve_request_bytes(ctypes.byref(req)))

    def submit(self, matrix, field_characteristic: int = 0, flags: int = 0, tol: float = 1e-9) -> Ticket:
        """RREF of a host matrix (same fields and dtypes as cuda_row_reduce)."""
        A = np.asarray(matrix)
        if A.ndim != 2:
            raise ValueError("expected a 2-d matrix")
        p = int(field_characteristic)
        dt = field_dtype(A, p)
        host = _as_field_array(A, dt)
        m, n = host.shape
        in_b = self._pool.take(host.nbytes)
        hin = np.asarray(in_b)[:host.nbytes].view(dt).reshape(m, n)
        np.copyto(hin, host)
        bufs, out, piv, rank = self._outputs(m, n, dt)
        req = lnc_serve_request(kind=SERVE_RREF, dtype=_lib.DTYPE_CODE[np.dtype(dt)], p=p, tol=tol, m=m, n=n,
                                host_in=hin.ctypes.data, ld_in=n, host_out=out.ctypes.data, ld_out=n,
                                host_pivot_cols=piv.ctypes.data, host_rank=rank.ctypes.data, flags=flags)
        try:
            tid = self._submit(req)
        except Exception:
            for b in bufs + [in_b]:
                self._pool.give(b)
            raise
        return Ticket(self, tid, (m, n), dt, bufs + [in_b], out, piv, rank, None)

    def submit_load(self, bases, lindices, field_characteristic: int, flags: int = 0) -> Ticket:
        """Monomial load out[r, c] = prod_t bases[r, lindices[c, t]] (mod p), then
        the RREF of the loaded matrix; the matrix never leaves the device."""
        p = int(field_characteristic)
        if p == 0:
            raise ValueError("load+RREF requests serve prime fields")
        dt = loader_dtype(p)
        B = np.ascontiguousarray(np.asarray(bases).astype(dt, copy=False) % dt.type(p))
        L = np.ascontiguousarray(np.asarray(lindices, dtype=np.uint32))
        if B.ndim != 2 or L.ndim != 2:
            raise ValueError("bases and lindices must be 2-d")
        if L.size and int(L.max()) >= B.shape[1]:
            raise ValueError("lindices refer past the basis columns")
        m, n = B.shape[0], L.shape[0]
        bufs, out, piv, rank = self._outputs(m, n, dt)
        req = lnc_serve_request(kind=SERVE_LOAD_RREF, dtype=_lib.DTYPE_CODE[np.dtype(dt)], p=p, tol=0.0, m=m, n=n,
                                host_bases=B.ctypes.data, basis_len=B.shape[1],
                                host_lindices=L.ctypes.data, degree=L.shape[1],
                                host_out=out.ctypes.data, ld_out=n,
                                host_pivot_cols=piv.ctypes.data, host_rank=rank.ctypes.data, flags=flags)
        try:
            tid = self._submit(req)
        except Exception:
            for b in bufs:
                self._pool.give(b)
            raise
        return Ticket(self, tid, (m, n), dt, bufs, out, piv, rank, (B, L))

    # -- monitoring ---------------------------------------------------------------------
    def stats(self) -> dict:
        st = lnc_serve_stats()
        _lib.check(_lib.lib().lnc_serve_stats_read(self._h, ctypes.byref(st)), "lnc_serve_stats_read")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def reset_stats(self):
        _lib.check(_lib.lib().lnc_serve_stats_reset(self._h), "lnc_serve_stats_reset")

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().lnc_server_destroy(self._h)
            self._h = None
            self._pool.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
