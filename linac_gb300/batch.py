"""Batched RREF of many uneven matrices over F_p (a prime per matrix).

linac reduces one matrix per ``cuda_row_reduce`` call and its callers loop
(linac/vector_spaces/over_function_fields.py:74-101,
linac/linear_system_solver.py:41-45).  ``rref_batch`` reduces a whole list in
one CUDA-graph launch of the tensor-core path (csrc/batch.cu); ``BatchPlan``
keeps the device buffers and the captured graph so that a batch of the same
shapes can be re-run on new contents without re-planning.

The work split of the contraction kernels (output tiles per CTA) and the
candidate-block height are chosen by ``autotune`` from timings on a sample of
the batch, cached per size signature in ``$LINAC_GB300_CACHE`` (default
``~/.cache/linac_gb300/autotune.json``).
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import _lib
from .primes import check_prime


class lnc_batch_matrix(ctypes.Structure):
    _fields_ = [("p", ctypes.c_uint64), ("m", ctypes.c_int64), ("n", ctypes.c_int64),
                ("dev_in", ctypes.c_void_p), ("ld_in", ctypes.c_int64),
                ("dev_out", ctypes.c_void_p), ("ld_out", ctypes.c_int64),
                ("dev_pivot_cols", ctypes.c_void_p), ("dev_rank", ctypes.c_void_p)]


_bound = False


def _bind():
    global _bound
    if _bound:
        return
    vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    _lib.bind("lnc_batch_plan_create", [ci, vp, i64, ci, ci, vp, vp])
    _lib.bind("lnc_batch_plan_run", [vp, vp])
    _lib.bind("lnc_batch_plan_finish", [vp, vp, vp])
    _lib.bind("lnc_batch_plan_bytes", [vp], i64)
    _lib.bind("lnc_batch_plan_destroy", [vp])
    _lib.bind("lnc_rref_batch_device", [ci, vp, i64, vp, ci])
    _lib.bind("lnc_rref_float_batch", [ci, vp, i64, ctypes.c_double, ci, ci, vp])
    _lib.bind("lnc_batch_group_create", [vp, i64, vp])
    _lib.bind("lnc_batch_group_run", [vp, vp])
    _lib.bind("lnc_batch_group_destroy", [vp])
    _bound = True


class lnc_mixed_result(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("redone_fp64", ctypes.c_int), ("error_estimate", ctypes.c_double)]


def _align(x: int, a: int = 256) -> int:
    return (x + a - 1) // a * a


class BatchPlan:
    """Device buffers + captured graph for one list of matrix shapes."""

    def __init__(self, shapes, primes, tiles_per_cta: int = 0, cand_rows: int = 0, stream=None):
        _bind()
        self.shapes = [(int(m), int(n)) for m, n in shapes]
        self.primes = [int(p) for p in primes]
        if len(self.shapes) != len(self.primes) or not self.shapes:
            raise ValueError("need one prime per matrix and at least one matrix")
        for p in set(self.primes):
            if p >= 2**32:
                raise ValueError("the batched path serves primes below 2^32")
            check_prime(p)
        self.stream = stream if stream is not None else _lib.Stream()
        s = self.stream.handle
        self.offsets = []
        off = 0
        for m, n in self.shapes:
            self.offsets.append(off)
            off += _align(4 * m * n)
        self.total_bytes = off
        self.d_in = _lib.DeviceBuffer(off)
        self.d_out = _lib.DeviceBuffer(off)
        kmax = [min(m, n) for m, n in self.shapes]
        self.piv_off = np.concatenate([[0], np.cumsum(kmax)]).astype(np.int64)
        self.d_piv = _lib.DeviceBuffer(8 * int(self.piv_off[-1]) + 8)
        self.d_rank = _lib.DeviceBuffer(8 * len(self.shapes))
        descs = (lnc_batch_matrix * len(self.shapes))()
        for i, ((m, n), p) in enumerate(zip(self.shapes, self.primes)):
            d = descs[i]
            d.p, d.m, d.n = p, m, n
            d.dev_in = self.d_in.ptr + self.offsets[i]
            d.ld_in = n
            d.dev_out = self.d_out.ptr + self.offsets[i]
            d.ld_out = n
            d.dev_pivot_cols = self.d_piv.ptr + 8 * int(self.piv_off[i])
            d.dev_rank = self.d_rank.ptr + 8 * i
        self._descs = descs
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().lnc_batch_plan_create(_lib.LNC_U32, ctypes.addressof(descs), len(self.shapes),
                                                    int(tiles_per_cta), int(cand_rows), s, ctypes.byref(h)),
                   "lnc_batch_plan_create")
        self.handle = h.value
        self.redone = 0

    @property
    def device_bytes(self) -> int:
        return int(_lib.lib().lnc_batch_plan_bytes(self.handle)) + 2 * self.total_bytes

    def upload_packed(self, host_packed: np.ndarray):
        """Copy a packed host buffer (layout of ``pack``) to the device input."""
        _lib.check(_lib.lib().lnc_memcpy_h2d(self.d_in.ptr, host_packed.ctypes.data, self.total_bytes,
                                             self.stream.handle))

    def pack(self, matrices, out: np.ndarray | None = None) -> np.ndarray:
        """Pack matrices into one host buffer (uint8 view of the device layout)."""
        buf = out if out is not None else np.empty(self.total_bytes, dtype=np.uint8)
        for (m, n), off, A in zip(self.shapes, self.offsets, matrices):
            view = buf[off:off + 4 * m * n].view(np.uint32).reshape(m, n)
            np.copyto(view, A, casting="unsafe")
        return buf

    def run(self):
        _lib.check(_lib.lib().lnc_batch_plan_run(self.handle, self.stream.handle), "lnc_batch_plan_run")

    def finish(self) -> int:
        n = ctypes.c_int64(0)
        _lib.check(_lib.lib().lnc_batch_plan_finish(self.handle, self.stream.handle, ctypes.byref(n)),
                   "lnc_batch_plan_finish")
        self.redone = int(n.value)
        return self.redone

    def download_packed(self, host_packed: np.ndarray):
        _lib.check(_lib.lib().lnc_memcpy_d2h(host_packed.ctypes.data, self.d_out.ptr, self.total_bytes,
                                             self.stream.handle))
        self.stream.synchronize()
        return host_packed

    def unpack(self, host_packed: np.ndarray):
        return [host_packed[off:off + 4 * m * n].view(np.uint32).reshape(m, n)
                for (m, n), off in zip(self.shapes, self.offsets)]

    def pivots_and_ranks(self):
        piv = np.empty(int(self.piv_off[-1]) + 1, dtype=np.int64)
        self.d_piv.download(piv, self.stream.handle)
        ranks = np.empty(len(self.shapes), dtype=np.int64)
        self.d_rank.download(ranks, self.stream.handle)
        return [list(piv[self.piv_off[i]:self.piv_off[i] + ranks[i]]) for i in range(len(self.shapes))], ranks

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().lnc_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def chunk_bounds(shapes, chunks: int):
    """Cut a list of matrix shapes into at most `chunks` consecutive, non-empty
    ranges [a, b) of about equal work (m n min(m, n) each)."""
    work = np.array([m * n * min(m, n) for m, n in shapes], dtype=np.float64)
    if len(work) == 0:
        return []
    cum = np.cumsum(work)
    chunks = max(1, min(int(chunks), len(shapes)))
    cuts = [0] + [int(np.searchsorted(cum, cum[-1] * k / chunks)) + 1 for k in range(1, chunks)] + [len(shapes)]
    cuts = sorted(set(min(max(c, 0), len(shapes)) for c in cuts))
    return [(a, b) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]


class PipelinedBatch:
    """A batch cut into consecutive chunks of about equal work, one BatchPlan
    (one CUDA graph) each, so that the host-to-device copy of chunk k + 1, the
    graph of chunk k and the copy back of chunk k - 1 overlap: the copies run
    on two copy streams, every graph on its own stream behind an event of its
    input copy, and the graphs of consecutive chunks overlap one another (a
    graph's last steps hold few large matrices).  At most ``window`` chunk
    graphs run at once in ``run`` (graph k starts after graph k - window has
    finished), so that finished chunks stream back while later ones compute
    instead of all finishing together; 0 lets every graph start as soon as
    its input has landed.  On the 4096-matrix batch in 32 chunks a window of 6
    measured best (401 ms per batch end to end; unlimited 412, 2: 440, 1:
    566)."""

    def __init__(self, shapes, primes, chunks: int = 4, tiles_per_cta: int = 0, cand_rows: int = 0,
                 window: int = 6):
        _bind()
        shapes = [(int(m), int(n)) for m, n in shapes]
        primes = [int(p) for p in primes]
        if len(shapes) != len(primes) or not shapes:
            raise ValueError("need one prime per matrix and at least one matrix")
        self.bounds = chunk_bounds(shapes, chunks)
        self.plans = [BatchPlan(shapes[a:b], primes[a:b], tiles_per_cta, cand_rows, stream=_lib.Stream())
                      for a, b in self.bounds]
        self.s_in, self.s_out = _lib.Stream(), _lib.Stream()
        self._group = None
        self.s_group = None
        self.ev_in = [_lib.Event() for _ in self.plans]
        self.ev_done = [_lib.Event() for _ in self.plans]
        self.window = max(0, int(window))
        self.redone = 0

    @property
    def device_bytes(self) -> int:
        return sum(p.device_bytes for p in self.plans)

    def pinned_buffers(self):
        """One pinned host buffer per chunk (layout of BatchPlan.pack)."""
        return [_lib.PinnedArray((p.total_bytes,), np.uint8).array for p in self.plans]

    def pack(self, matrices, bufs=None):
        bufs = bufs if bufs is not None else self.pinned_buffers()
        for (a, b), p, buf in zip(self.bounds, self.plans, bufs):
            p.pack(matrices[a:b], out=buf)
        return bufs

    def run(self, host_in, host_out) -> int:
        """Copy every chunk in, reduce it and copy it back, overlapped;
        returns the number of matrices redone by the exhaustive path."""
        L = _lib.lib()
        for k, p in enumerate(self.plans):
            _lib.check(L.lnc_memcpy_h2d(p.d_in.ptr, host_in[k].ctypes.data, p.total_bytes, self.s_in.handle))
            self.ev_in[k].record(self.s_in)
            self.ev_in[k].wait_on(p.stream)
            if self.window and k >= self.window:
                self.ev_done[k - self.window].wait_on(p.stream)
            p.run()
            self.ev_done[k].record(p.stream)
            self.ev_done[k].wait_on(self.s_out)
            _lib.check(L.lnc_memcpy_d2h(host_out[k].ctypes.data, p.d_out.ptr, p.total_bytes, self.s_out.handle))
        self.s_out.synchronize()
        self.redone = 0
        for k, p in enumerate(self.plans):
            r = p.finish()
            if r:  # matrices redone after their chunk was copied back: copy the chunk again
                p.download_packed(host_out[k])
            self.redone += r
        return self.redone

    def run_device(self) -> int:
        """Reduce the chunks already on the device (their graphs overlap on
        their own streams); returns the number of matrices redone."""
        for p in self.plans:
            p.run()
        self.redone = sum(p.finish() for p in self.plans)
        return self.redone

    def launch_graph(self):
        """One launch, on ``self.s_group``, of a graph whose child graphs are
        every chunk's graph (no dependency between chunks); asynchronous, and
        ordered after the work already queued on every chunk's stream."""
        if self._group is None:
            h = ctypes.c_void_p()
            arr = (ctypes.c_void_p * len(self.plans))(*[p.handle for p in self.plans])
            _lib.check(_lib.lib().lnc_batch_group_create(arr, len(self.plans), ctypes.byref(h)),
                       "lnc_batch_group_create")
            self._group = h.value
            self.s_group = _lib.Stream()
        for ev, p in zip(self.ev_in, self.plans):
            ev.record(p.stream)
            ev.wait_on(self.s_group)
        _lib.check(_lib.lib().lnc_batch_group_run(self._group, self.s_group.handle), "lnc_batch_group_run")

    def run_graph(self) -> int:
        """Reduce the chunks already on the device with one graph launch
        (launch_graph); returns the number of matrices redone."""
        self.launch_graph()
        self.s_group.synchronize()
        self.redone = sum(p.finish() for p in self.plans)
        return self.redone

    def unpack(self, host_out):
        res = []
        for p, buf in zip(self.plans, host_out):
            res.extend(p.unpack(buf))
        return res

    def pivots_and_ranks(self):
        pivs, ranks = [], []
        for p in self.plans:
            pv, rk = p.pivots_and_ranks()
            pivs.extend(pv)
            ranks.extend(int(x) for x in rk)
        return pivs, np.array(ranks, dtype=np.int64)

    def close(self):
        if self._group is not None:
            _lib.lib().lnc_batch_group_destroy(self._group)
            self._group = None
        for p in self.plans:
            p.close()


def _residues_u64(A: np.ndarray, q: int) -> np.ndarray:
    """Entries of A reduced to [0, q) as uint64 (integer or object arrays)."""
    if A.dtype == object:
        return np.vectorize(lambda x: int(x) % q, otypes=[object])(A).astype(np.uint64)
    if A.dtype.kind == "u":
        return A.astype(np.uint64) % np.uint64(q)
    if A.dtype.kind != "i":
        raise TypeError("F_p batches take integer matrices")
    a = A.astype(np.int64)
    if q < 2**63:
        return np.mod(a, np.int64(q)).astype(np.uint64)
    # q > |a|: a mod q is a, or a + q for a negative a (two's complement wraps to it)
    return a.view(np.uint64) + (a < 0).astype(np.uint64) * np.uint64(q)


# batches of at least this many input bytes are cut into overlapped chunks
PIPELINE_BYTES = 256 << 20


def pipeline_chunks(count: int) -> int:
    """Chunks of a pipelined batch: about 128 matrices each, 2 to 32 (the 4096-matrix benchmark batch
    end to end: 7.7k solves/s with 4 chunks, 8.6k with 16, 9.5k with 32; 10.4k on the device)."""
    return max(2, min(32, count // 128))


def rref_batch(matrices, primes, return_pivots: bool = False, tune: bool = True):
    """RREF of every matrix of the list over F_{primes[i]}.

    Returns the list of RREFs, and the pivot columns when ``return_pivots``.
    With every prime below 2^32 the residues are uint32 and one plan (one CUDA
    graph) covers the whole list; with any prime above, every matrix is
    reduced as uint64 residues (linac's dtype rule,
    linac/pycuda_row_reduce.py:41-46) through the single-matrix 64-bit path
    on concurrent worker streams.
    """
    mats = [np.asarray(A) for A in matrices]
    if isinstance(primes, (int, np.integer)):
        primes = [int(primes)] * len(mats)
    if len(primes) != len(mats):
        raise ValueError("one prime per matrix")
    if any(A.ndim != 2 for A in mats):
        raise ValueError("rref_batch expects 2-D matrices")
    wide = any(int(q) > 2**32 - 1 for q in primes)
    empty = [i for i, A in enumerate(mats) if A.size == 0]
    if empty:  # an empty matrix is its own RREF, without pivots
        full = [i for i, A in enumerate(mats) if A.size != 0]
        dt = np.uint64 if wide else np.uint32
        res = [np.zeros(A.shape, dtype=dt) for A in mats]
        pivs = [[] for _ in mats]
        if full:
            sub = rref_batch([mats[i] for i in full], [primes[i] for i in full], return_pivots=True, tune=tune)
            for i, R, pv in zip(full, *sub):
                res[i], pivs[i] = R, pv
        return (res, pivs) if return_pivots else res
    if wide:
        cb = ConcurrentBatch([A.shape for A in mats], np.uint64, primes)
        packed = cb.pack([_residues_u64(A, int(q)) for A, q in zip(mats, primes)])
        cb.upload(packed)
        cb.run()
        res = [R.copy() for R in cb.unpack(cb.download())]
        if return_pivots:
            pivs, _ = cb.pivots_and_ranks()
            return res, [[int(x) for x in p] for p in pivs]
        return res
    shapes = [A.shape for A in mats]
    tpc, cand = autotune(shapes, primes) if tune else (0, 0)
    if sum(4 * m * n for m, n in shapes) >= PIPELINE_BYTES and len(shapes) >= 8:
        pb = PipelinedBatch(shapes, primes, pipeline_chunks(len(shapes)), tpc, cand)
        try:
            outs = pb.pinned_buffers()
            pb.run(pb.pack(mats), outs)
            res = [R.copy() for R in pb.unpack(outs)]
            if return_pivots:
                pivs, _ = pb.pivots_and_ranks()
                return res, [[int(x) for x in p] for p in pivs]
            return res
        finally:
            pb.close()
    plan = BatchPlan(shapes, primes, tpc, cand)
    try:
        host = plan.pack(mats)
        plan.upload_packed(host)
        plan.run()
        plan.finish()
        out = plan.download_packed(np.empty(plan.total_bytes, dtype=np.uint8))
        res = [R.copy() for R in plan.unpack(out)]
        if return_pivots:
            pivs, _ = plan.pivots_and_ranks()
            return res, [[int(x) for x in p] for p in pivs]
        return res
    finally:
        plan.close()


class ConcurrentBatch:
    """Device buffers for a list of matrices (inputs and outputs packed,
    256-byte aligned) and their descriptors; ``run`` solves them all, each
    through the single-matrix path, on concurrent worker streams.

    float64 / complex128 batches go to lnc_rref_float_batch; uint64 batches
    (64-bit residues, ``primes[i]`` per matrix) to lnc_rref_batch_device."""

    DTYPES = (np.dtype(np.float64), np.dtype(np.complex128), np.dtype(np.uint64))

    def __init__(self, shapes, dtype, primes=None):
        _bind()
        self.dtype = np.dtype(dtype)
        if self.dtype not in self.DTYPES:
            raise ValueError(f"{type(self).__name__} holds {', '.join(str(d) for d in self.DTYPES)} matrices")
        self.modp = self.dtype == np.dtype(np.uint64)
        if self.modp:
            if primes is None:
                raise ValueError("a uint64 batch needs a prime per matrix")
            primes = [int(primes)] * len(shapes) if isinstance(primes, (int, np.integer)) else [int(q) for q in primes]
            if len(primes) != len(shapes):
                raise ValueError("one prime per matrix")
            for q in primes:
                check_prime(q)
        self.primes = primes
        self.code = _lib.DTYPE_CODE[self.dtype]
        self.shapes = [(int(m), int(n)) for m, n in shapes]
        elt = self.dtype.itemsize
        self.offsets, off = [], 0
        for m, n in self.shapes:
            self.offsets.append(off)
            off += _align(elt * m * n)
        self.total_bytes = off
        self.d_in = _lib.DeviceBuffer(off)
        self.d_out = _lib.DeviceBuffer(off)
        kmax = [min(m, n) for m, n in self.shapes]
        self.piv_off = np.concatenate([[0], np.cumsum(kmax)]).astype(np.int64)
        self.d_piv = _lib.DeviceBuffer(8 * int(self.piv_off[-1]) + 8)
        self.d_rank = _lib.DeviceBuffer(8 * max(1, len(self.shapes)))
        descs = (lnc_batch_matrix * max(1, len(self.shapes)))()
        for i, (m, n) in enumerate(self.shapes):
            d = descs[i]
            d.p, d.m, d.n = (self.primes[i] if self.modp else 0), m, n
            d.dev_in = self.d_in.ptr + self.offsets[i]
            d.ld_in = n
            d.dev_out = self.d_out.ptr + self.offsets[i]
            d.ld_out = n
            d.dev_pivot_cols = self.d_piv.ptr + 8 * int(self.piv_off[i])
            d.dev_rank = self.d_rank.ptr + 8 * i
        self._descs = descs
        self.reports = (lnc_mixed_result * max(1, len(self.shapes)))()

    def pack(self, matrices) -> np.ndarray:
        buf = _lib.PinnedArray((self.total_bytes,), np.uint8).array
        for (m, n), off, A in zip(self.shapes, self.offsets, matrices):
            np.copyto(buf[off:off + self.dtype.itemsize * m * n].view(self.dtype).reshape(m, n), A)
        return buf

    def upload(self, packed: np.ndarray, stream=None):
        _lib.check(_lib.lib().lnc_memcpy_h2d(self.d_in.ptr, packed.ctypes.data, self.total_bytes, stream))
        _lib.check(_lib.lib().lnc_stream_synchronize(stream))

    def run(self, mixed: bool = True, workers: int = 16, tol: float = 1e-9):
        if self.modp:
            _lib.check(_lib.lib().lnc_rref_batch_device(self.code, ctypes.addressof(self._descs), len(self.shapes),
                                                        None, 0), "lnc_rref_batch_device")
            return
        flags = _lib.LNC_FLAG_MIXED if mixed else 0
        _lib.check(_lib.lib().lnc_rref_float_batch(self.code, ctypes.addressof(self._descs), len(self.shapes),
                                                   float(tol), flags, int(workers),
                                                   ctypes.addressof(self.reports)), "lnc_rref_float_batch")

    def download(self, packed: np.ndarray | None = None, stream=None) -> np.ndarray:
        packed = packed if packed is not None else _lib.PinnedArray((self.total_bytes,), np.uint8).array
        _lib.check(_lib.lib().lnc_memcpy_d2h(packed.ctypes.data, self.d_out.ptr, self.total_bytes, stream))
        _lib.check(_lib.lib().lnc_stream_synchronize(stream))
        return packed

    def unpack(self, packed: np.ndarray):
        return [packed[off:off + self.dtype.itemsize * m * n].view(self.dtype).reshape(m, n)
                for (m, n), off in zip(self.shapes, self.offsets)]

    def pivots_and_ranks(self):
        piv = np.empty(int(self.piv_off[-1]) + 1, dtype=np.int64)
        self.d_piv.download(piv)
        ranks = np.empty(max(1, len(self.shapes)), dtype=np.int64)
        self.d_rank.download(ranks)
        return [list(piv[self.piv_off[i]:self.piv_off[i] + ranks[i]]) for i in range(len(self.shapes))], \
            ranks[:len(self.shapes)]

    def report_list(self):
        return [{"iterations": r.iterations, "redone_fp64": bool(r.redone_fp64),
                 "error_estimate": None if r.redone_fp64 else r.error_estimate}
                for r in self.reports[:len(self.shapes)]]


class FloatBatch(ConcurrentBatch):
    """A ConcurrentBatch of float64 / complex128 matrices."""

    DTYPES = (np.dtype(np.float64), np.dtype(np.complex128))

    def __init__(self, shapes, dtype):
        super().__init__(shapes, dtype)


def rref_float_batch(matrices, mixed: bool = True, workers: int = 16, return_pivots: bool = False,
                     return_reports: bool = False, tol: float = 1e-9):
    """RREF of every float64 / complex128 matrix of the list (linac's float
    semantics: rows pre-scaled by their largest |a|, partial pivoting,
    threshold ``tol``), solved concurrently by ``workers`` host threads on
    their own streams.  ``mixed=True`` uses the mixed-precision path (its
    per-matrix reports, with the error estimate, when ``return_reports``).
    All matrices take one element type: complex128 if any is complex."""
    mats = [np.asarray(A) for A in matrices]
    cplx = any(np.iscomplexobj(A) and np.any(A.imag) for A in mats)
    dt = np.complex128 if cplx else np.float64
    fb = FloatBatch([A.shape for A in mats], dt)
    fb.upload(fb.pack([A.real if (not cplx and np.iscomplexobj(A)) else A for A in mats]))
    fb.run(mixed=mixed, workers=workers, tol=tol)
    res = [R.copy() for R in fb.unpack(fb.download())]
    out = [res]
    if return_pivots:
        pivs, _ = fb.pivots_and_ranks()
        out.append([[int(x) for x in p] for p in pivs])
    if return_reports:
        out.append(fb.report_list())
    return out[0] if len(out) == 1 else tuple(out)


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
TILE_CHOICES = (4, 8, 16, 32)
CAND_CHOICES = (136, 160)


def _cache_path() -> str:
    d = os.environ.get("LINAC_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "linac_gb300")
    return os.path.join(d, "autotune.json")


def signature(shapes) -> str:
    """Size signature of a batch: count, mean and max rows / columns, bucketed."""
    ms = np.array([s[0] for s in shapes], dtype=np.float64)
    ns = np.array([s[1] for s in shapes], dtype=np.float64)
    def b(x):  # half-octave bucket
        return int(round(np.log2(max(x, 1.0)) * 2))
    return f"c{b(len(shapes))}-m{b(ms.mean())}-{b(ms.max())}-n{b(ns.mean())}-{b(ns.max())}"


def _load_cache() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(cache: dict):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass


def autotune(shapes, primes, sample: int = 96, reps: int = 2, seed: int = 0, force: bool = False):
    """(tiles_per_cta, cand_rows) for a batch of these shapes.

    Times every combination of TILE_CHOICES x CAND_CHOICES on a sample of up
    to `sample` matrices drawn from the batch (random residues), keeps the
    fastest and caches it under the batch's size signature.
    """
    key = signature(shapes)
    cache = _load_cache()
    if not force and key in cache:
        v = cache[key]
        return int(v["tiles_per_cta"]), int(v["cand_rows"])
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(shapes), size=min(sample, len(shapes)), replace=False)
    sub_shapes = [shapes[i] for i in idx]
    sub_primes = [int(primes[i]) for i in idx]
    mats = [rng.integers(0, p, size=s, dtype=np.uint64).astype(np.uint32) for s, p in zip(sub_shapes, sub_primes)]
    best, timings = None, {}
    for tpc in TILE_CHOICES:
        for cand in CAND_CHOICES:
            plan = BatchPlan(sub_shapes, sub_primes, tpc, cand)
            try:
                plan.upload_packed(plan.pack(mats))
                plan.run()
                plan.finish()
                t0 = time.perf_counter()
                for _ in range(reps):  # each run re-reads the uploaded inputs
                    plan.run()
                plan.stream.synchronize()
                dt = (time.perf_counter() - t0) / reps
            finally:
                plan.close()
            timings[f"{tpc}x{cand}"] = dt
            if best is None or dt < best[0]:
                best = (dt, tpc, cand)
    cache[key] = {"tiles_per_cta": best[1], "cand_rows": best[2], "seconds": best[0], "timings": timings}
    _store_cache(cache)
    return best[1], best[2]
