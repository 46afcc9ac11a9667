"""Benchmark of the GB300 RREF path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload rref_u32_20000]

Default workload: the single large RREF over F_p, p = 2^31-1, of a
20,000 x 20,000 uint32 matrix uniform in [0, p) (seeded).  One step is one
full RREF of that matrix.

* ``value``: solves/s with the input already resident in HBM: each step
  restores the pristine input on the device (D2D copy, 1.6 GB) and runs
  ``lnc_rref_device``; K steps timed with CUDA events on the stream, bracketed
  by a device synchronise (and a barrier across ranks).  The 1.6 GB input is
  larger than L2, so no flush is needed between steps.
* ``e2e``: the same metric through the public call ``cuda_row_reduce`` with
  pinned host input / output arrays (host->device copy, RREF, device->host
  copy of the result and the pivots inside the timed region).
* ``roofline``: the dominant kernel class, timed live with CUDA events on its
  launching stream during the timed steps.
* ``cpu_baseline``: the C oracle (restatement of linac's CPU row_reduce) on
  the machine's host cores, timed on the first pivot steps of the same matrix and
  extrapolated by the algorithmic work of the full elimination.
* ``--impl reference``: the reference's CPU algorithm (the oracle port, all
  host threads) on bounded samples of the same workload, one sample per step.

Multi-GPU (torchrun): replicas only -- every rank reduces its own matrix; no
data crosses ranks; ``value`` sums the ranks' solves over the max elapsed time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bit-exact mod-p RREF solves/sec + p99 latency: served/batched vs plain, 1 GB300"
P31 = 2**31 - 1
# README.md:133 of the reference: 20,000^2 RREF mod 2^31-1 in 23.40 s on an A100 80GB
PUBLISHED_20K_SECONDS = 23.40

WORKLOADS = {
    "rref_u32_20000": dict(m=20000, n=20000, p=P31, dtype="u32"),
    "rref_u32_8192": dict(m=8192, n=8192, p=P31, dtype="u32"),
    "rref_u32_4096": dict(m=4096, n=4096, p=P31, dtype="u32"),
}


# ---------------------------------------------------------------------------
# distributed helpers (torch only when launched with WORLD_SIZE > 1)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend="gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def gen_matrix(m: int, n: int, p: int, seed: int, out: np.ndarray | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    A = out if out is not None else np.empty((m, n), dtype=np.uint32)
    chunk = max(1, (1 << 26) // max(n, 1))
    for r0 in range(0, m, chunk):
        r1 = min(m, r0 + chunk)
        A[r0:r1] = rng.integers(0, p, size=(r1 - r0, n), dtype=np.uint32)
    return A


def rref_work(m: int, n: int, pivots) -> float:
    """Algorithmic work W = sum_k m * (n - c_k) field multiply-adds."""
    pv = np.asarray(pivots, dtype=np.float64)
    return float(m) * float(np.sum(n - pv))


# ---------------------------------------------------------------------------
# CPU baseline: the oracle on a bounded sample
# ---------------------------------------------------------------------------
def cpu_sample(m: int, n: int, p: int, seed: int, target_s: float = 8.0):
    """Time the first pivot steps of the elimination with the C oracle on all
    host threads; return (solves_per_s_extrapolated, threads, description)."""
    import oracle
    threads = oracle.default_threads()
    A = gen_matrix(m, n, p, seed).astype(np.uint64)
    steps, total_t, done = 8, 0.0, 0
    while total_t < target_s and done < min(m, n):
        t0 = time.perf_counter()
        k = oracle.rref_modp_partial(A, p, done + steps, threads)
        total_t += time.perf_counter() - t0
        steps = done = k
        steps = max(8, min(steps * 2, min(m, n) - done))
    # work of the sampled steps: pivots 0..done-1 are columns 0..done-1 here
    w_sample = float(m) * sum(n - j for j in range(done))
    w_total = float(m) * (n * (n + 1) / 2.0) if m >= n else rref_work(m, n, range(min(m, n)))
    t_full = total_t * w_total / w_sample
    desc = (f"first {done} pivot steps of the {m}x{n} elimination mod {p} "
            f"({total_t:.1f} s, {100.0 * w_sample / w_total:.2f}% of the work), extrapolated by work")
    return 1.0 / t_full, threads, desc, t_full


# ---------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------
def run_ours(args, dist: Dist):
    from linac_gb300 import _lib, cuda_row_reduce, pinned_empty

    if dist.world > 1:
        _lib.check(_lib.lib().lnc_set_device(dist.local_rank))
    wl = WORKLOADS[args.workload]
    m, n, p = wl["m"], wl["n"], wl["p"]
    L = _lib.lib()
    nbytes = m * n * 4
    seed = 1234 + dist.rank
    host_in = pinned_empty((m, n), np.uint32)
    gen_matrix(m, n, p, seed, out=host_in)
    host_out = pinned_empty((m, n), np.uint32)

    d_src = _lib.DeviceBuffer(nbytes)
    d_work = _lib.DeviceBuffer(nbytes)
    d_out = _lib.DeviceBuffer(nbytes)
    kmax = min(m, n)
    d_piv = _lib.DeviceBuffer(8 * kmax)
    d_rank = _lib.DeviceBuffer(8)
    stream = _lib.Stream()
    d_src.upload(host_in, stream.handle)
    stream.synchronize()

    def step():
        _lib.check(L.lnc_memcpy_d2d(d_work.ptr, d_src.ptr, nbytes, stream.handle))
        _lib.check(L.lnc_rref_device(_lib.LNC_U32, m, n, p, 0.0, d_work.ptr, n, d_out.ptr, n, d_piv.ptr,
                                     d_rank.ptr, stream.handle, args.flags))

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    _lib.device_status()

    # ---- timed region (device-resident) ----
    _lib.kernel_timing(True)
    ev = [(_lib.Event(), _lib.Event()) for _ in range(args.steps)]
    ev_all = (_lib.Event(), _lib.Event())
    dist.barrier()
    _lib.check(L.lnc_device_synchronize())
    launches0 = _lib.launch_count()
    with ClockSampler(dist.local_rank if dist.world > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)) as clk:
        t_host0 = time.perf_counter()
        ev_all[0].record(stream.handle)
        for i in range(args.steps):
            ev[i][0].record(stream.handle)
            step()
            ev[i][1].record(stream.handle)
        ev_all[1].record(stream.handle)
        stream.synchronize()
        t_host = time.perf_counter() - t_host0
    _lib.check(L.lnc_device_synchronize())
    dist.barrier()
    launches = _lib.launch_count() - launches0
    total_ms = ev_all[0].elapsed_ms(ev_all[1])
    lat = [a.elapsed_ms(b) for a, b in ev]
    kt = {name: _lib.kernel_timing_read(kc) for name, kc in
          (("panel", _lib.KC_PANEL), ("trailing", _lib.KC_TRAILING), ("gather", _lib.KC_GATHER))}
    kt_work = {name: _lib.kernel_timing_work(kc) for name, kc in
               (("panel", _lib.KC_PANEL), ("trailing", _lib.KC_TRAILING), ("gather", _lib.KC_GATHER))}
    _lib.kernel_timing(False)
    _lib.device_status()

    # ---- correctness of the timed result (untimed): full rank -> identity
    d_out.download(host_out, stream.handle)
    piv = np.empty(kmax, dtype=np.int64)
    d_piv.download(piv, stream.handle)
    rank = int(np.count_nonzero(piv >= 0))
    ident_ok = bool(rank == n and np.all(piv == np.arange(n)))
    if ident_ok:
        diag = host_out.reshape(-1)[:: n + 1]
        ident_ok = bool(np.all(diag == 1) and int(np.count_nonzero(host_out)) == n)

    t_max = dist.max(total_ms / 1000.0)
    solves = dist.sum(float(args.steps))
    value = solves / t_max

    # ---- end-to-end through the public call with pinned host buffers ----
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    cuda_row_reduce(host_in, p, out=host_out)  # warm
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        R, pv = cuda_row_reduce(host_in, p, out=host_out, return_pivots=True)
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e_value = dist.sum(float(e2e_steps)) / t_e2e

    # ---- roofline of the dominant kernel class ----
    peaks = measured_peaks()
    W = rref_work(m, n, range(n)) if ident_ok else rref_work(m, n, piv[piv >= 0])
    dom = max(("panel", "trailing"), key=lambda k: kt[k][1])
    work = kt_work[dom]
    if dom == "trailing":
        if args.flags & _lib.LNC_FLAG_SIMT_TRAILING:
            # SIMT integer contraction: report its HBM traffic against the copy roofline
            launches = max(1, kt["trailing"][0])
            bytes_per_launch = trailing_bytes(m, n, 128) / launches
            achieved = trailing_bytes(m, n, 128) / (kt["trailing"][1] / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": "trailing_simt_kernel", "achieved": achieved,
                    "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                    "traffic": traffic_per_launch("trailing_simt"),
                    "peak_source": f"{peaks['source']} copy bandwidth",
                    "bytes_per_launch": bytes_per_launch}
        else:
            # tensor-core limb GEMM: 2 * L^2 bf16 flops per field multiply-add (L = 4 digits)
            flops = 2.0 * 16.0 * work
            achieved = flops / (kt["trailing"][1] / 1e3) / 1e12
            peak = peaks["bf16_tflops_sustained"]
            roof = {"bound": "tensor", "kernel": "tc::limb_gemm_kernel", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic_per_launch("limb_gemm"),
                    "peak_source": f"{peaks['source']} bf16 sustained (kernel timed inside a long solve)",
                    "work_unit": "field multiply-adds m*N*128 per launch, x 2*4*4 bf16 flops",
                    "flops_per_launch": flops / max(1, kt["trailing"][0])}
    else:
        achieved = work / (kt["panel"][1] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "panel (cand_panel_kernel / panel_kernel)", "achieved": achieved,
                "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "traffic": traffic_per_launch("panel"), "peak_source": f"{peaks['source']} copy bandwidth",
                "note": "latency-bound: one pivot step per column"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": value / (1.0 / PUBLISHED_20K_SECONDS) if args.workload == "rref_u32_20000" else None,
        "dtype": "u32",
        "data": "synthetic (uniform residues mod 2^31-1, seed 1234+rank)",
        "config": {"workload": f"rref_u32_{m}x{n}_p2^31-1", "m": m, "n": n, "p": p,
                   "parallelism": f"replicas x{dist.world}", "panel_width": 128,
                   "trailing": "simt" if args.flags & _lib.LNC_FLAG_SIMT_TRAILING else "tensor_core",
                   "panel": "exhaustive" if args.flags & (_lib.LNC_FLAG_ROBUST_PANEL | _lib.LNC_FLAG_SIMT_TRAILING)
                   else "candidate block + exhaustive fallback",
                   "l2": "input 1.6 GB > L2 (129 MB); no flush needed"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "min": float(min(lat)), "max": float(max(lat))},
        "bit_exact": ident_ok,
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes + 8 * (kmax + 1), "call": "linac_gb300.cuda_row_reduce"},
        "gpu_launches": launches,
        "kernel_ms": {k: {"launches": v[0], "total_ms": v[1], "work": kt_work[k]} for k, v in kt.items()},
        "roofline": roof,
        "clocks": clk.summary(),
        "host_wall_s": t_host,
        "work_field_macs_per_solve": W,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        v, threads, desc, t_full = cpu_sample(m, n, p, seed, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": threads, "kind": "port", "sample": desc,
                                "extrapolated_s_per_solve": t_full}
    return line


def trailing_work(m: int, n: int, b: int) -> float:
    """Field multiply-adds done by the trailing updates of a full-rank square
    RREF with panel width b: sum over panels of m * b * (n - (q+1) b)."""
    w = 0.0
    for j0 in range(0, n, b):
        N = n - min(n, j0 + b)
        w += float(m) * b * N
    return w


def trailing_bytes(m: int, n: int, b: int) -> float:
    """Algorithmic HBM bytes of the trailing updates (uint32): read and write
    the m x N trailing block, read the transform (m x b) and pivot rows (b x N)."""
    tot = 0.0
    for j0 in range(0, n, b):
        N = n - min(n, j0 + b)
        if N > 0:
            tot += 4.0 * (2 * m * N + m * b + b * N)
    return tot


def traffic_per_launch(kernel: str):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(kernel)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU algorithm (oracle port), bounded samples
# ---------------------------------------------------------------------------
def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return None
    wl = WORKLOADS[args.workload]
    m, n, p = wl["m"], wl["n"], wl["p"]
    import oracle
    oracle.build()
    for _ in range(args.warmup):
        cpu_sample(m, n, p, 1234, target_s=0.5)
    vals, t_fulls = [], []
    t0 = time.perf_counter()
    desc, threads = "", 1
    for _ in range(args.steps):
        v, threads, desc, t_full = cpu_sample(m, n, p, 1234, target_s=args.ref_seconds)
        vals.append(v)
        t_fulls.append(t_full)
    wall = time.perf_counter() - t0
    value = float(np.mean(vals))
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(t_fulls)),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (uniform residues mod 2^31-1, seed 1234)",
        "config": {"workload": f"rref_u32_{m}x{n}_p2^31-1", "m": m, "n": n, "p": p,
                   "parallelism": "cpu (all host threads)"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("linac's CPU row_reduce algorithm (C restatement, OpenMP over rows) on bounded samples of "
                 "the workload, extrapolated by algorithmic work; the reference's pycuda GPU path cannot "
                 "run here (no pycuda, kernels JIT-compiled by pycuda)"),
        "host_wall_s": wall,
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="rref_u32_20000")
    ap.add_argument("--simt", action="store_true", help="force the SIMT trailing update")
    ap.add_argument("--robust-panel", action="store_true", help="force the exhaustive grid-wide panel")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--ref-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    dist = Dist()
    if args.gpus != dist.world and dist.world > 1:
        print(f"warning: --gpus {args.gpus} but WORLD_SIZE {dist.world}", file=sys.stderr)
    if args.impl == "reference":
        line = run_reference(args, dist)
    else:
        from linac_gb300 import _lib  # fails loudly if the library is missing
        args.flags = (_lib.LNC_FLAG_SIMT_TRAILING if args.simt else 0) | \
            (_lib.LNC_FLAG_ROBUST_PANEL if args.robust_panel else 0)
        line = run_ours(args, dist)
    if dist.rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
