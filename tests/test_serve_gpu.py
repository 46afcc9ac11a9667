"""GPU tests of the serving loop (csrc/serve.cu, linac_gb300/serving.py).

Every request served in a mix (many in flight on their own streams, admitted
by device memory as others finish) must give exactly the result it gives
alone through the drop-in calls (cuda_load_matrix + cuda_row_reduce), and
the small ones must equal the oracle."""
import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads
from linac_gb300.matrix_loader import cuda_load_matrix
from linac_gb300.row_reduce import cuda_row_reduce
from linac_gb300.serving import Server

pytestmark = pytest.mark.gpu


def _mixed_requests(seed: int, n_load: int = 10, n_rref: int = 8):
    """Load+RREF requests (d = 3..5, random primes below 2^31) and RREF
    requests (rank-deficient, uniform, a 64-bit prime, a structured matrix
    whose candidate panels miss pivots)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_load):
        d = 3 + i % 3
        p = workloads.random_prime_below(2**31, rng)
        reqs.append(("load", workloads.serve_load_request(rng, d, p), p))
    for i in range(n_rref):
        p = workloads.random_prime_below(2**31, rng)
        m = int(rng.integers(50, 900))
        n = int(rng.integers(50, 900))
        if i % 3 == 0:
            r = max(1, min(m, n) - int(rng.integers(1, 20)))
            A = workloads.rank_deficient_modp(m, n, r, p, rng).astype(np.uint32)
        else:
            A = rng.integers(0, p, size=(m, n), dtype=np.uint64).astype(np.uint32)
        reqs.append(("rref", A, p))
    A = rng.integers(0, workloads.P61, size=(300, 280), dtype=np.uint64)
    reqs.append(("rref", A, workloads.P61))
    S = rng.integers(0, 2**31 - 1, size=(600, 500), dtype=np.uint64).astype(np.uint32)
    S[:300, :40] = 0  # the first candidate block misses the leading pivots
    reqs.append(("rref", S, 2**31 - 1))
    return reqs


def _alone(kind, payload, p):
    if kind == "load":
        bases, lind = payload
        A = cuda_load_matrix(bases, lind, (bases.shape[0], lind.shape[0]), field_characteristic=p)
    else:
        A = payload
    R, piv = cuda_row_reduce(A, field_characteristic=p, return_pivots=True)
    return A, R, piv


def _submit(srv, kind, payload, p):
    if kind == "load":
        return srv.submit_load(payload[0], payload[1], p)
    return srv.submit(payload, p)


def test_served_results_equal_alone_and_oracle():
    reqs = _mixed_requests(11)
    alone = [_alone(*r) for r in reqs]
    with Server(max_inflight=6) as srv:
        tickets = [_submit(srv, *r) for r in reqs]
        for (kind, payload, p), (A, R_ref, piv_ref), t in zip(reqs, alone, tickets):
            R, piv, rank = t.result()
            assert np.array_equal(R, R_ref), (kind, A.shape, p)
            assert piv == piv_ref and rank == len(piv_ref)
            if A.size <= 400_000:
                R_o, piv_o, _ = oracle.rref_modp(A, p)
                assert np.array_equal(R.astype(np.uint64), R_o)
                assert piv == piv_o
            q_ms, tot_ms = t.latency()
            assert 0.0 <= q_ms <= tot_ms
            t.release()
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["redone"] >= 1  # the structured matrix
        assert st["p99_ms"] >= st["p50_ms"] > 0.0
        assert st["inflight"] == 0 and st["bytes_in_use"] == 0


def test_served_mix_is_repeatable_and_order_independent():
    reqs = _mixed_requests(12, n_load=6, n_rref=6)
    outs = []
    for order in (list(range(len(reqs))), list(reversed(range(len(reqs))))):
        res = [None] * len(reqs)
        with Server(max_inflight=4) as srv:
            ts = {i: _submit(srv, *reqs[i]) for i in order}
            for i, t in ts.items():
                res[i] = t.result()
                t.release()
        outs.append(res)
    for a, b in zip(*outs):
        assert np.array_equal(a[0], b[0]) and a[1] == b[1] and a[2] == b[2]


def test_admission_by_memory_budget():
    rng = np.random.default_rng(3)
    p = 2**31 - 1
    mats = [rng.integers(0, p, size=(700, 700), dtype=np.uint64).astype(np.uint32) for _ in range(6)]
    with Server(budget_bytes=1, max_inflight=4) as tiny:
        with pytest.raises(_lib.AdmissionError):
            tiny.submit(mats[0], p)
    with Server(max_inflight=4) as probe:
        t = probe.submit(mats[0], p)
        t.result()
        need = probe.stats()["peak_bytes"]
        t.release()
    budget = int(need * 1.5)  # room for one request at a time
    with Server(budget_bytes=budget, max_inflight=4) as srv:
        ts = [srv.submit(A, p) for A in mats]
        for A, t in zip(mats, ts):
            R, piv, rank = t.result()
            R_o, piv_o, _ = oracle.rref_modp(A, p)
            assert np.array_equal(R.astype(np.uint64), R_o) and piv == piv_o
            t.release()
        st = srv.stats()
        assert st["peak_bytes"] <= budget and st["completed"] == len(mats)


def test_served_float_and_complex_match_direct_call():
    rng = np.random.default_rng(4)
    A = workloads.conditioned_matrix(200, rng, cond=1e4)
    C = rng.standard_normal((150, 170)) + 1j * rng.standard_normal((150, 170))
    with Server(max_inflight=2) as srv:
        ta, tc = srv.submit(A, 0), srv.submit(C, 0)
        Ra, _, _ = ta.result()
        Rc, _, _ = tc.result()
    assert np.array_equal(Ra, cuda_row_reduce(A, 0))
    assert np.array_equal(Rc, cuda_row_reduce(C, 0))


def test_invalid_requests_fail_at_submit():
    with Server(max_inflight=2) as srv:
        with pytest.raises(ZeroDivisionError):
            srv.submit(np.ones((4, 4), dtype=np.uint32), 2**31 - 2)  # not prime
        with pytest.raises(ValueError):
            srv.submit_load(np.ones((4, 3), dtype=np.uint32), np.array([[5]], dtype=np.uint32), 7)
