"""GPU parity of the batched RREF (csrc/batch.cu): every matrix of an uneven
batch with its own prime must equal the oracle bit for bit, including
rank-deficient, tiny, wide / tall and structured matrices that make the
candidate panels miss pivots (those are redone exhaustively)."""
import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads
from linac_gb300.batch import BatchPlan, rref_batch

pytestmark = pytest.mark.gpu


def _batch(count, seed, m_lo=20, m_hi=700):
    rng = np.random.default_rng(seed)
    shapes = workloads.batch_shapes(count, rng, m_lo, m_hi)
    mats, primes = [], []
    for m, n, r, p in shapes:
        mats.append(workloads.rank_deficient_modp(m, n, r, p, rng).astype(np.uint32) if r < min(m, n)
                    else rng.integers(0, p, size=(m, n), dtype=np.uint64).astype(np.uint32))
        primes.append(p)
    return mats, primes


def test_batch_uneven_primes_matches_oracle():
    mats, primes = _batch(48, 1)
    res, pivs = rref_batch(mats, primes, return_pivots=True, tune=False)
    for A, p, R, pv in zip(mats, primes, res, pivs):
        R_ref, piv_ref, _ = oracle.rref_modp(A, p)
        assert np.array_equal(R.astype(np.uint64), R_ref)
        assert pv == piv_ref


def test_batch_barrett_primes_match_oracle():
    """Primes the limb epilogue reduces by Barrett (p = 2 and 2^31 <= p < 2^32) next to
    Montgomery ones in one plan, with matrices wide enough for several column tiles."""
    rng = np.random.default_rng(11)
    specs = [(300, 420, 4294967291), (260, 700, 2147483659), (200, 333, 2), (150, 160, 3221225473),
             (330, 300, 2**31 - 1)]
    mats, primes = [], []
    for m, n, p in specs:
        r = min(m, n) - 7
        mats.append(workloads.rank_deficient_modp(m, n, r, p, rng).astype(np.uint32) if p > 2
                    else rng.integers(0, 2, size=(m, n), dtype=np.uint64).astype(np.uint32))
        primes.append(p)
    res, pivs = rref_batch(mats, primes, return_pivots=True, tune=False)
    for A, p, R, pv in zip(mats, primes, res, pivs):
        R_ref, piv_ref, _ = oracle.rref_modp(A, p)
        assert np.array_equal(R.astype(np.uint64), R_ref)
        assert pv == piv_ref


def test_batch_structured_and_edge_matrices():
    rng = np.random.default_rng(5)
    p = 2**31 - 1
    mats = [np.zeros((40, 30), dtype=np.uint32),                                       # zero
            rng.integers(0, p, size=(1, 300), dtype=np.uint64).astype(np.uint32),      # one row
            rng.integers(0, p, size=(300, 1), dtype=np.uint64).astype(np.uint32),      # one column
            rng.integers(0, p, size=(129, 257), dtype=np.uint64).astype(np.uint32)]    # ragged
    A = rng.integers(0, p, size=(600, 500), dtype=np.uint64).astype(np.uint32)
    A[:300, :40] = 0  # candidate rows miss the leading pivots: exhaustive redo
    mats.append(A)
    primes = [p, 2**31 - 19, 3, 65521, p]
    plan = BatchPlan([M.shape for M in mats], primes)
    try:
        plan.upload_packed(plan.pack(mats))
        for _ in range(2):  # the plan re-runs on the same inputs
            plan.run()
            redone = plan.finish()
            out = plan.unpack(plan.download_packed(np.empty(plan.total_bytes, dtype=np.uint8)))
            for M, q, R in zip(mats, primes, out):
                R_ref, _, _ = oracle.rref_modp(M, q)
                assert np.array_equal(R.astype(np.uint64), R_ref)
        assert redone >= 1
    finally:
        plan.close()


def test_batch_single_large_and_many_small():
    rng = np.random.default_rng(9)
    p = 2**31 - 1
    mats = [rng.integers(0, p, size=(1500, 1400), dtype=np.uint64).astype(np.uint32)]
    mats += [rng.integers(0, p, size=(int(m), int(m) + 3), dtype=np.uint64).astype(np.uint32)
             for m in rng.integers(2, 90, size=60)]
    primes = [p] * len(mats)
    res = rref_batch(mats, primes, tune=False)
    for A, R in zip(mats, res):
        R_ref, _, _ = oracle.rref_modp(A, p)
        assert np.array_equal(R.astype(np.uint64), R_ref)


def test_matmul_and_fill_helpers_exact():
    import ctypes
    from linac_gb300 import _lib
    L = _lib.lib()
    p = 2**31 - 19
    rng = np.random.default_rng(3)
    for (m, k, n) in [(300, 77, 500), (129, 300, 65), (5, 1, 3)]:
        A = rng.integers(0, p, size=(m, k), dtype=np.uint64).astype(np.uint32)
        B = rng.integers(0, p, size=(k, n), dtype=np.uint64).astype(np.uint32)
        dA, dB, dC = _lib.DeviceBuffer(A.nbytes), _lib.DeviceBuffer(B.nbytes), _lib.DeviceBuffer(4 * m * n)
        s = _lib.Stream()
        dA.upload(A, s.handle)
        dB.upload(B, s.handle)
        _lib.check(L.lnc_matmul_modp_device(_lib.LNC_U32, m, k, n, p, dA.ptr, k, dB.ptr, n, dC.ptr, n, s.handle))
        C = np.empty((m, n), dtype=np.uint32)
        dC.download(C, s.handle)
        assert np.array_equal(C.astype(np.uint64), oracle.matmul_modp(A, B, p))
    d = _lib.DeviceBuffer(4 * 100000)
    _lib.check(L.lnc_fill_uniform_modp(d.ptr, 100000, 65521, 7, _lib.LNC_U32, None))
    x = np.empty(100000, dtype=np.uint32)
    d.download(x)
    # 100000 draws from 65521 values: about 51300 distinct are expected
    assert x.max() < 65521 and 48000 < len(np.unique(x)) < 54000


def test_u64_batch_uneven_primes_matches_oracle():
    """64-bit residues: a prime per matrix up to 2^64 - 59, uneven and
    rank-deficient shapes, every result against the oracle."""
    rng = np.random.default_rng(64)
    primes64 = [2**61 - 1, 2**64 - 59, 2**62 - 57, 4294967311]
    mats, primes = [], []
    for i, (m, n) in enumerate([(300, 280), (64, 900), (700, 500), (129, 129), (1, 50), (50, 1), (450, 470),
                                (257, 300)]):
        p = primes64[i % len(primes64)]
        if i % 3 == 2:  # rank deficient: a product of thin factors mod p
            r = max(1, min(m, n) // 2)
            B = rng.integers(0, p, size=(m, r), dtype=np.uint64)
            C = rng.integers(0, p, size=(r, n), dtype=np.uint64)
            A = oracle.matmul_modp(B, C, p)
        else:
            A = rng.integers(0, p, size=(m, n), dtype=np.uint64)
        mats.append(A)
        primes.append(p)
    mats.append(np.zeros((40, 30), dtype=np.uint64))
    primes.append(2**61 - 1)
    res, pivs = rref_batch(mats, primes, return_pivots=True)
    for A, p, R, pv in zip(mats, primes, res, pivs):
        R_ref, piv_ref, _ = oracle.rref_modp(A, p)
        assert R.dtype == np.uint64
        assert np.array_equal(R, R_ref)
        assert pv == piv_ref


def test_pipelined_batch_chunks_match_oracle():
    """The chunked, overlapped path (copy in | graph | copy back per chunk)
    gives every matrix bit-exactly, including a structured one that is redone
    after its chunk was copied back."""
    from linac_gb300.batch import PipelinedBatch
    mats, primes = _batch(40, 21)
    A = np.random.default_rng(3).integers(0, 2**31 - 1, size=(600, 500), dtype=np.uint64).astype(np.uint32)
    A[:300, :40] = 0  # candidate rows miss the leading pivots
    mats.append(A)
    primes.append(2**31 - 1)
    pb = PipelinedBatch([M.shape for M in mats], primes, chunks=3)
    try:
        assert len(pb.plans) == 3
        ins, outs = pb.pack(mats), pb.pinned_buffers()
        for _ in range(2):
            redone = pb.run(ins, outs)
            res = pb.unpack(outs)
            pivs, ranks = pb.pivots_and_ranks()
            for M, q, R, pv in zip(mats, primes, res, pivs):
                R_ref, piv_ref, _ = oracle.rref_modp(M, q)
                assert np.array_equal(R.astype(np.uint64), R_ref)
                assert [int(x) for x in pv] == piv_ref
        assert redone >= 1
        # the same chunks through one launch of the grouped graph, twice
        for _ in range(2):
            for p, buf in zip(pb.plans, ins):
                p.upload_packed(buf)
                _lib.check(_lib.lib().lnc_memset(p.d_out.ptr, 0xFF, p.total_bytes, p.stream.handle))
            assert pb.run_graph() >= 1
            outs = [p.download_packed(np.zeros_like(buf)) for p, buf in zip(pb.plans, ins)]
            res = pb.unpack(outs)
            pivs, _ = pb.pivots_and_ranks()
            for M, q, R, pv in zip(mats, primes, res, pivs):
                R_ref, piv_ref, _ = oracle.rref_modp(M, q)
                assert np.array_equal(R.astype(np.uint64), R_ref)
                assert [int(x) for x in pv] == piv_ref
    finally:
        pb.close()


@pytest.mark.parametrize("wide", [False, True])
def test_batch_with_empty_matrices(wide):
    """Empty matrices in a batch come back as empty RREFs without pivots; the
    others are reduced as usual (32- and 64-bit residues)."""
    p = 2**61 - 1 if wide else 2**31 - 1
    rng = np.random.default_rng(8)
    A = rng.integers(0, p, size=(50, 60), dtype=np.uint64)
    mats = [np.zeros((0, 7), dtype=np.uint64), A, np.zeros((5, 0), dtype=np.uint64)]
    res, pivs = rref_batch(mats, [p, p, p], return_pivots=True, tune=False)
    assert res[0].shape == (0, 7) and res[2].shape == (5, 0) and pivs[0] == [] and pivs[2] == []
    R_ref, piv_ref, _ = oracle.rref_modp(A, p)
    assert np.array_equal(res[1].astype(np.uint64), R_ref) and pivs[1] == piv_ref
