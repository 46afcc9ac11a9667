"""Host logic of the batched paths (no GPU): chunking of a pipelined batch
and the reduction of integer matrices to uint64 residues."""
import numpy as np

from linac_gb300.batch import _residues_u64, chunk_bounds


def test_chunk_bounds_cover_consecutively_with_balanced_work():
    rng = np.random.default_rng(0)
    shapes = [(int(m), int(m) + 3) for m in rng.integers(64, 2048, size=500)]
    for chunks in (1, 2, 3, 4, 7):
        b = chunk_bounds(shapes, chunks)
        assert b[0][0] == 0 and b[-1][1] == len(shapes)
        assert all(x[1] == y[0] for x, y in zip(b[:-1], b[1:]))
        assert all(hi > lo for lo, hi in b)
        assert len(b) <= chunks
        work = [sum(m * n * min(m, n) for m, n in shapes[lo:hi]) for lo, hi in b]
        assert max(work) <= 1.5 * sum(work) / len(b)


def test_chunk_bounds_edge_cases():
    assert chunk_bounds([], 4) == []
    assert chunk_bounds([(5, 5)], 4) == [(0, 1)]
    assert chunk_bounds([(5, 5), (6, 6)], 8) in ([(0, 1), (1, 2)], [(0, 2)])
    one_big = [(2000, 2000)] + [(10, 10)] * 9
    b = chunk_bounds(one_big, 4)
    assert b[0] == (0, 1) and b[-1][1] == 10


def test_residues_u64_exact_for_every_integer_kind():
    for q in (2**61 - 1, 2**64 - 59, 4294967311):
        a = np.array([[-1, 5, -(2**62)], [2**62, -(2**63), 2**63 - 1]], dtype=np.int64)
        want = [int(x) % q for x in a.ravel()]
        assert [int(x) for x in _residues_u64(a, q).ravel()] == want
        u = np.array([[0, 2**64 - 1, q]], dtype=np.uint64)
        assert [int(x) for x in _residues_u64(u, q).ravel()] == [int(x) % q for x in u.ravel()]
        o = np.array([[-(2**70), 3 * q + 1]], dtype=object)
        assert [int(x) for x in _residues_u64(o, q).ravel()] == [int(x) % q for x in o.ravel()]
