"""CPU model of the candidate-block panel's fraction-free elimination (the
steps the cluster kernel runs, in exact integer arithmetic): every other row
becomes a*x - f*v, the pivot column becomes the transform column (-f, 1 in the
pivot row), and the pivot block's inverse is recovered at the end as
    X[t][u] = T[p_t, p_u] * S_u * S_t / (a_0 ... a_(k-1)),   S_u = a_0 ... a_(u-1).
The model must give X = A[P, Q]^-1 and the pivots of the reference's RREF
(first candidate row with a non-zero entry == the oracle's pivot columns)."""
import numpy as np
import pytest

import oracle


def fraction_free_panel(B, p):
    B = [[int(x) % p for x in row] for row in B]
    n, bw = len(B), len(B[0])
    T = [row[:] for row in B]
    isp = [False] * n
    pr, pc, pa = [], [], []
    for c in range(bw):
        pi = next((i for i in range(n) if not isp[i] and T[i][c]), -1)
        if pi < 0:
            continue
        a = T[pi][c]
        f = [T[i][c] for i in range(n)]
        isp[pi] = True
        for cc in list(range(c + 1, bw)) + pc:  # columns to the right, earlier transform columns
            v = T[pi][cc]
            for i in range(n):
                if i != pi:
                    T[i][cc] = (a * T[i][cc] - f[i] * v) % p
        for i in range(n):
            T[i][c] = 1 if i == pi else (-f[i]) % p
        pr.append(pi)
        pc.append(c)
        pa.append(a)
    k = len(pr)
    S = [1] * (k + 1)
    for t in range(k):
        S[t + 1] = S[t] * pa[t] % p
    Pinv = pow(S[k], p - 2, p) if k else 1
    X = [[T[pr[t]][pc[u]] * S[u] % p * S[t] % p * Pinv % p for u in range(k)] for t in range(k)]
    return X, pr, pc


@pytest.mark.parametrize("seed", range(12))
def test_inverse_of_the_pivot_block(seed):
    rng = np.random.default_rng(seed)
    p = [2**31 - 1, 4294967291, 2**61 - 1, 7][seed % 4]
    n, bw = int(rng.integers(1, 14)), int(rng.integers(1, 12))
    B = rng.integers(0, min(p, 2**62), size=(n, bw), dtype=np.uint64) % np.uint64(p)
    B[rng.random((n, bw)) < 0.3] = 0
    if seed % 3 == 0 and n > 1:  # dependent rows
        B[1::2] = (B[0::2][: len(B[1::2])] * np.uint64(3)) % np.uint64(p) if p < 2**32 else B[0::2][: len(B[1::2])]
    X, pr, pc = fraction_free_panel(B.tolist(), p)
    k = len(pr)
    M = [[int(B[pr[t]][pc[u]]) for u in range(k)] for t in range(k)]
    for t in range(k):
        for u in range(k):
            assert sum(X[t][j] * M[j][u] for j in range(k)) % p == (1 if t == u else 0)
    # the pivot columns are the RREF's (uniqueness of the RREF over a field)
    _, piv_ref, rank_ref = oracle.rref_modp(B, p)
    assert sorted(pc) == list(piv_ref) and k == rank_ref
