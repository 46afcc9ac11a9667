"""CPU checks of the host helpers of linac_gb300.linear_algebra (semantics of
linac/linear_algebra_tools.py:10-77): pivots, zero-row dropping and the
RREF <-> canonical kernel round trip, for integer and float RREFs."""
import numpy as np
import pytest

from linac_gb300.linear_algebra import (_host_kernel, drop_bottom_zero_rows,
                                        non_pivot_columns_from_row_reduced_echelon_form,
                                        pivot_columns_from_row_reduced_echelon_form,
                                        row_reduced_echelon_form_from_canonical_kernel)


def _rref(dt, piv, n, seed):
    rng = np.random.default_rng(seed)
    R = np.zeros((len(piv), n), dtype=dt)
    for t, c in enumerate(piv):
        R[t, c] = 1
        for j in range(c + 1, n):
            if j not in piv:
                R[t, j] = rng.integers(2, 1000)
    return R


@pytest.mark.parametrize("dt", [np.uint32, np.int64, np.float64])
def test_round_trip_and_pivots(dt):
    piv = [0, 2, 5, 6, 9]
    R = _rref(dt, piv, 12, 1)
    assert pivot_columns_from_row_reduced_echelon_form(R) == piv
    assert non_pivot_columns_from_row_reduced_echelon_form(R) == [1, 3, 4, 7, 8, 10, 11]
    K = _host_kernel(R, piv)
    assert K.shape == (12, 7) and K.dtype == np.result_type(R.dtype, int)
    assert not (R.astype(np.float64) @ K.astype(np.float64)).any()
    back = row_reduced_echelon_form_from_canonical_kernel(K)
    assert np.array_equal(back.astype(np.float64), R.astype(np.float64))


def test_drop_bottom_zero_rows():
    R = _rref(np.float64, [1, 3], 6, 2)
    Z = np.vstack([R, np.zeros((3, 6))])
    assert np.array_equal(drop_bottom_zero_rows(Z), R)
    assert drop_bottom_zero_rows(np.zeros((3, 4))).shape == (0, 4)
