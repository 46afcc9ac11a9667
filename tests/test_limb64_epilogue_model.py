"""Exact model (Python integers, no GPU) of the 64-bit limb contraction's
integer epilogue (linac_gb300/csrc/tc64_kernels.cuh, constants from
trailing_tc64.cu): the fifteen digit-group sums y_g enter as the bit patterns
b_g = y_g + 0x4B400000 of their magic-number conversion; with the weights
w_g = 2^(8g) 2^64 mod p (centred) split as w_g = wh_g 2^32 + wl_g, the sums of
b_g wl_g and b_g wh_g are formed modulo 2^64 from the start values
-0x4B400000 sum wl and -0x4B400000 sum wh, read as signed 64-bit values,
combined with the offset in 128 bits and reduced by one Montgomery step.  The
model checks, at the extreme group values the digit bounds allow, that every
intermediate is exact and that the result is old + sum_g y_g 256^g mod p."""
import random

import pytest

MAGIC_I = 0x4B400000
M32 = (1 << 32) - 1
M64 = (1 << 64) - 1
M128 = (1 << 128) - 1


def s64(x):
    x &= M64
    return x - (1 << 64) if x >> 63 else x


def constants(p):
    w, x = [], (1 << 64) % p
    for _ in range(15):
        w.append(x - p if x > p // 2 else x)
        x = (x * 256) % p
    off = (((1 << 91) + p - 1) // p) * p
    pinv = (-pow(p, -1, 1 << 64)) % (1 << 64)
    return w, off, pinv


def redc(lo, hi, p, pinv):
    """FieldU64::redc: (hi 2^64 + lo) 2^-64 mod p for hi 2^64 + lo < p 2^64."""
    m = (lo * pinv) & M64
    t = hi + ((m * p) >> 64) + (1 if lo else 0)
    assert t < 2 * p
    return t - p if t >= p else t


def epilogue(y, p, old):
    w, off, pinv = constants(p)
    wl = [x & M32 for x in w]            # unsigned low words
    wh = [x >> 32 for x in w]             # signed high words (w = wh 2^32 + wl)
    assert all(h * (1 << 32) + l == x for x, h, l in zip(w, wh, wl))
    a0 = (-MAGIC_I * sum(wl)) & M64
    a1 = (-MAGIC_I * sum(wh)) & M64
    for yg, l, h in zip(y, wl, wh):
        b = (yg + MAGIC_I) & M32
        assert 0 < b < (1 << 31)
        a0 = (a0 + b * l) & M64
        a1 = (a1 + b * h) & M64
    assert s64(a0) == sum(yg * l for yg, l in zip(y, wl))
    assert s64(a1) == sum(yg * h for yg, h in zip(y, wh))
    T = (off + s64(a0) + (s64(a1) << 32)) & M128
    assert T == off + sum(yg * x for yg, x in zip(y, w)) and 0 <= T < (p << 64)
    v = redc(T & M64, T >> 64, p, pinv)
    return (old + v) % p


# |y_g| <= n_g 2^14 K with n_g = min(g + 1, 15 - g) digit pairs and K = 64; the fast conversion
# needs |y_g| <= 2^22 (groups 0-3 and 11-14 always meet it, groups 4-10 are checked)
BOUND = [min(g + 1, 15 - g) * (1 << 20) for g in range(15)]
FAST = [min(b, 1 << 22) for b in BOUND]
PRIMES = [2**32 + 15, 2**40 + 15, 2**61 - 1, 2**63 + 29, 2**64 - 59]


@pytest.mark.parametrize("p", PRIMES)
def test_epilogue64_exact_at_the_bounds(p):
    rng = random.Random(p)
    cases = []
    for bounds in (FAST, BOUND):
        cases += [[s * b for b in bounds] for s in (1, -1)]
        cases += [[(1 if (g + k) % 2 else -1) * b for g, b in enumerate(bounds)] for k in range(2)]
        cases += [[rng.randint(-b, b) for b in bounds] for _ in range(200)]
    for y in cases:
        for old in (0, p - 1, rng.randrange(p)):
            want = (old + sum(yg * 256**g for g, yg in enumerate(y))) % p
            assert epilogue(y, p, old) == want
