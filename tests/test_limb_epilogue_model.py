"""Exact model (Python integers, no GPU) of the 32-bit limb contraction's
integer epilogue (linac_gb300/csrc/tc_kernels.cuh: limb_constants and the
fast and slow paths of limb_cta): the seven digit-group sums y_g are
converted through their FP32 bit patterns, groups (0, 1), (2, 3) and (5, 6)
are paired by a shift-add, the weighted sum is formed modulo 2^64 and reduced
by one Montgomery step (odd p < 2^31) or Barrett (otherwise), and the result
is added to the old value of C.  The model checks,
at the extreme group values the digit bounds allow, that the true sum stays
in the reduction's range and that the result is sum_g y_g 256^g mod p."""
import random

import pytest

MAGIC_I = 0x4B400000   # bit pattern of 1.5 * 2^23
KPAIR = 0x0B400000     # (257 * MAGIC_I + 2^31) mod 2^32
M64 = (1 << 64) - 1
M32 = (1 << 32) - 1


def limb_constants(p):
    redc = (p & 1) == 1 and p < (1 << 31)
    w0 = (1 << 32) % p if redc else 1 % p
    w = []
    for _ in range(7):
        w.append(w0 - p if w0 > p // 2 else w0)
        w0 = (w0 * 256) % p
    off = (3 * p) << 29 if redc else (((1 << 62) + p - 1) // p) * p
    pinv = (-pow(p, -1, 1 << 32)) % (1 << 32) if p & 1 else 0
    return redc, w, off, pinv


def s32(x):
    x &= M32
    return x - (1 << 32) if x >> 31 else x


def reduce(v, p, redc, pinv):
    if redc:
        m = (v * pinv) & M32
        t = m * p + v
        assert t < (1 << 64) and t & M32 == 0
        u = t >> 32
        assert u < 2 * p
        return min(u, (u - p) & M32)
    return v % p


def add_residue(old, r, p, redc):
    if redc:
        s = old + r
        assert s < (1 << 32)
        return min(s, (s - p) & M32)
    return (old + r) % p


def fast_path(y, p, old):
    redc, w, off, pinv = limb_constants(p)
    b = [(MAGIC_I + yg) & M32 for yg in y]          # bits of fadd(D_g, 1.5 2^23)
    b0n, b2n, b5n = (b[g] | 0x80000000 for g in (0, 2, 5))  # bits of fadd(-D_g, -1.5 2^23)
    z01 = s32((b[1] << 8) + b0n)
    z23 = s32((b[3] << 8) + b2n)
    z56 = s32((b[6] << 8) + b5n)
    assert z01 == y[0] + 256 * y[1] + KPAIR and z23 == y[2] + 256 * y[3] + KPAIR
    assert z56 == y[5] + 256 * y[6] + KPAIR
    bias3 = (off - KPAIR * (w[0] + w[2] + w[5]) - MAGIC_I * w[4]) & M64
    v = (bias3 + z01 * w[0] + z23 * w[2] + s32(b[4]) * w[4] + z56 * w[5]) & M64
    true_v = (off + (y[0] + 256 * y[1]) * w[0] + (y[2] + 256 * y[3]) * w[2] + y[4] * w[4]
              + (y[5] + 256 * y[6]) * w[5])
    assert 0 <= true_v < ((p << 32) if redc else (1 << 64)) and v == true_v
    return add_residue(old, reduce(v, p, redc, pinv), p, redc)


def slow_path(y, p, old):
    redc, w, off, pinv = limb_constants(p)
    true_v = off + sum(yg * wg for yg, wg in zip(y, w))
    assert 0 <= true_v < ((p << 32) if redc else (1 << 64))
    return add_residue(old, reduce(true_v & M64, p, redc, pinv), p, redc)


# |y_g| bounds: groups 0 and 6 hold one digit product per K step (<= 2^14 * 128), groups 1 and 5 two;
# the fast path also requires |y_2|, |y_3|, |y_4| <= 2^22 (group 4 always meets it for p < 2^31,
# whose top digit is at most 64 in magnitude), the slow path allows 2^23
FAST = [1 << 21, 1 << 22, 1 << 22, 1 << 22, 1 << 22, 1 << 22, 1 << 21]
SLOW = [1 << 21, 1 << 22, 1 << 23, 1 << 23, 1 << 23, 1 << 22, 1 << 21]
PRIMES = [3, 65521, 2**30 + 3, 2147483629, 2**31 - 1, 2**31 + 11, 4294967291, 2]


@pytest.mark.parametrize("p", PRIMES)
def test_epilogue_exact_at_the_bounds(p):
    rng = random.Random(p)
    cases = [[s * b for b in FAST] for s in (1, -1)]
    cases += [[(1 if (g + k) % 2 else -1) * b for g, b in enumerate(FAST)] for k in range(2)]
    cases += [[rng.randint(-b, b) for b in FAST] for _ in range(300)]
    for y in cases:
        for old in (0, p - 1, rng.randrange(p)):
            want = (old + sum(yg * 256**g for g, yg in enumerate(y))) % p
            assert fast_path(y, p, old) == want
    for y in [[s * b for b in SLOW] for s in (1, -1)] + [[rng.randint(-b, b) for b in SLOW] for _ in range(300)]:
        for old in (0, p - 1):
            want = (old + sum(yg * 256**g for g, yg in enumerate(y))) % p
            assert slow_path(y, p, old) == want
