"""Primality and field-constant helpers for the host side.

linac's GPU path computes inverses by Fermat's little theorem
(linac/row_reduce.cu:92-101), which silently gives garbage for a non-prime
modulus; its CPU path raises ZeroDivisionError only when it meets a
non-invertible pivot (linac/row_reduce.py:63-64).  This build validates the
modulus on the host once per call with a deterministic Miller-Rabin test and
raises ``ZeroDivisionError`` with the reference's wording for a non-prime.
"""
from __future__ import annotations

_MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)


def is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3.3e24 (covers every 64-bit n)."""
    n = int(n)
    if n < 2:
        return False
    for q in _MR_BASES:
        if n % q == 0:
            return n == q
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in _MR_BASES:
        x = pow(a, d, n)
        if x == 1 or x == n - 1:
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def largest_primes_below(bound: int, count: int) -> list[int]:
    """The `count` largest primes strictly below `bound`, in decreasing order."""
    out = []
    n = int(bound) - 1
    while len(out) < count and n >= 2:
        if is_prime(n):
            out.append(n)
        n -= 1
    return out


def check_prime(p: int) -> None:
    if not is_prime(p):
        raise ZeroDivisionError(
            f"Inverse mod {p} does not exist in general. Are you sure {p} is prime?")
