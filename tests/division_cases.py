"""Divisors and hard dividends for the tests of the device's division by a constant
(csrc/cnv_sor.cuh, div_rn_const): shared by tests/test_exact_arith.py (GPU) and
tests/test_division_cases.py (CPU checks of these inputs themselves)."""
from __future__ import annotations

import math

import numpy as np


def den_of(n, L=1.0):
    dx = L / n
    return 2 * (dx * dx + dx * dx)


DIVISORS = [den_of(768), den_of(1536), den_of(100), den_of(37), den_of(7), den_of(3000), 3.0, -7.0, 0.1,
            1.0 / 3.0, 1 + 2.0 ** -52, 2 - 2.0 ** -52, -(2 - 2.0 ** -52), 0.75, 2.0 ** -30,
            2.0 ** -100 * 1.5, 2.0 ** 100 * 1.999, 2.0 ** 101 * 1.25, 2.0 ** -101 * 1.75, 1e-300, 1e300]


def _significand(b):
    m, e = math.frexp(abs(b))  # abs(b) = m * 2^e, 0.5 <= m < 1
    B = int(m * 2 ** 53)
    return B, e - 53


def near_ties(b, count, seed):
    """Dividends a with a / b within about t * 2^-104 (relative; t odd, |t| <= 15) of a tie between
    two doubles for a divisor with a 53-bit significand: with
    b = B * 2^eb (B odd), pick an odd 54-bit M with B*M = t (mod 2^k) for a small odd t, so that
    A = (B*M - t) / 2^k is a 53-bit integer and a = A * 2^E gives a / b = (M - t/B) * 2^x, where
    M * 2^x is the midpoint between two consecutive doubles."""
    rng = np.random.default_rng(seed)
    B, eb = _significand(b)
    while B % 2 == 0:
        B //= 2
        eb += 1
    nb = B.bit_length()
    out = []
    while len(out) < count:
        t = int(rng.integers(-7, 8)) * 2 + 1
        k = nb + int(rng.integers(0, 2))
        M0 = (t * pow(B, -1, 1 << k)) % (1 << k)
        lo = -(-((1 << 53) - M0) // (1 << k))
        hi = ((1 << 54) - 1 - M0) // (1 << k)
        if lo > hi:
            continue
        M = M0 + int(rng.integers(lo, hi + 1)) * (1 << k)
        P = B * M - t
        A = P >> k
        if P % (1 << k) or not (1 << 52) <= A < (1 << 53):
            continue
        a = math.ldexp(A, int(rng.integers(-60, 60)))
        out.append(-a if rng.integers(0, 2) else a)
    return np.array(out)
