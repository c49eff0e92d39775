"""The inputs of the division tests, checked on the CPU with exact rational arithmetic: the
constructed dividends put a / b within 2^-98 (relative) of a tie between two doubles, which
is as close as a quotient of two doubles can come for a divisor with a long significand, and
numpy's quotients, the GPU test's reference, are the correctly rounded ones on this host."""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np
import pytest

from division_cases import DIVISORS, near_ties


def rel_distance_to_tie(a: float, b: float) -> float:
    q = Fraction(a) / Fraction(b)
    r = float(q)  # Fraction -> float rounds to nearest, ties to even
    half = Fraction(math.ulp(r)) / 2
    return float(min(abs(q - (Fraction(r) - half)), abs(q - (Fraction(r) + half))) / abs(q))


def correctly_rounded(a: float, b: float) -> float:
    return float(Fraction(a) / Fraction(b))


def long_significand(b: float) -> bool:
    m, _ = math.frexp(abs(b))
    B = int(m * 2 ** 53)
    while B % 2 == 0:
        B //= 2
    return B.bit_length() > 40


@pytest.mark.parametrize("b", [b for b in DIVISORS if 1e-250 < abs(b) < 1e250])
def test_near_ties_are_near_ties(b):
    a = near_ties(b, 60, 1)
    assert a.shape == (60,) and np.all(np.isfinite(a))
    d = max(rel_distance_to_tie(float(x), b) for x in a)
    if long_significand(b):
        assert d < 2.0 ** -98, d
    else:
        # a short odd significand B keeps every quotient at least about 1/B ulp from a tie
        assert d < 2.0 ** -40, d


@pytest.mark.parametrize("b", [b for b in DIVISORS if 1e-250 < abs(b) < 1e250])
def test_numpy_quotients_are_correctly_rounded(b):
    rng = np.random.default_rng(5)
    x = np.concatenate([near_ties(b, 40, 2), rng.standard_normal(200) * np.exp2(rng.integers(-60, 60, 200))])
    got = x / b
    want = np.array([correctly_rounded(float(v), b) for v in x])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
