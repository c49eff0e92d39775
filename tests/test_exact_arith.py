"""The exact Poisson update's integer multiply (csrc/cnv_sor.cuh, mul_rn) and its division by a
constant (div_rn_const) against IEEE 754.

On GB300 the FP64 pipe bounds the exact SOR update, so its two multiplications by constants
(beta/4 * t and (1 - beta) * old) run as integer arithmetic on the 53-bit significands, falling
back to the FP64 pipe for subnormal, infinite and NaN operands and for products outside the
normal range. Every result must equal the correctly rounded product, which numpy
computes on the host (IEEE binary64, round to nearest, ties to even). The operands cover the whole
exponent range, products that are exact halfway cases (c = 1.5 or 0.75 with odd significands),
the edges of the normal range and the special values.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from division_cases import DIVISORS, den_of, near_ties

pytestmark = pytest.mark.gpu


def beta_ref(n):
    """SOR factor of the reference (src/main.c:134) for an n x n grid."""
    return 0.5 * (2 / (1 + math.sin(math.pi / (n + 1))) + 2 / (1 + math.sin(math.pi / (n + 1))))


CONSTANTS = [beta_ref(1024) / 4, 1 - beta_ref(1024), beta_ref(64) / 4, 1 - beta_ref(64), beta_ref(2048) / 4,
             1 - beta_ref(2048), 1.5, 0.75, -1.5, 1 + 2.0 ** -52, 2 - 2.0 ** -52, 3.0, 0.1, 2.0 ** -1022,
             np.finfo(np.float64).max, 0.375]


def operands(rng, count):
    """Random finite doubles over the whole exponent range, both signs, plus the special values
    and the edges of the normal range."""
    mant = rng.integers(0, 1 << 52, size=count, dtype=np.uint64)
    expo = rng.integers(1, 2047, size=count, dtype=np.uint64)  # every normal exponent
    sign = rng.integers(0, 2, size=count, dtype=np.uint64) << np.uint64(63)
    x = (sign | (expo << np.uint64(52)) | mant).view(np.float64)
    fi = np.finfo(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, fi.max, -fi.max, fi.tiny, -fi.tiny,
                        fi.tiny * 2 ** -10, -fi.tiny * 2 ** -30, 5e-324, 1.0, -1.0, 2.0 ** -28, 2.0 ** 46])
    return np.concatenate([x, special])


def same_bits(a, b):
    nan = np.isnan(a) & np.isnan(b)
    return (a.view(np.uint64) == b.view(np.uint64)) | nan


@pytest.mark.parametrize("c", CONSTANTS)
def test_integer_multiply_is_correctly_rounded(cnv, c):
    rng = np.random.default_rng(abs(hash(c)) % (1 << 32))
    x = operands(rng, 1 << 20)
    got = cnv.check_mul_rn(x, c)
    with np.errstate(all="ignore"):
        want = x * c
    bad = ~same_bits(got, want)
    assert not bad.any(), f"c={c!r}: {bad.sum()} mismatches, first x={x[bad][0]!r}: {got[bad][0]!r} vs {want[bad][0]!r}"


def test_halfway_products_round_to_even(cnv):
    """c = 1.5 and 0.75 make every odd significand an exact tie; near the top of the range and at
    the bottom the product leaves the normal range (hardware path), in between it must round
    half to even on the integer path."""
    rng = np.random.default_rng(7)
    mant = rng.integers(0, 1 << 52, size=1 << 18, dtype=np.uint64) | np.uint64(1)  # odd significands
    for expo in (1, 2, 100, 1023, 1500, 2045, 2046):
        x = ((np.uint64(expo) << np.uint64(52)) | mant).view(np.float64)
        for c in (1.5, 0.75, -1.5, 3.0):
            got = cnv.check_mul_rn(x, c)
            with np.errstate(all="ignore"):
                want = x * c
            assert same_bits(got, want).all(), (expo, c)


# ---------------------------------------------------------------------------------------------
# Division by a constant (csrc/cnv_sor.cuh, div_rn_const): the exact update's x / den and the
# transport pass's (c4 f) / den on grids where den = 2 (dx^2 + dy^2) is not a power of two (every
# n that is not a power of two, dx = L / n as src/main.c:138 sets it). The quotient comes from a
# two-term reciprocal and an exact residual test, with the IEEE division where the test cannot
# prove it; every result must equal numpy's correctly rounded quotient.

@pytest.mark.parametrize("b", DIVISORS)
def test_division_by_constant_is_correctly_rounded(cnv, b):
    rng = np.random.default_rng(abs(hash(b)) % (1 << 32))
    x = np.concatenate([operands(rng, 1 << 20), near_ties(b, 4000, 1)])
    got, fast = cnv.check_div_rn(x, b)
    with np.errstate(all="ignore"):
        want = x / b
    bad = ~same_bits(got, want)
    assert not bad.any(), f"b={b!r}: {bad.sum()} mismatches, first x={x[bad][0]!r}: {got[bad][0]!r} vs {want[bad][0]!r}"
    assert 0 <= fast <= x.size


@pytest.mark.parametrize("n", [768, 1536, 100, 37])
def test_division_by_den_takes_the_short_path(cnv, n):
    """On dividends of the solver's range (|x| between 2^-60 and 2^20) the three-operation path
    proves nearly every quotient; only the constructed near-ties may need the IEEE division."""
    b = den_of(n)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(1 << 20) * np.exp2(rng.integers(-60, 20, size=1 << 20))
    got, fast = cnv.check_div_rn(x, b)
    assert same_bits(got, x / b).all()
    assert fast >= 0.999 * x.size, fast / x.size
    ties = near_ties(b, 2000, n)
    got, _ = cnv.check_div_rn(ties, b)
    assert same_bits(got, ties / b).all()
