"""The integer algorithms of the exact Poisson update (csrc/cnv_sor.cuh, csrc/cnv_poisson.cu),
restated in Python and checked on the CPU against exact integer and rational arithmetic. The GPU
tests (tests/test_exact_arith.py, tests/test_gpu_parity.py) check the CUDA code bit for bit; these
check that the algorithms the CUDA code implements are right, on inputs chosen to reach every
branch: the multiply's rounding step and normalisation (mul_rn_core), the stop norm's split of
|dpsi| into 32-bit chunk counters (norm_add), the row-aligned interior chunks (interior_chunks)
and the acceptance test of the division by a constant (div_rn_const_fast)."""
from __future__ import annotations

import math
import random
import struct
from fractions import Fraction

import pytest

M32 = (1 << 32) - 1
M64 = (1 << 64) - 1


def funnelshift_l(lo: int, hi: int, shift: int) -> int:
    """CUDA __funnelshift_l: the upper 32 bits of (hi:lo) << (shift & 31)."""
    return ((((hi << 32) | lo) << (shift & 31)) >> 32) & M32


def funnelshift_r(lo: int, hi: int, shift: int) -> int:
    """CUDA __funnelshift_r: the lower 32 bits of (hi:lo) >> (shift & 31)."""
    return (((hi << 32) | lo) >> (shift & 31)) & M32


# ---------------------------------------------------------------------------------------------
# mul_rn_core: significands mx, mc in [2^52, 2^53); the product rounded to 53 bits, half to even,
# by adding 2^(sh-1) - 1 plus the lowest kept bit and truncating; the shift by sh = 52 or 53 taken
# as two funnel shifts of the upper words by k = sh - 32.

def mul_core_model(mx: int, mc: int) -> tuple[int, int]:
    """(significand, bits dropped) as the device computes them."""
    p = mx * mc
    lo, hi = p & M64, p >> 64
    top = (hi >> 41) != 0
    k = 21 if top else 20
    keep = ((lo >> 32) >> k) & 1
    lo2 = lo + (((1 << 52) - 1) if top else ((1 << 51) - 1)) + keep
    hi2 = hi + (lo2 >> 64)
    lo2 &= M64
    h0, h1 = hi2 & M32, hi2 >> 32
    mant = (funnelshift_r(h0, h1, k) << 32) | funnelshift_r(lo2 >> 32, h0, k)
    sh = 32 + k
    if mant >> 53:
        mant >>= 1
        sh += 1
    return mant, sh


def mul_core_exact(mx: int, mc: int) -> tuple[int, int]:
    p = mx * mc
    sh = p.bit_length() - 53
    q, r = divmod(p, 1 << sh)
    half = 1 << (sh - 1)
    if r > half or (r == half and q & 1):
        q += 1
    if q >> 53:
        q >>= 1
        sh += 1
    return q, sh


def _significands(rng, count):
    out = [rng.randrange(1 << 52, 1 << 53) for _ in range(count)]
    out += [1 << 52, (1 << 53) - 1, 3 << 51, (1 << 52) + 1, (1 << 53) - 3]
    return out


def test_multiply_rounding_and_normalisation():
    rng = random.Random(1)
    xs, cs = _significands(rng, 3000), _significands(rng, 40)
    for mx in xs:
        for mc in cs:
            assert mul_core_model(mx, mc) == mul_core_exact(mx, mc), (mx, mc)


def test_multiply_exact_ties_round_to_even():
    """c = 1.5 makes every odd significand an exact tie (the dropped bits are exactly half)."""
    rng = random.Random(2)
    for _ in range(20000):
        mx = rng.randrange(1 << 52, 1 << 53) | 1
        for mc in (3 << 51, (1 << 52) | (1 << 51)):
            assert mul_core_model(mx, mc) == mul_core_exact(mx, mc), (mx, mc)


# ---------------------------------------------------------------------------------------------
# norm_add's common case: d = |a - b| < 2^52 of two values with the same sign and exponent, shifted
# by s = e - 995 (0..73) into four 32-bit chunks held by 64-bit counters.

def chunks_model(d: int, s: int) -> list[int]:
    d0, d1 = d & M32, d >> 32
    w, r = s >> 5, s & 31
    x0 = (d0 << r) & M32
    x1 = funnelshift_l(d0, d1, r)
    x2 = funnelshift_l(d1, 0, r)
    return [x0 if w == 0 else 0,
            x1 if w == 0 else (x0 if w == 1 else 0),
            x2 if w == 0 else (x1 if w == 1 else x0),
            x2 if w == 1 else (x1 if w == 2 else 0)]


def test_stop_norm_chunks_hold_the_shifted_difference():
    rng = random.Random(3)
    for s in range(74):
        for d in [rng.randrange(0, 1 << 52) for _ in range(300)] + [0, 1, (1 << 52) - 1, M32, 1 << 32]:
            c = chunks_model(d, s)
            assert all(0 <= x <= M32 for x in c)
            assert sum(x << (32 * k) for k, x in enumerate(c)) == d << s, (d, s)


# ---------------------------------------------------------------------------------------------
# interior_chunks, folded form: row-aligned chunks of 64 cells give the cells of the flat mapping.

def cells_flat(ri0, ri1, ci0, ci1, colour):
    w, h = ci1 - ci0, ri1 - ri0
    wq = (w + 1) >> 1
    out = []
    for x in range(h * wq):
        r, t = divmod(x, wq)
        i = ri0 + r
        j = ci0 + 2 * t + ((i + ci0 + colour) & 1)
        if j < ci1:
            out.append((i, j))
    return out


def cells_rows(ri0, ri1, ci0, ci1, colour):
    w, h = ci1 - ci0, ri1 - ri0
    wq = (w + 1) >> 1
    per_row = (wq + 63) >> 6
    out = []
    for c in range(h * per_row):
        r, b = divmod(c, per_row)
        i = ri0 + r
        j0 = ci0 + ((i + ci0 + colour) & 1)
        for u in range(2):
            for lane in range(32):
                tt = b * 64 + u * 32 + lane
                if tt < wq and j0 + 2 * tt < ci1:
                    out.append((i, j0 + 2 * tt))
    return out


@pytest.mark.parametrize("seed", range(4))
def test_row_aligned_chunks_cover_the_same_cells(seed):
    rng = random.Random(seed)
    for _ in range(60):
        ri0, ci0 = rng.randint(1, 30), rng.randint(1, 30)
        h, w = rng.randint(1, 12), rng.randint(96, 300)  # the path is taken from 48 cells of a colour
        for colour in (0, 1):
            a = cells_flat(ri0, ri0 + h, ci0, ci0 + w, colour)
            b = cells_rows(ri0, ri0 + h, ci0, ci0 + w, colour)
            assert sorted(a) == sorted(b) and len(set(b)) == len(b)
            assert all((i + j) % 2 == colour for i, j in b)


# ---------------------------------------------------------------------------------------------
# div_rn_const_fast's acceptance test: q is kept only when |a - b q| < |b| ulp(q) / 2 and q is not a
# power of two; then q is the correctly rounded quotient.

def bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def accepted(a: float, b: float, q: float) -> bool:
    """The device's test, with the residual formed exactly (as one FMA gives it when it is a double)
    and rounded to a double otherwise."""
    r = Fraction(a) - Fraction(b) * Fraction(q)
    rb = bits(abs(float(r)))
    eq = (bits(q) >> 52) & 0x7FF
    hb = (bits(abs(b)) + ((eq - 1076) << 52)) & M64
    return (bits(q) & ((1 << 52) - 1)) != 0 and rb < hb


def test_division_acceptance_implies_correct_rounding():
    """Candidates near the quotient, including wrong ones: every accepted candidate is the
    correctly rounded quotient, and the correctly rounded one is accepted unless it is a power of
    two."""
    rng = random.Random(4)
    divisors = [2 * (2 * (1 / n) ** 2) for n in (37, 100, 768, 1536)] + [3.0, 0.1, 1 / 3, 1.75]
    for b in divisors:
        for _ in range(400):
            a = rng.uniform(0.5, 2.0) * 2.0 ** rng.randint(-60, 60) * rng.choice((1, -1))
            exact = Fraction(a) / Fraction(b)
            correct = float(exact)
            for steps in (-2, -1, 0, 1, 2):
                q = correct
                for _ in range(abs(steps)):
                    q = math.nextafter(q, math.inf if steps > 0 else -math.inf)
                if accepted(a, b, q):
                    assert q == correct, (a, b, q, correct)
            if bits(correct) & ((1 << 52) - 1):
                assert accepted(a, b, correct), (a, b)
