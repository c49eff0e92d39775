// cnv_sor.cuh -- device pieces shared by the persistent SOR kernels (cnv_poisson.cu,
// cnv_poisson_tb.cu): the exact fixed-point stop norm, the exact multiply by a constant, and
// the point update of src/poisson.c:247 in its three arithmetic forms. Both kernels
// use these same functions so that they produce the same bits.
#pragma once

#include "cnv_kernels.h"
#include "cnv_sync.cuh"

namespace cnv {
namespace {

// (x2:hi:lo) * 2^-80 rounded to the nearest double, ties to even, where x2 holds bits 128..191:
// the stop norm's fixed-point total converted with one correct rounding (such values are normal).
__host__ __device__ __forceinline__ double fixed80_to_double(unsigned long long lo, unsigned long long hi,
                                                             unsigned long long x2) {
    bool sticky = false;  // non-zero bits below lo after a renormalisation
    int scale = -80;
    if (x2) {
        sticky = lo != 0;
        lo = hi;
        hi = x2;
        scale += 64;
    }
    if ((lo | hi) == 0) return 0.0;
#ifdef __CUDA_ARCH__
    const int top = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);  // leading bit
#else
    const int top = hi ? 127 - __builtin_clzll(hi) : 63 - __builtin_clzll(lo);
#endif
    const int drop = top - 52;  // bits below the 53-bit significand
    unsigned long long m;
    bool up = false;
    if (drop <= 0) {
        m = lo << (-drop);  // top <= 52: hi == 0, exact (no sticky bits: x2 was 0)
    } else {
        unsigned long long rh, rl;  // the dropped bits
        if (drop >= 64) {
            const int d = drop - 64;
            m = hi >> d;
            rh = d ? hi & ((1ull << d) - 1) : 0;
            rl = lo;
        } else {
            m = (lo >> drop) | (hi << (64 - drop));
            rh = 0;
            rl = lo & ((1ull << drop) - 1);
        }
        const unsigned long long hh = drop - 1 >= 64 ? 1ull << (drop - 65) : 0;  // half an ulp
        const unsigned long long hl = drop - 1 >= 64 ? 0 : 1ull << (drop - 1);
        const bool eq = rh == hh && rl == hl;
        const bool gt = rh > hh || (rh == hh && rl > hl) || (eq && sticky);
        up = gt || (eq && !sticky && (m & 1));
    }
    m += up ? 1 : 0;
    int e = top;
    if (m >> 53) {  // rounded up to the next power of two
        m >>= 1;
        ++e;
    }
    const unsigned long long bits = ((unsigned long long)(e + scale + 1023) << 52) | (m & ((1ull << 52) - 1));
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)bits);
#else
    double out;
    __builtin_memcpy(&out, &bits, sizeof out);
    return out;
#endif
}

// The stop norm from its four 32-bit chunk counters (chunk w holds bits 32w.. of the total in
// units of 2^-80, each counter up to 2^64): carry-propagate into a 160-bit integer and convert.
__host__ __device__ __forceinline__ double norm_total(const unsigned long long c[4]) {
    unsigned long long t = c[0];
    unsigned long long lo = t & 0xffffffffull;
    t = c[1] + (t >> 32);
    lo |= (t & 0xffffffffull) << 32;
    t = c[2] + (t >> 32);
    unsigned long long hi = t & 0xffffffffull;
    t = c[3] + (t >> 32);
    hi |= (t & 0xffffffffull) << 32;
    return fixed80_to_double(lo, hi, t >> 32);
}

// Stop-norm accumulator of one thread. |psi_new - psi_old| is summed exactly as integers in
// units of 2^-80, in four 32-bit chunks held by 64-bit counters (no carries while accumulating),
// for every cell whose two values lie below 2^46 in magnitude. Each value is truncated to a
// multiple of 2^-80 first: values of 2^-28 or more are multiples already, so a cell is off by
// less than 2^-80 only when one of its values lies below 2^-28, and the total is off by less than
// (number of cells) * 2^-80 (about 1e-18 at 1024^2). Cells with a value of 2^46 or more (or a
// non-finite one) are left to the caller, which adds them to an FP64 side sum in shared memory
// (norm_side_add): they are far outside any realistic streamfunction, and the reference sums them
// in FP64 too. The side sum lives outside the accumulator so that the sweep loops carry only the
// four integer chunks.
struct NormAcc {
    unsigned long long c[4];
};

// |nw - old| into an FP64 side sum (a block's shared accumulator): the rare cells norm_add leaves.
// Inlined: a call to an out-of-line function, even one never taken, made the sweep loops keep
// registers free around it (0.8 % of the 1024^2 sweep rate).
__device__ __forceinline__ void norm_side_add(double* side, double nw, double old) {
    atomicAdd(side, fabs(__dsub_rn(nw, old)));
}

// |x| * 2^80, truncated, as a 128-bit integer (hi:lo), for |x| < 2^46; values below 2^-80 give 0.
__device__ __forceinline__ void abs_fixed80(double x, unsigned long long& lo, unsigned long long& hi) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    const int ex = (int)(b >> 52);
    const unsigned long long mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int s = ex - 995;  // |x| * 2^80 = mant * 2^s, s < 74
    lo = 0;
    hi = 0;
    if (ex == 0) return;     // zero or below 2^-1022
    if (s >= 64) {
        hi = mant << (s - 64);
    } else if (s > 0) {
        lo = mant << s;
        hi = mant >> (64 - s);
    } else if (s > -53) {
        lo = mant >> (-s);
    }
}

// acc += |nw - old| exactly in fixed point (both truncated at 2^-80) on the integer pipes. Returns
// false, adding nothing, when a value reaches 2^46 or is not finite (the caller's FP64 side sum).
__device__ __forceinline__ bool norm_add(NormAcc& acc, double nw, double old) {
    {
        // the common case, same sign and exponent e with 2^-28 <= |x| < 2^46: both images are
        // exact (no truncation), and their difference is the significands' difference (the
        // difference of the bit patterns) times 2^(e - 995)
        const unsigned long long a = (unsigned long long)__double_as_longlong(nw);
        const unsigned long long b = (unsigned long long)__double_as_longlong(old);
        const int e = (int)((a >> 52) & 0x7ff);
        if (((a ^ b) >> 52) == 0 && e >= 995 && e < 1069) {
            const long long sd = (long long)(a - b);
            const unsigned long long d = (unsigned long long)(sd < 0 ? -sd : sd);  // < 2^52
            const int s = e - 995;                                                   // 0 .. 73
            // d << s in 32-bit words: d << (s & 31) is three words x0..x2 (funnel shifts), which
            // land in chunks w, w+1, w+2 for w = s >> 5 (for w = 2, x2 is 0: d << 9 < 2^61)
            const unsigned d0 = (unsigned)d, d1 = (unsigned)(d >> 32);
            const int w = s >> 5, r = s & 31;
            const unsigned x0 = d0 << r;
            const unsigned x1 = __funnelshift_l(d0, d1, r);
            const unsigned x2 = __funnelshift_l(d1, 0u, r);
            acc.c[0] += w == 0 ? x0 : 0u;
            acc.c[1] += w == 0 ? x1 : (w == 1 ? x0 : 0u);
            acc.c[2] += w == 0 ? x2 : (w == 1 ? x1 : x0);
            acc.c[3] += w == 1 ? x2 : (w == 2 ? x1 : 0u);
            return true;
        }
    }
    if (((unsigned long long)__double_as_longlong(nw) & 0x7fffffffffffffffull) >= (1069ull << 52) ||
        ((unsigned long long)__double_as_longlong(old) & 0x7fffffffffffffffull) >= (1069ull << 52))
        return false;  // a value of 2^46 or more, Inf or NaN: the FP64 side sum
    unsigned long long al, ah, bl, bh;
    abs_fixed80(nw, al, ah);
    abs_fixed80(old, bl, bh);
    unsigned long long dl, dh;
    if ((__double_as_longlong(nw) ^ __double_as_longlong(old)) < 0) {  // opposite signs: |a| + |b|
        dl = al + bl;
        dh = ah + bh + (dl < al);
    } else {  // same sign: ||a| - |b||
        const bool a_ge = ah > bh || (ah == bh && al >= bl);
        if (a_ge) {
            dl = al - bl;
            dh = ah - bh - (al < bl);
        } else {
            dl = bl - al;
            dh = bh - ah - (bl < al);
        }
    }
    acc.c[0] += dl & 0xffffffffull;
    acc.c[1] += dl >> 32;
    acc.c[2] += dh & 0xffffffffull;
    acc.c[3] += dh >> 32;
    return true;
}

__device__ __forceinline__ bool big_or_zero(double x) {
    // |x| >= 2^-960 (biased exponent >= 63) or x == +-0
    const int hi = __double2hiint(x);
    const int lo = __double2loint(x);
    return ((hi & 0x7ff00000) >= (63 << 20)) || (((hi & 0x7fffffff) | lo) == 0);
}

// big_or_zero of all four: one minimum of the exponent fields for the common case (all at least
// 2^-960), the zero cases only when that fails.
__device__ __forceinline__ bool all_big_or_zero(double a, double b, double c, double d) {
    const unsigned ea = (unsigned)__double2hiint(a) & 0x7ff00000u, eb = (unsigned)__double2hiint(b) & 0x7ff00000u;
    const unsigned ec = (unsigned)__double2hiint(c) & 0x7ff00000u, ed = (unsigned)__double2hiint(d) & 0x7ff00000u;
    if (min(min(ea, eb), min(ec, ed)) >= (63u << 20)) return true;
    return big_or_zero(a) && big_or_zero(b) && big_or_zero(c) && big_or_zero(d);
}

// The rounding core of the integer multiply: the product of two 53-bit significands mx, mc (with
// their leading bits) and biased exponents ex, ec, rounded to nearest, ties to even, with the
// given sign bit. Returns false when the result leaves the normal range.
__device__ __forceinline__ bool mul_rn_core(unsigned long long sign, int ex, unsigned long long mx, int ec,
                                            unsigned long long mc, double& out) {
    const unsigned long long lo = mx * mc;
    const unsigned long long hi = __umul64hi(mx, mc);  // 2^104 <= hi:lo < 2^106
    const bool top = (hi >> 41) != 0;                    // the product is >= 2^105
    int e = ex + ec - 1023 + (top ? 1 : 0);              // biased exponent before rounding
    if (e <= 0) return false;
    // round to nearest, ties to even, dropping sh = 52 or 53 bits: add 2^(sh-1) - 1 plus the
    // lowest kept bit, then truncate (a remainder above half carries, one below does not, and
    // exactly half carries only from an odd significand)
    const int k = top ? 21 : 20;  // sh - 32: the dropped bits reach into lo's upper word
    const unsigned long long keep = ((unsigned)(lo >> 32) >> k) & 1u;
    const unsigned long long lo2 = lo + (top ? (1ull << 52) - 1 : (1ull << 51) - 1) + keep;
    const unsigned long long hi2 = hi + (lo2 < lo ? 1 : 0);
    // (hi2:lo2) >> sh from the upper three words by two funnel shifts
    const unsigned h0 = (unsigned)hi2, h1 = (unsigned)(hi2 >> 32);
    unsigned long long mant = ((unsigned long long)__funnelshift_r(h0, h1, k) << 32) |
                              __funnelshift_r((unsigned)(lo2 >> 32), h0, k);
    if (mant >> 53) {  // rounded up to 2^53
        mant >>= 1;
        ++e;
    }
    if (e >= 0x7ff) return false;
    out = __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | (mant & ((1ull << 52) - 1))));
    return true;
}

// x * c rounded to nearest, ties to even, by integer arithmetic, for a normal constant c (bit
// pattern cb): the 106-bit product of the two 53-bit significands, its top 53 bits, and the
// IEEE 754 round-half-to-even rule on the rest. A zero x gives the signed zero. Returns false
// (the caller multiplies on the FP64 pipe instead) for a subnormal, infinite or NaN x, a c that
// is not normal, and products outside the normal range, so every result equals __dmul_rn(x, c).
// The exact update uses it for its multiplications by constants (two in the folded form, four in
// the general one), which moves them from the FP64 pipe (the solver's bottleneck) to the integer
// pipes.
__device__ __forceinline__ bool mul_rn_int(double x, unsigned long long cb, double& out) {
    const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
    const unsigned long long sign = (xb ^ cb) & 0x8000000000000000ull;
    const int ex = (int)((xb >> 52) & 0x7ff);
    const int ec = (int)((cb >> 52) & 0x7ff);
    if (ec == 0 || ec == 0x7ff) return false;
    if (ex == 0) {
        if ((xb << 1) != 0) return false;  // subnormal
        out = __longlong_as_double((long long)sign);
        return true;
    }
    if (ex == 0x7ff) return false;
    const unsigned long long frac = (1ull << 52) - 1;
    return mul_rn_core(sign, ex, (xb & frac) | (1ull << 52), ec, (cb & frac) | (1ull << 52), out);
}

// c * x as the exact update computes it: on the integer pipes where mul_rn_int applies, on the
// FP64 pipe otherwise (the same bits either way).
__device__ __forceinline__ double mul_rn(double c, double x) {
    double r;
    if (!mul_rn_int(x, (unsigned long long)__double_as_longlong(c), r)) r = __dmul_rn(c, x);
    return r;
}

// The quotient a / d.b from the two-term reciprocal, q = RN(a*zh + RN(a*zl)) (the method of
// Brisebarre, Muller and Raina, "Accelerating correctly rounded floating-point division when the
// divisor is known in advance", IEEE Trans. Computers 53(8), 2004), with an exact test that q is
// a / b rounded to nearest. Returns false (q unproven) outside the tested range, for a q that is
// a power of two, and where the test fails.
// The test. If |q - a/b| < ulp(q), the residual a - b*q is a double (it is a multiple of
// ulp(b)*ulp(q) below |b|*ulp(q) in magnitude), so one FMA gives it exactly; q = RN(a/b) iff
// |a/b - q| < ulp(q)/2, i.e. |r| < |b| * ulp(q)/2, for q not a power of two (whose lower
// neighbour is nearer); equality (a tie) is left to the caller. If |q - a/b| >= ulp(q),
// |a - b*q| >= |b| * ulp(q), which no rounding brings below the bound, so the test fails. With
// 2^-700 <= |a| < 2^701 and 2^-100 <= |b| < 2^101 (d.fast) every value here stays normal.
// q is within ulp(q)/2 + 2^-104 |a/b| of a/b, so the test fails only for quotients that close to
// a tie: the division costs three FP64 operations and a few integer ones.
__device__ __forceinline__ bool div_rn_const_fast(double a, const DivConst& d, double& out) {
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
    const int ea = (int)((ab >> 52) & 0x7ff);
    if (!d.fast || ea < 1023 - 700 || ea > 1023 + 700) return false;
    const double q = __fma_rn(a, d.zh, __dmul_rn(a, d.zl));
    const double r = __fma_rn(-q, d.b, a);  // a - b*q
    const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
    const unsigned long long rb = (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
    const int eq = (int)((qb >> 52) & 0x7ff);
    // |b| * ulp(q) / 2 = |b| * 2^(eq - 1023 - 53): an exponent shift of |b|'s bit pattern
    const unsigned long long hb = d.babs + ((unsigned long long)(long long)(eq - 1076) << 52);
    if ((qb & ((1ull << 52) - 1)) == 0 || rb >= hb) return false;
    out = q;
    return true;
}

// a / d.b rounded to nearest, ties to even: the same bits as __ddiv_rn(a, d.b).
__device__ __forceinline__ double div_rn_const(double a, const DivConst& d) {
    double q;
    if (!div_rn_const_fast(a, d, q)) q = __ddiv_rn(a, d.b);
    return q;
}

// k.c * x as mul_rn_int computes it, for a constant prepared on the host (mul_const): its
// significand, exponent and sign come from the launch parameters. The folded update uses it for
// its two constants (2048^2: 52.3 vs 52.6 us per sweep); in the general update, with four
// constants and the division, it ran slower (1536^2: 77.6 vs 60.9 us) and is not used there.
__device__ __forceinline__ bool mul_rn_int_k(double x, const MulConst& k, double& out) {
    const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((xb >> 52) & 0x7ff);
    if (!k.ok) return false;
    const unsigned long long sign = (xb & 0x8000000000000000ull) ^ k.sign;
    if (ex == 0) {
        if ((xb << 1) != 0) return false;  // subnormal
        out = __longlong_as_double((long long)sign);
        return true;
    }
    if (ex == 0x7ff) return false;
    return mul_rn_core(sign, ex, (xb & ((1ull << 52) - 1)) | (1ull << 52), k.e, k.m, out);
}

__device__ __forceinline__ double mul_rn_k(const MulConst& k, double x) {
    double r;
    if (!mul_rn_int_k(x, k, r)) r = __dmul_rn(k.c, x);
    return r;
}

// The new value of one cell (no norm).
template <Arith A, int KIND, bool FOLD>
__device__ __forceinline__ double point_value(const PoissonParams& p, double up, double dn, double rt,
                                              double lt, double g, double old) {
    double nw;
    if (A == Arith::kExact) {
        if (FOLD) {
            // g holds c4*f/dx^2 (exact power-of-two scaling of the reference's c4*f)
            const double s1 = __dadd_rn(up, dn);
            const double s2 = __dadd_rn(rt, lt);
            const double S = __dadd_rn(s1, s2);
            const double t = __dsub_rn(S, g);
            if (all_big_or_zero(s1, s2, S, t)) {
                if (KIND == CNV_POISSON_SOR)
                    nw = __dadd_rn(mul_rn_k(p.kb4, t), mul_rn_k(p.komb, old));
                else
                    nw = __dmul_rn(0.25, t);
            } else {
                const double gr = __dmul_rn(g, p.dx2);  // back to c4*f exactly
                const double num = __dsub_rn(__dadd_rn(__dmul_rn(p.dy2, s1), __dmul_rn(p.dx2, s2)), gr);
                if (KIND == CNV_POISSON_SOR)
                    nw = __dadd_rn(__dmul_rn(__dmul_rn(p.beta, num), p.rden), __dmul_rn(p.omb, old));
                else
                    nw = __dmul_rn(num, p.rden);
            }
        } else {
            // beta*(dy*dy*(up+dn) + dx*dx*(rt+lt) - dx*dx*dy*dy*f) / (2*(dx*dx+dy*dy)) + (1-beta)*u0,
            // its four multiplications by constants on the integer pipes and the division by den
            // as three FP64 operations (div_rn_const): 8 on the FP64 pipe where the IEEE division
            // alone took more (1536^2: 88.6 -> 60.6 us per sweep, the same bits)
            const double num = __dsub_rn(__dadd_rn(mul_rn(p.dy2, __dadd_rn(up, dn)),
                                                   mul_rn(p.dx2, __dadd_rn(rt, lt))), g);
            if (KIND == CNV_POISSON_SOR) {
                const double bn = mul_rn(p.beta, num);
                const double q = p.den_pow2 ? __dmul_rn(bn, p.rden) : div_rn_const(bn, p.dden);
                nw = __dadd_rn(q, mul_rn(p.omb, old));
            } else {
                nw = p.den_pow2 ? __dmul_rn(num, p.rden) : div_rn_const(num, p.dden);
            }
        }
        return nw;
    } else {
        const double gs = fma(p.wy, up + dn, fma(p.wx, rt + lt, -g));
        nw = KIND == CNV_POISSON_SOR ? fma(p.beta, gs - old, old) : gs;
        return nw;
    }
}

// The new value of one cell, with |new - old| added to the stop norm (to the FP64 side sum *side
// for a value of 2^46 or more).
template <Arith A, int KIND, bool FOLD>
__device__ __forceinline__ double point_update(const PoissonParams& p, double up, double dn, double rt,
                                               double lt, double g, double old, NormAcc& acc, double* side) {
    const double nw = point_value<A, KIND, FOLD>(p, up, dn, rt, lt, g, old);
    if (!norm_add(acc, nw, old)) norm_side_add(side, nw, old);
    return nw;
}

}  // namespace
}  // namespace cnv
