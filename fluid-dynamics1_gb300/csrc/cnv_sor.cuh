// cnv_sor.cuh -- device pieces shared by the persistent SOR kernels (cnv_poisson.cu,
// cnv_poisson_tb.cu): the exact fixed-point stop norm, the exact multiply by a constant, and
// the point update of src/poisson.c:247 in its three arithmetic forms. Both kernels
// use these same functions so that they produce the same bits.
#pragma once

#include "cnv_kernels.h"
#include "cnv_sync.cuh"

namespace cnv {
namespace {

// exact 128-bit fixed-point image (scale 2^80, truncated) of a non-negative double
__device__ __forceinline__ void to_fixed96(double x, unsigned long long& lo, unsigned long long& hi) {
    lo = hi = 0;
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0 || ex == 0x7ff || (b >> 63)) return;  // zero, subnormal (< 2^-1022), inf/nan, negative
    const unsigned long long mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int s = ex - 1075 + 80;  // value * 2^80 = mant * 2^s
    if (s >= 64 + 11) {            // would not fit 128 bits: saturate
        lo = ~0ull;
        hi = ~0ull >> 1;
    } else if (s >= 64) {
        hi = mant << (s - 64);
    } else if (s > 0) {
        lo = mant << s;
        hi = mant >> (64 - s);
    } else if (s > -53) {
        lo = mant >> (-s);
    }
}

__device__ __forceinline__ double from_fixed96(unsigned long long lo, unsigned long long hi) {
    return (double)hi * 0x1.0p-16 + (double)lo * 0x1.0p-80;
}

// Stop-norm accumulator of one thread: |psi_new - psi_old| summed exactly as integers in units
// of 2^-80, in four 32-bit chunks held by 64-bit counters (no carries while accumulating).
struct NormAcc {
    unsigned long long c[4];
    unsigned int big;  // set if a value reached 2^46 (outside the fixed-point range)
};

// |x| * 2^80, truncated, as a 128-bit integer (hi:lo); values below 2^-80 give 0.
__device__ __forceinline__ void abs_fixed80(double x, unsigned long long& lo, unsigned long long& hi,
                                            unsigned int& big) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    const int ex = (int)(b >> 52);
    const unsigned long long mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int s = ex - 995;  // |x| * 2^80 = mant * 2^s
    lo = 0;
    hi = 0;
    if (ex == 0) return;     // zero or below 2^-1022
    if (s >= 74) {           // |x| >= 2^46 (also inf/nan)
        big = 1;
        return;
    }
    if (s >= 64) {
        hi = mant << (s - 64);
    } else if (s > 0) {
        lo = mant << s;
        hi = mant >> (64 - s);
    } else if (s > -53) {
        lo = mant >> (-s);
    }
}

// acc += |nw - old|, exactly in fixed point (both truncated at 2^-80), on the integer pipes.
__device__ __forceinline__ void norm_add(NormAcc& acc, double nw, double old) {
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
            unsigned long long dl, dh;
            if (s == 0) {
                dl = d;
                dh = 0;
            } else if (s < 64) {
                dl = d << s;
                dh = d >> (64 - s);
            } else {
                dl = 0;
                dh = d << (s - 64);
            }
            acc.c[0] += dl & 0xffffffffull;
            acc.c[1] += dl >> 32;
            acc.c[2] += dh & 0xffffffffull;
            acc.c[3] += dh >> 32;
            return;
        }
    }
    unsigned long long al, ah, bl, bh;
    abs_fixed80(nw, al, ah, acc.big);
    abs_fixed80(old, bl, bh, acc.big);
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
}

__device__ __forceinline__ bool big_or_zero(double x) {
    // |x| >= 2^-960 (biased exponent >= 63) or x == +-0
    const int hi = __double2hiint(x);
    const int lo = __double2loint(x);
    return ((hi & 0x7ff00000) >= (63 << 20)) || (((hi & 0x7fffffff) | lo) == 0);
}

// x * c rounded to nearest, ties to even, by integer arithmetic, for a normal constant c (bit
// pattern cb): the 106-bit product of the two 53-bit significands, its top 53 bits, and the
// IEEE 754 round-half-to-even rule on the rest. A zero x gives the signed zero. Returns false
// (the caller multiplies on the FP64 pipe instead) for a subnormal, infinite or NaN x, a c that
// is not normal, and products outside the normal range, so every result equals __dmul_rn(x, c).
// The exact update uses it for its two multiplications by constants, which moves them from the
// FP64 pipe (the solver's bottleneck at 7 FP64 operations per cell) to the integer pipes.
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
    const unsigned long long mx = (xb & frac) | (1ull << 52);
    const unsigned long long mc = (cb & frac) | (1ull << 52);
    const unsigned long long lo = mx * mc;
    const unsigned long long hi = __umul64hi(mx, mc);  // 2^104 <= hi:lo < 2^106
    const int top = (int)(hi >> 41);                     // 1 when the product is >= 2^105
    int e = ex + ec - 1023 + top;                        // biased exponent before rounding
    if (e <= 0) return false;
    unsigned long long mant, rem, half;
    if (top) {
        mant = (hi << 11) | (lo >> 53);
        rem = lo & ((1ull << 53) - 1);
        half = 1ull << 52;
    } else {
        mant = (hi << 12) | (lo >> 52);
        rem = lo & ((1ull << 52) - 1);
        half = 1ull << 51;
    }
    mant += (rem > half || (rem == half && (mant & 1))) ? 1 : 0;
    if (mant >> 53) {  // rounded up to 2^53
        mant >>= 1;
        ++e;
    }
    if (e >= 0x7ff) return false;
    out = __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | (mant & frac)));
    return true;
}

// c * x as the exact update computes it: on the integer pipes where mul_rn_int applies, on the
// FP64 pipe otherwise (the same bits either way).
__device__ __forceinline__ double mul_rn(double c, double x) {
    double r;
    if (!mul_rn_int(x, (unsigned long long)__double_as_longlong(c), r)) r = __dmul_rn(c, x);
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
            if (big_or_zero(s1) && big_or_zero(s2) && big_or_zero(S) && big_or_zero(t)) {
                if (KIND == CNV_POISSON_SOR)
                    nw = __dadd_rn(mul_rn(p.b4, t), mul_rn(p.omb, old));
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
            // beta*(dy*dy*(up+dn) + dx*dx*(rt+lt) - dx*dx*dy*dy*f) / (2*(dx*dx+dy*dy)) + (1-beta)*u0
            const double num = __dsub_rn(__dadd_rn(__dmul_rn(p.dy2, __dadd_rn(up, dn)),
                                                   __dmul_rn(p.dx2, __dadd_rn(rt, lt))), g);
            if (KIND == CNV_POISSON_SOR) {
                const double bn = __dmul_rn(p.beta, num);
                const double q = p.den_pow2 ? __dmul_rn(bn, p.rden) : __ddiv_rn(bn, p.den);
                nw = __dadd_rn(q, __dmul_rn(p.omb, old));
            } else {
                nw = p.den_pow2 ? __dmul_rn(num, p.rden) : __ddiv_rn(num, p.den);
            }
        }
        return nw;
    } else {
        const double gs = fma(p.wy, up + dn, fma(p.wx, rt + lt, -g));
        nw = KIND == CNV_POISSON_SOR ? fma(p.beta, gs - old, old) : gs;
        return nw;
    }
}

// The new value of one cell, with |new - old| added to the stop norm.
template <Arith A, int KIND, bool FOLD>
__device__ __forceinline__ double point_update(const PoissonParams& p, double up, double dn, double rt,
                                               double lt, double g, double old, NormAcc& acc) {
    const double nw = point_value<A, KIND, FOLD>(p, up, dn, rt, lt, g, old);
    norm_add(acc, nw, old);
    return nw;
}

}  // namespace
}  // namespace cnv
