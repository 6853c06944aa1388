// divlimb.cuh -- one-limb division helpers shared by the long division
// (divsmall.cuh), the shifted inverse (divcore.cuh) and the batched division
// primitives (prims.cu): the reciprocal of a normalised limb and the 2-by-1
// division that uses it, and the 3-by-2 reciprocal and division that long
// division's quotient-limb estimate uses.
#pragma once

#include <stdint.h>

namespace bi {

// floor((2^128 - 1) / d) - 2^64 for d >= 2^63: the low limb of a one-limb
// reciprocal (the quotient is in (2^64, 2^65)), in integer arithmetic apart
// from the seed.  Seed: the correctly rounded single-precision reciprocal of
// the top 24 bits of d (relative error below 2^-22, so v is off by less than
// 2^43).  Two Newton steps Y <- Y + Y r / 2^128 on Y = 2^64 + v, with
// r = r(v) = (B - d) B - 1 - v d the exact residual (a signed 128-bit value),
// take the error to a few units; comparing r(v) with 0 and d then fixes v to
// the exact floor (at most two unit steps over 220,000 checked divisors,
// including 2^63, 2^64 - 1 and every divisor with a one-bit tail).
__device__ __forceinline__ void recip_residual(uint64_t d, uint64_t v, int64_t& r_hi, uint64_t& r_lo) {
    const uint64_t a_hi = (0 - d) - 1, a_lo = ~0ull;   // (B - d) B - 1
    const uint64_t p_lo = v * d, p_hi = __umul64hi(v, d);
    r_lo = a_lo - p_lo;
    r_hi = (int64_t)(a_hi - p_hi - (a_lo < p_lo ? 1 : 0));
}

// One Newton step: Y r / 2^128 = r_hi + v r_hi / 2^64 + (a part below 2),
// added to v with saturation to [0, 2^64 - 1], where the answer lies.
__device__ __forceinline__ uint64_t recip_newton(uint64_t d, uint64_t v) {
    int64_t r_hi;
    uint64_t r_lo;
    recip_residual(d, v, r_hi, r_lo);
    if (r_hi >= 0) {
        const uint64_t m = (uint64_t)r_hi;
        const uint64_t hi = __umul64hi(v, m);
        const uint64_t delta = m + hi;                 // < 2^44: no wrap
        return v + delta < v ? ~0ull : v + delta;
    }
    const uint64_t m = (uint64_t)(-r_hi);
    const uint64_t delta = m + __umul64hi(v, m);
    return delta > v ? 0ull : v - delta;
}

__device__ __forceinline__ uint64_t recip_limb(uint64_t d) {
    // seed: 1 / f for f = the top 24 bits of d, f in [2^23, 2^24) exactly
    // representable; the reciprocal lies in (2^-24, 2^-23]
    const float rf = __frcp_rn(__uint2float_rn((uint32_t)(d >> 40)));
    const uint32_t bits = __float_as_uint(rf);
    // (1 + frac 2^-23) 2^-24 * 2^88 = 2^64 + frac 2^41; 2^-23 only for f = 2^23
    uint64_t v = ((bits >> 23) & 0xffu) == 127u - 23u ? ~0ull : (uint64_t)(bits & 0x7fffffu) << 41;
    v = recip_newton(d, v);
    v = recip_newton(d, v);
    int64_t r_hi;
    uint64_t r_lo;
    for (int it = 0; it < 8; it++) {   // at most two steps
        recip_residual(d, v, r_hi, r_lo);
        if (r_hi < 0 && v > 0) { v -= 1; continue; }
        if ((r_hi > 0 || r_lo >= d) && v < ~0ull) { v += 1; continue; }
        break;
    }
    return v;
}

// 2-by-1 division of (u1, u0) by a normalised d (top bit set), u1 < d, with
// its reciprocal v = recip_limb(d) (Moller and Granlund, "Improved division
// by invariant integers", IEEE Trans. Computers 60(2), 2011, Algorithm 4).
__device__ __forceinline__ uint64_t div_2by1(uint64_t u1, uint64_t u0, uint64_t d, uint64_t v, uint64_t& r) {
    uint64_t q0 = v * u1;
    uint64_t q1 = __umul64hi(v, u1);
    const uint64_t s = q0 + u0;
    q1 += u1 + (s < q0 ? 1 : 0);
    q0 = s;
    q1 += 1;
    uint64_t rr = u0 - q1 * d;
    if (rr > q0) {
        q1 -= 1;
        rr += d;
    }
    if (rr >= d) {
        q1 += 1;
        rr -= d;
    }
    r = rr;
    return q1;
}

// The 3-by-2 reciprocal of a normalised two-limb divisor (d1, d0):
// v = floor((B^3 - 1) / (d1 B + d0)) - B, from the one-limb reciprocal v of
// d1 (recip_limb) by Moller and Granlund's Algorithm 6 ("Improved division by
// invariant integers", IEEE Trans. Computers 60(2), 2011): d1 v + d0 and the
// high limb of v d0 added up, v stepped down once or twice on each carry.
// (A line-for-line model of this code and of div_3by2 is checked against
// exact division in tests/test_div_estimate_model.py.)
__device__ __forceinline__ uint64_t recip_3by2(uint64_t d1, uint64_t d0, uint64_t v) {
    uint64_t p = d1 * v;
    p += d0;
    if (p < d0) {                 // carry
        v -= 1;
        if (p >= d1) {
            v -= 1;
            p -= d1;
        }
        p -= d1;
    }
    const uint64_t t0 = v * d0, t1 = __umul64hi(v, d0);
    p += t1;
    if (p < t1) {                 // carry
        v -= 1;
        if (p > d1 || (p == d1 && t0 >= d0)) v -= 1;
    }
    return v;
}

// The quotient limb floor((u2 B^2 + u1 B + u0) / (d1 B + d0)) for a
// normalised (d1, d0) with (u2, u1) < (d1, d0), from its 3-by-2 reciprocal v
// (Moller and Granlund, "Improved division by invariant integers", IEEE
// Trans. Computers 60(2), 2011, Algorithm 5): two products for the
// candidate, one remainder check that steps it down (about half the time),
// one rare check that steps it up.  This is the long division's estimate
// with Knuth's q-hat * v_(n-2) test built in (TAOCP 4.3.1, step D3): at most
// one too large for the full divisor.
__device__ __forceinline__ uint64_t div_3by2(uint64_t u2, uint64_t u1, uint64_t u0, uint64_t d1, uint64_t d0,
                                             uint64_t v) {
    // (q1, q0) = v u2 + (u2, u1)
    uint64_t q0 = v * u2;
    uint64_t q1 = __umul64hi(v, u2);
    const uint64_t s = q0 + u1;
    q1 += u2 + (s < q0 ? 1 : 0);
    q0 = s;
    // (r1, r0) = (u1 - q1 d1, u0) - q1 d0 - (d1, d0)  (mod B^2)
    uint64_t r1 = u1 - q1 * d1;
    const uint64_t t0 = d0 * q1, t1 = __umul64hi(d0, q1);
    uint64_t r0 = u0 - t0;
    r1 = r1 - t1 - (u0 < t0 ? 1 : 0);
    const uint64_t r0d = r0 - d0;
    r1 = r1 - d1 - (r0 < d0 ? 1 : 0);
    r0 = r0d;
    // the two adjustments as selects, not branches: the estimate is on every
    // quotient limb's critical path
    const bool down = r1 >= q0;   // the candidate q1 + 1 is one too large
    q1 += down ? 0 : 1;
    const uint64_t x = r0 + (down ? d0 : 0);
    r1 += (down ? d1 : 0) + (x < r0 ? 1 : 0);
    r0 = x;
    q1 += (r1 > d1 || (r1 == d1 && r0 >= d0)) ? 1 : 0;   // one too small (rare)
    return q1;
}

}  // namespace bi
