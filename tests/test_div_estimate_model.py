"""A line-for-line Python model of the long division's quotient-limb estimate
(divlimb.cuh: recip_3by2, div_3by2; divsmall.cuh: qhat_3by2) checked
against exact integer division, on random and extreme operands: the 3-by-2
reciprocal floor((B^3 - 1) / (d1 B + d0)) - B, the 3-by-2 quotient, and the
capped estimate against floor((u2 u1 u0) / (d1 d2)).  The CUDA code itself is
checked by the GPU division tests; this pins the arithmetic it transcribes
(Moller and Granlund, "Improved division by invariant integers", 2011,
Algorithms 5 and 6)."""
import random

B = 1 << 64
M = B - 1


def recip_limb(d):
    """floor((B^2 - 1) / d) - B for a normalised d (what recip_limb returns)."""
    return (B * B - 1) // d - B


def recip_3by2(d1, d0, v):
    p = (d1 * v) & M
    p = (p + d0) & M
    if p < d0:
        v -= 1
        if p >= d1:
            v -= 1
            p = (p - d1) & M
        p = (p - d1) & M
    t = v * d0
    t0, t1 = t & M, t >> 64
    p = (p + t1) & M
    if p < t1:
        v -= 1
        if p > d1 or (p == d1 and t0 >= d0):
            v -= 1
    return v


def div_3by2(u2, u1, u0, d1, d0, v):
    p = v * u2
    q0, q1 = p & M, p >> 64
    s = (q0 + u1) & M
    q1 = (q1 + u2 + (1 if s < q0 else 0)) & M
    q0 = s
    r1 = (u1 - q1 * d1) & M
    t = d0 * q1
    t0, t1 = t & M, t >> 64
    r0 = (u0 - t0) & M
    r1 = (r1 - t1 - (1 if u0 < t0 else 0)) & M
    r0d = (r0 - d0) & M
    r1 = (r1 - d1 - (1 if r0 < d0 else 0)) & M
    r0 = r0d
    down = r1 >= q0
    q1 = (q1 + (0 if down else 1)) & M
    x = (r0 + (d0 if down else 0)) & M
    r1 = (r1 + (d1 if down else 0) + (1 if x < r0 else 0)) & M
    r0 = x
    if r1 > d1 or (r1 == d1 and r0 >= d0):
        q1 += 1
    return q1


def qhat_3by2(u2, u1, u0, d1, d2, v3):
    q = div_3by2(u2, u1, u0, d1, d2, v3)
    return M if (u2 > d1 or (u2 == d1 and u1 >= d2)) else q


def _divisors(rng, n):
    for _ in range(n):
        d1 = rng.choice([rng.randrange(B // 2, B), B // 2, M, B // 2 + 1, M - 1])
        d0 = rng.choice([rng.randrange(B), 0, M, 1, M - 1])
        yield d1, d0


def test_reciprocal_3by2_is_exact():
    rng = random.Random(11)
    for d1, d0 in _divisors(rng, 20000):
        assert recip_3by2(d1, d0, recip_limb(d1)) == (B ** 3 - 1) // (d1 * B + d0) - B, (hex(d1), hex(d0))


def test_quotient_3by2_is_exact():
    rng = random.Random(12)
    for d1, d0 in _divisors(rng, 20000):
        D = d1 * B + d0
        v = recip_3by2(d1, d0, recip_limb(d1))
        top = rng.choice([rng.randrange(D), D - 1, 0])
        u0 = rng.choice([rng.randrange(B), 0, M])
        U = top * B + u0
        assert div_3by2(top >> 64, top & M, u0, d1, d0, v) == U // D


def test_capped_estimate_is_the_3by2_quotient():
    rng = random.Random(13)
    for d1, d2 in _divisors(rng, 20000):
        v = recip_3by2(d1, d2, recip_limb(d1))
        # a running remainder's top limbs: (u2, u1) <= (d1, d2)
        top = rng.choice([rng.randrange(d1 * B + d2 + 1), d1 * B + d2, d1 * B])
        u0 = rng.randrange(B)
        want = min((top * B + u0) // (d1 * B + d2), M)
        assert qhat_3by2(top >> 64, top & M, u0, d1, d2, v) == want
