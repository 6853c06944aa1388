// divcore.cuh -- the CTA-level shifted-inverse division shared by the uniform
// batch kernel (div.cu) and the uneven-batch kernel (batch.cu).  See div.cu
// for the algorithm and its correspondence with the reference.
#pragma once

#include <type_traits>

#include "blockops.cuh"

namespace bi {

constexpr int DIV_MAX_CORRECTIONS = 8;

struct DivGeom {
    uint32_t mu, mv;        // limbs per dividend / divisor in the caller's type
    uint32_t MU, MV;        // the same in 64-bit limbs
    uint32_t Pmax;          // largest reciprocal precision (limbs)
    uint32_t oUn, oVn, oY, oX;
    uint32_t oVs, oT, oProd, oW;             // phase N (Newton) offsets inside X
    uint32_t oBig, oQ, oQV, oR, oW2;         // phases Q/R offsets inside X
    uint32_t smem_limbs;
};

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

// The shifted inverse starts at the largest scheduled precision up to this
// many limbs, computed by recip_longdiv instead of Newton steps.
constexpr int DIV_LONGDIV_MAX = 10;

// Y[0..n] = floor((B^(2n) - 1) / D) for D = the top n limbs of the
// normalised divisor (Vn[K-n .. K-1], zeros below when K < n): a shifted
// inverse at precision n computed directly by schoolbook long division
// (Knuth, TAOCP vol. 2, 4.3.1, Algorithm D) with 2-by-1 quotient estimates.
// One thread; u holds 2n + 1 limbs of scratch.  vr = recip_limb(Vn[K-1]).
// Kept out of line and as a plain loop: it runs once per division, where a
// compact body costs fewer instruction fetches than an unrolled one.
__device__ __noinline__ static void recip_longdiv(uint64_t* Y, int n, const uint64_t* Vn, int K, uint64_t vr,
                                                  uint64_t* u) {
    auto D = [&](int i) -> uint64_t {
        const int src = K - n + i;
        return src >= 0 ? Vn[src] : 0;
    };
    for (int i = 0; i < 2 * n; i++) u[i] = ~0ull;
    u[2 * n] = 0;
    const uint64_t d1 = D(n - 1), d2 = n >= 2 ? D(n - 2) : 0;
    for (int j = n; j >= 0; j--) {
        const uint64_t u2 = u[j + n], u1 = u[j + n - 1], u0 = (j + n >= 2) ? u[j + n - 2] : 0;
        uint64_t qh, rh;
        bool rh_over = false;
        if (u2 >= d1) {                  // u2 == d1: q-hat = B - 1, r-hat = u1 + d1
            qh = ~0ull;
            rh = u1 + d1;
            rh_over = rh < u1;
        } else {
            qh = div_2by1(u2, u1, d1, vr, rh);
        }
        for (int t = 0; t < 2 && !rh_over; t++) {   // q-hat * d2 > r-hat * B + u0: one too large
            const uint64_t p_lo = qh * d2, p_hi = __umul64hi(qh, d2);
            if (p_hi > rh || (p_hi == rh && p_lo > u0)) {
                qh -= 1;
                const uint64_t nr = rh + d1;
                rh_over = nr < rh;
                rh = nr;
            } else {
                break;
            }
        }
        // u[j .. j+n] -= q-hat * D
        uint64_t carry = 0, borrow = 0;
        for (int i = 0; i < n; i++) {
            const uint64_t d = D(i);
            const uint64_t plo = qh * d, phi = __umul64hi(qh, d);
            const uint64_t sub = plo + carry;
            carry = phi + (sub < plo ? 1 : 0);
            const uint64_t x = u[j + i];
            const uint64_t y = x - sub;
            const uint64_t b1 = x < sub ? 1 : 0;
            u[j + i] = y - borrow;
            borrow = b1 | (y < borrow ? 1 : 0);
        }
        const uint64_t x = u[j + n];
        const uint64_t y = x - carry;
        const uint64_t b1 = x < carry ? 1 : 0;
        u[j + n] = y - borrow;
        const bool neg = (b1 | (y < borrow ? 1 : 0)) != 0;
        if (neg) {                       // one too large after all: add D back
            qh -= 1;
            uint64_t c = 0;
            for (int i = 0; i < n; i++) {
                const uint64_t d = D(i);
                const uint64_t s = u[j + i] + d;
                const uint64_t c1 = s < d ? 1 : 0;
                const uint64_t s2 = s + c;
                c = c1 | (s2 < s ? 1 : 0);
                u[j + i] = s2;
            }
            u[j + n] += c;
        }
        Y[j] = qh;
    }
}

// Newton steps up to this precision (limbs) run on warp 0 alone
// (WarpGroup): their operands are small, and one warp with __syncwarp
// finishes them sooner than the whole CTA with its barriers.
constexpr int DIV_WARP_NEWTON_MAX = 64;

// One Newton step of the shifted inverse, from precision p to pn: Y_p (p + 1
// limbs at Yb + (Pmax - p)) becomes Y_pn (pn + 1 limbs at Yb + (Pmax - pn)).
template <typename Grp>
__device__ __forceinline__ void newton_step(const DivGeom& g, const uint64_t* Vn, int K, uint64_t* Yb, uint64_t* X,
                                            uint32_t* scratch, int p, int pn) {
    const uint32_t Pmax = g.Pmax;
    uint64_t* Vs = X + g.oVs;
    uint64_t* Tb = X + g.oT;
    uint64_t* Pr = X + g.oProd;
    uint64_t* Wb = X + g.oW;
    const int sl = pn + 1;
    // divisor prefix: the top sl limbs of v (zero-extended below when K < sl)
    for (int i = Grp::rank(); i < sl; i += Grp::size()) {
        const int src = K - sl + i;
        Vs[i] = src >= 0 ? Vn[src] : 0;
    }
    Grp::sync();
    const uint64_t* Yp = Yb + (Pmax - p);
    // T = Vs * Y_p mod B^(sl+1); E = B^(sl+p) - Vs*Y_p, |E| < B^(sl+1)/2
    block_mul<Grp>(Vs, sl, Yp, p + 1, Tb, sl + 1, Wb, scratch);
    const bool e_neg = (Tb[sl] >> 63) == 0;    // T small: E = -T
    if (!e_neg) block_addsub<Grp>(Tb, nullptr, 0, Tb, sl + 1, sl + 1, true, scratch);   // |E| = -T
    // D = floor(Y_p * |E| / B^(2p+1)), from a short product (columns >= 2p-1):
    // at most one unit short, which the next step's residual absorbs
    block_mul<Grp>(Yp, p + 1, Tb, sl + 1, Pr, p + sl + 2, Wb, scratch, 2 * p - 1);
    const uint64_t* D = Pr + 2 * p + 1;
    const int Dlen = sl - p + 1;
    // Y_pn = Y_p * B^(pn-p) +/- D
    for (int i = Grp::rank(); i < pn - p; i += Grp::size()) Yb[Pmax - pn + i] = 0;
    Grp::sync();
    uint64_t* Ypn = Yb + (Pmax - pn);
    block_addsub<Grp>(Ypn, Ypn, pn + 1, D, Dlen, pn + 1, e_neg, scratch);
}

// One division on a cooperating group (the CTA, or one warp): u has g.MU
// 64-bit limbs, v has g.MV; load_u(i) and load_v(i) supply limbs,
// store_q(i, x) for i < g.MU and store_r(i, x) for i < g.MV receive the
// results, set_status(code) the status (rank 0).  Every thread of the group
// calls it with the same arguments.
template <typename Grp = CtaGroup, typename LoadU, typename LoadV, typename StoreQ, typename StoreR,
          typename SetStatus>
__device__ __forceinline__ void div_cta(const DivGeom& g, uint64_t* smem, LoadU load_u, LoadV load_v,
                                        StoreQ store_q, StoreR store_r, SetStatus set_status) {
    uint64_t* Un = smem + g.oUn;
    uint64_t* Vn = smem + g.oVn;
    uint64_t* Yb = smem + g.oY;
    uint64_t* X = smem + g.oX;
    uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + g.smem_limbs);
    const uint32_t MU = g.MU, MV = g.MV, Pmax = g.Pmax;
    const uint32_t rk = (uint32_t)Grp::rank(), sz = (uint32_t)Grp::size();
    // ---- raw operands: u into X[0, MU), v into X[MU, MU+MV)
    uint64_t* Uraw = X;
    uint64_t* Vraw = X + MU;
    for (uint32_t i = rk; i < MU; i += sz) Uraw[i] = load_u(i);
    for (uint32_t i = rk; i < MV; i += sz) Vraw[i] = load_v(i);
    Grp::sync();
    const int K = block_prec<Grp>(Vraw, (int)MV, scratch);
    if (K == 0) {                                  // division by zero
        for (uint32_t i = rk; i < MU; i += sz) store_q(i, 0);
        for (uint32_t i = rk; i < MV; i += sz) store_r(i, 0);
        if (rk == 0) set_status(1);
        Grp::sync();
        return;
    }
    const int s = __clzll((long long)Vraw[K - 1]);
    block_shl_bits<Grp>(Vn, Vraw, K, K, s);
    block_shl_bits<Grp>(Un, Uraw, (int)MU, (int)MU + 1, s);
    Grp::sync();
    const int H = block_prec<Grp>(Un, (int)MU + 1, scratch);
    if (H < K) {                                   // u < v: q = 0, r = u
        for (uint32_t i = rk; i < MU; i += sz) store_q(i, 0);
        for (uint32_t i = rk; i < MV; i += sz) store_r(i, Uraw[i]);
        if (rk == 0) set_status(0);
        Grp::sync();
        return;
    }
    const int Qlen = H - K + 1;
    const int P = Qlen + 1;

    // ---- shifted inverse: Y_p at Yb + (Pmax - p), p + 1 limbs
    int sched[40];
    int ns = 0;
    {
        int x = P;
        sched[ns++] = x;
        while (x > 2 && ns < 40) {
            x = (x + 2) / 2;
            sched[ns++] = x;
        }
    }
    // start at p0, the largest scheduled precision <= DIV_LONGDIV_MAX, by long division
    int p0 = 1;
    for (int si = 0; si < ns; si++)
        if (sched[si] <= DIV_LONGDIV_MAX && sched[si] > p0) p0 = sched[si];
    if (rk == 0) {
        const uint64_t vr = recip_limb(Vn[K - 1]);
        if (p0 == 1) {
            Yb[Pmax - 1] = vr;
            Yb[Pmax] = 1;
        } else {
            recip_longdiv(Yb + (Pmax - p0), p0, Vn, K, vr, X + g.oProd);
        }
        Yb[Pmax + 1] = 0;
    }
    Grp::sync();
    int p = p0;
    if constexpr (std::is_same<Grp, CtaGroup>::value) {
        // the small steps on warp 0 alone, then one barrier
        if (threadIdx.x < 32) {
            int pw = p0;
            for (int si = ns - 1; si >= 0; si--) {
                const int pn = sched[si];
                if (pn <= pw) continue;
                if (pn > DIV_WARP_NEWTON_MAX) break;
                newton_step<WarpGroup>(g, Vn, K, Yb, X, scratch, pw, pn);
                pw = pn;
            }
        }
        __syncthreads();
        for (int si = ns - 1; si >= 0; si--) {     // where warp 0 stopped
            const int pn = sched[si];
            if (pn <= p) continue;
            if (pn > DIV_WARP_NEWTON_MAX) break;
            p = pn;
        }
    }
    for (int si = ns - 1; si >= 0; si--) {
        const int pn = sched[si];
        if (pn <= p) continue;
        newton_step<Grp>(g, Vn, K, Yb, X, scratch, p, pn);
        p = pn;
    }
    const uint64_t* Y = Yb + (Pmax - P);

    // ---- quotient estimate: floor(Un * Y / B^(P+K)) from a short product
    // (columns >= P+K-2): at most one short, corrected below with the rest
    uint64_t* Big = X + g.oBig;
    uint64_t* Qb = X + g.oQ;
    uint64_t* QV = X + g.oQV;
    uint64_t* Rb = X + g.oR;
    uint64_t* W2 = X + g.oW2;
    block_mul<Grp>(Un, H, Y, P + 1, Big, H + P + 1, W2, scratch, P + K - 2);
    for (int i = rk; i < Qlen + 1; i += sz) Qb[i] = i < Qlen ? Big[P + K + i] : 0;
    Grp::sync();

    // ---- remainder r = u - q*v from the low K+1 limbs, then corrections
    block_mul<Grp>(Qb, Qlen + 1, Vn, K, QV, K + 1, W2, scratch);
    block_addsub<Grp>(Rb, Un, K + 1, QV, K + 1, K + 1, true, scratch);
    int fixes = 0;
    bool ok = true;
    while ((Rb[K] >> 63) != 0) {                  // r < 0
        if (++fixes > DIV_MAX_CORRECTIONS) { ok = false; break; }
        block_addsub<Grp>(Rb, Rb, K + 1, Vn, K, K + 1, false, scratch);
        // q -= 1
        uint64_t* onebuf = QV;                     // QV is free now
        if (rk == 0) onebuf[0] = 1;
        Grp::sync();
        block_addsub<Grp>(Qb, Qb, Qlen + 1, onebuf, 1, Qlen + 1, true, scratch);
    }
    fixes = 0;
    while (ok && block_cmp<Grp>(Rb, K + 1, Vn, K, K + 1, scratch) >= 0) {   // r >= v
        if (++fixes > DIV_MAX_CORRECTIONS) { ok = false; break; }
        block_addsub<Grp>(Rb, Rb, K + 1, Vn, K, K + 1, true, scratch);
        uint64_t* onebuf = QV;
        if (rk == 0) onebuf[0] = 1;
        Grp::sync();
        block_addsub<Grp>(Qb, Qb, Qlen + 1, onebuf, 1, Qlen + 1, false, scratch);
    }

    // ---- outputs: q, and r shifted back by s bits
    uint64_t* Rout = QV;
    block_shr_bits<Grp>(Rout, Rb, K, K, s);
    Grp::sync();
    for (uint32_t i = rk; i < MU; i += sz) store_q(i, (int)i < Qlen + 1 ? Qb[i] : 0);
    for (uint32_t i = rk; i < MV; i += sz) store_r(i, (int)i < K ? Rout[i] : 0);
    if (rk == 0) set_status(ok ? 0 : 2);
    Grp::sync();
}

__host__ __device__ inline DivGeom div_geom(uint32_t mu, uint32_t mv, int wbytes) {
    DivGeom g;
    g.mu = mu;
    g.mv = mv;
    g.MU = wbytes == 8 ? mu : (mu + 1) / 2;
    g.MV = wbytes == 8 ? mv : (mv + 1) / 2;
    g.Pmax = g.MU + 2;
    const uint32_t MU = g.MU, MV = g.MV, Pm = g.Pmax;
    g.oUn = 0;
    g.oVn = g.oUn + MU + 2;
    g.oY = g.oVn + MV + 2;
    g.oX = g.oY + Pm + 4;
    // phase N
    g.oVs = 0;
    g.oT = g.oVs + Pm + 4;
    g.oProd = g.oT + Pm + 4;
    const uint32_t prodlen = 2 * Pm + 8;
    g.oW = g.oProd + prodlen;
    const uint32_t endN = g.oW + (prodlen + 7) / 8 * BLOCK_MUL_WS + BLOCK_MUL_WS;
    // phases Q and R
    const uint32_t biglen = MU + Pm + 4;
    g.oBig = 0;
    g.oQ = g.oBig + biglen;
    g.oQV = g.oQ + Pm + 4;
    g.oR = g.oQV + (MV + 4 > Pm + 4 ? MV + 4 : Pm + 4);
    g.oW2 = g.oR + MV + 4;
    const uint32_t endQ = g.oW2 + (biglen + 7) / 8 * BLOCK_MUL_WS + BLOCK_MUL_WS;
    // the raw operands are staged in X too
    uint32_t endX = endN > endQ ? endN : endQ;
    if (endX < MU + MV) endX = MU + MV;
    g.smem_limbs = g.oX + endX;
    return g;
}


__host__ __device__ inline size_t div_smem_bytes(const DivGeom& g) { return (size_t)g.smem_limbs * 8 + BLOCKOPS_SCRATCH_WORDS * 4; }
__host__ __device__ inline int div_threads(uint32_t MU) {
    return MU >= 1024 ? 512 : MU >= 256 ? 256 : MU >= 64 ? 128 : MU >= 16 ? 64 : 32;
}

}  // namespace bi
