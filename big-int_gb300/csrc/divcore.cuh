// divcore.cuh -- the CTA-level shifted-inverse division shared by the uniform
// batch kernel (div.cu) and the uneven-batch kernel (batch.cu).  See div.cu
// for the algorithm and its correspondence with the reference.
#pragma once

#include <type_traits>

#include "blockops.cuh"
#include "divlimb.cuh"
#include "divsmall.cuh"

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

// The first iterate of the shifted inverse comes from long division: the
// whole inverse when its precision is at most DIV_INIT_LONG_ALL limbs (no
// Newton step at all; div_warp<2> holds divisors up to 64 limbs), else up to
// DIV_INIT_LONG_MAX limbs -- on one warp a quotient limb costs about 800
// cycles and a Newton step on the CTA 13-18K at these precisions, so long
// division to 32 limbs and one more step beat long division to 64 (512/256
// limbs: 167K -> 163K cycles; 1024/512: 334K -> 326K).
constexpr int DIV_INIT_LONG_ALL = 64;
constexpr int DIV_INIT_LONG_MAX = 32;

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
    // start at p0 -- P itself when P <= DIV_INIT_LONG_ALL, else the largest
    // scheduled precision <= DIV_INIT_LONG_MAX: Y_p0 = floor((B^(2 p0) - 1) / D)
    // for D = the top p0 limbs of v, by long division on one warp
    // (divsmall.cuh) -- about p0 quotient limbs of a few hundred cycles each,
    // where the Newton steps it replaces cost a block product and barriers each
    int p0 = 2;
    const int init_cap = P <= DIV_INIT_LONG_ALL ? P : DIV_INIT_LONG_MAX;
    for (int si = 0; si < ns; si++)
        if (sched[si] <= init_cap && sched[si] > p0) p0 = sched[si];
    const bool init_warp = std::is_same<Grp, CtaGroup>::value ? threadIdx.x < 32 : true;
    if (init_warp) {
        auto ld_u = [](uint32_t) { return ~0ull; };
        auto ld_v = [&](uint32_t i) -> uint64_t {
            const int src = K - p0 + (int)i;
            return src >= 0 ? Vn[src] : 0;
        };
        auto st_q = [&](uint32_t i, uint64_t x) {
            if (i <= (uint32_t)p0) Yb[Pmax - p0 + i] = x;   // the quotient has p0 + 1 limbs
        };
        auto st_r = [](uint32_t, uint64_t) {};
        if (p0 <= 32)
            div_warp<1>(2 * (uint32_t)p0, (uint32_t)p0, ld_u, ld_v, st_q, st_r);
        else
            div_warp<2>(2 * (uint32_t)p0, (uint32_t)p0, ld_u, ld_v, st_q, st_r);
        if ((threadIdx.x & 31) == 0) Yb[Pmax + 1] = 0;
    }
    Grp::sync();
    int p = p0;
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
