// divblock.cuh -- long division of one instance on one warp (or on the NW
// warps of a CTA), the quotient KB limbs at a time.
//
// The quotient and remainder of u / v are unique, so this returns what the
// reference's shifted-inverse division (prototypes/div.c:427-467) returns;
// the method is schoolbook long division in base B^KB (Knuth, TAOCP vol. 2,
// 4.3.1, Algorithm D, with KB-limb quotient digits).  Per block of KB
// quotient limbs:
//   1. the block's quotient Q-hat = floor(U / V'), from the top 2 KB + 1
//      limbs U of the running remainder W and the top KB + 1 limbs V' of the
//      normalised divisor D -- a small long division on one thread with 3-by-2
//      estimates (divlimb.cuh), capped at B^KB - 1.  With W < D B^KB and
//      V' >= B^(KB+1) / 2, Q <= Q-hat <= Q + 1 for the true block quotient
//      Q = floor(W / D): a one-limb-longer prefix of the divisor than the
//      quotient is long keeps the truncation error below one unit.  The
//      small division leaves U - Q-hat V' in place, so the top KB + 1 limbs
//      of the divisor need no second multiply;
//   2. W -= Q-hat (D - V' B^(MX-KB-1)) as KB rows of KB x VPL limb products
//      in every lane (two carry chains a row, the same register blocking as
//      the multiply's row_mac8): each lane subtracts the part of its rows
//      that lands on its own limbs and accumulates the part above them (its
//      spill, KB + 1 limbs) for the next lane;
//   3. each lane subtracts the spill of the lane below -- a borrow out of
//      that is rare (the spill is a KB-limb number taken from KB + 1 limbs)
//      -- and the lane-to-lane borrows are resolved by two ballots (and, on
//      several warps, one exchange through shared memory);
//   4. the sign of what lands above the divisor's top limb says whether
//      Q-hat was one too large; then D is added back (rare);
//   5. the remainder window moves up KB limbs and KB dividend limbs enter at
//      the bottom.
// Against one quotient limb per step (divsmall.cuh), the estimate, the
// ballots, the shuffles and the window slide are paid once per KB limbs and
// the multiply-subtract's rows have no ballot between them.  The library uses
// it for divisors above 1024 limbs, on two (up to 2048 limbs) or four warps:
// there the one-limb-per-step kernels run out of registers.  Up to 1024 limbs
// it divides no faster than they do (GB300, 2m/m: 512/256 limbs 7.1M vs 8.1M
// div/s, 1024/512 1.7M vs 2.1M, 2048/1024 590K vs 607K) -- per quotient limb
// the rows still cost about 11.5 instructions a limb product and the one-
// thread small division about 190 instructions, so the count of instructions
// changes little, and its 255 registers a thread at 32 limbs a lane leave no
// room to run products ahead of their carry chains.
//
// Layout: lane gl (of NL = 32 NW lanes) holds window and divisor positions
// gl VPL .. gl VPL + VPL - 1 (MX = NL VPL positions); the top lane (gl =
// NL - 1) also holds the KB window limbs above the divisor, positions
// MX .. MX + KB - 1, in X[VPL ..].  The divisor D = v 2^s B^(MX-K) (K the
// divisor's significant limbs, s the shift that sets D's top bit) and the
// dividend u 2^s B^(MX-K) give the same quotient as u / v; the remainder
// is read back from positions MX - K .. MX - 1 shifted right by s bits.
#pragma once

#include "chain.cuh"
#include "divlimb.cuh"
#include "divsmall.cuh"

namespace bi {

// Shared-memory exchange area of one division on NW > 1 warps.
template <int KB, int NW>
struct DivBlkShared {
    uint64_t q[KB];                // the block's quotient, from the top lane
    uint64_t spill[NW][KB + 1];    // warp w's lane-31 spill, for warp w + 1
    uint64_t slide[NW][KB];        // warp w's top KB window limbs, for warp w + 1
    uint64_t rnext[NW];            // warp w's lane-0 limb, for warp w - 1's remainder
    uint64_t tv;                   // the top lane's limb above the divisor less its spill
    uint32_t gp[NW];               // warp w's borrow out without / with a borrow in (bits 0, 1)
    uint32_t gp2[NW];              // the same for the add-back's carries
    uint32_t kw[NW];               // warp w's divisor precision
};

// floor(U / V) for a (2 KB + 1)-limb U and a normalised (KB + 1)-limb V,
// capped at B^KB - 1; U is left holding U - Q V.  The small long division:
// the cap is taken when U's top KB + 1 limbs are >= V, otherwise KB
// quotient limbs each from a 3-by-2 estimate (d1, d0 = V's top two limbs,
// v3 their reciprocal), a multiply-subtract of KB + 1 limbs and an add-back
// when the estimate was one too large.
template <int KB>
__device__ __forceinline__ void blk_estimate(uint64_t (&U)[2 * KB + 1], const uint64_t (&V)[KB + 1], uint64_t v3,
                                             uint64_t (&Q)[KB]) {
    const uint64_t d1 = V[KB], d0 = V[KB - 1];
    {
        uint64_t T[KB + 1];
#pragma unroll
        for (int k = 0; k <= KB; k++) T[k] = U[KB + k];
        const uint32_t bt = chain_sub_gen<KB + 1>(T, [&](int k) { return V[k]; }, 0u);
        if (bt == 0) {   // the quotient would be B^KB or more (rare): B^KB - 1
#pragma unroll
            for (int k = 0; k < KB; k++) Q[k] = ~0ull;
#pragma unroll
            for (int k = 0; k <= KB; k++) U[KB + k] = T[k];   // U -= V B^KB
            uint32_t c = chain_add_gen<KB + 1>(U, [&](int k) { return V[k]; }, 0u);   // U += V
#pragma unroll
            for (int k = KB + 1; k <= 2 * KB; k++) {
                const uint64_t y = U[k];
                U[k] = y + c;
                c &= y == ~0ull ? 1u : 0u;
            }
            return;
        }
    }
#pragma unroll
    for (int j = KB - 1; j >= 0; j--) {
        uint64_t qh = qhat_3by2(U[j + KB + 1], U[j + KB], U[j + KB - 1], d1, d0, v3);
        // U[j .. j+KB+1] -= qh V: the high halves one limb up, then the low
        // halves, whose borrow out is taken from U[j+KB+1]
        const uint32_t bA = chain_sub_gen<KB + 1>(&U[j + 1], [&](int k) { return __umul64hi(qh, V[k]); }, 0u);
        const uint32_t bo = chain_sub_gen<KB + 1>(&U[j], [&](int k) { return qh * V[k]; }, 0u);
        const bool bB = U[j + KB + 1] < bo;
        U[j + KB + 1] -= bo;
        if (bA != 0 || bB) {   // one too large: add V back
            qh -= 1;
            const uint32_t c = chain_add_gen<KB + 1>(&U[j], [&](int k) { return V[k]; }, 0u);
            U[j + KB + 1] += c;
        }
        Q[j] = qh;
    }
}

// Row I .. KB-1 of the block's multiply-subtract in one lane: X[I ..] -=
// Q[I] dm(.) shifted up I limbs, the part above the lane's VPL limbs added
// to the spill S (with the borrows out of X's top limb).  Two chains a row:
// the low halves of the products at positions I + c, the high halves at
// I + c + 1.
template <int VPL, int KB, int I, typename DM>
__device__ __forceinline__ void blk_rows(uint64_t (&X)[VPL + KB], uint64_t (&S)[KB + 1], DM dm,
                                         const uint64_t (&Q)[KB]) {
    if constexpr (I < KB) {
        const uint64_t q = Q[I];
        uint32_t b = chain_sub_gen<VPL - I>(&X[I], [&](int c) { return q * dm(c); }, 0u);
        if constexpr (I > 0) b = chain_add_gen<I>(S, [&](int c) { return q * dm(VPL - I + c); }, b);
        S[I] += b;
        uint32_t h = 0;
        if constexpr (VPL - 1 - I > 0)
            h = chain_sub_gen<VPL - 1 - I>(&X[I + 1], [&](int c) { return __umul64hi(q, dm(c)); }, 0u);
        h = chain_add_gen<I + 1>(S, [&](int c) { return __umul64hi(q, dm(VPL - 1 - I + c)); }, h);
        S[I + 1] += h;
        blk_rows<VPL, KB, I + 1>(X, S, dm, Q);
    }
}

// One instance on NW warps (all 32 NW lanes call with the same arguments;
// for NW > 1 the CTA is exactly those warps and `sh` their shared area, for
// NW = 1 any warp of a CTA and `sh` unused): u (MU 64-bit limbs through
// load_u) divided by v (MV <= 32 NW VPL limbs through load_v); writes MU
// quotient limbs and MV remainder limbs.  Returns the status: 0, or 1 when
// v == 0 (then q = r = 0).
template <int VPL, int KB, int NW, typename LoadU, typename LoadV, typename StoreQ, typename StoreR>
__device__ __forceinline__ uint8_t div_blk(uint32_t MU, uint32_t MV, LoadU load_u, LoadV load_v, StoreQ store_q,
                                           StoreR store_r, DivBlkShared<KB, NW>* sh) {
    static_assert(KB >= 2 && 32 % KB == 0, "div_blk: KB divides 32");
    static_assert(VPL >= KB + 1, "div_blk: the top lane holds the divisor's top KB + 1 limbs");
    constexpr int NL = 32 * NW, MX = NL * VPL;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31);
    const int w = NW == 1 ? 0 : (int)(threadIdx.x >> 5);
    const int gl = w * 32 + lane;
    const bool top = gl == NL - 1;

    // K = the divisor's significant limbs
    uint32_t K;
    {
        uint32_t kl = 0;
#pragma unroll 4
        for (int i = 0; i < VPL; i++) {
            const uint32_t idx = (uint32_t)(i * NL + gl);
            if (idx < MV && load_v(idx) != 0) kl = idx + 1;
        }
        K = __reduce_max_sync(FULL, kl);
        if constexpr (NW > 1) {
            if (lane == 0) sh->kw[w] = K;
            __syncthreads();
#pragma unroll
            for (int x = 0; x < NW; x++) K = max(K, sh->kw[x]);
        }
    }
    if (K == 0 || MU < K) {   // zero divisor (status 1), or u < v: q = 0, r = u
        for (uint32_t i = (uint32_t)gl; i < MU; i += NL) store_q(i, 0);
        for (uint32_t i = (uint32_t)gl; i < MV; i += NL) store_r(i, (K != 0 && i < MU) ? load_u(i) : 0);
        if constexpr (NW > 1) __syncthreads();
        return K == 0 ? 1 : 0;
    }
    const int s = __clzll((long long)load_v(K - 1));
    const int rs = 63 - s;   // x >> (64 - s) written as (x >> 1) >> rs: 0 when s == 0
    const int zl = MX - (int)K;
    uint64_t D[VPL];
    {
        auto vl = [&](int j) -> uint64_t { return (j >= 0 && j < (int)K) ? load_v((uint32_t)j) : 0; };
        uint64_t prev = vl(gl * VPL - zl - 1);
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t cur = vl(gl * VPL + i - zl);
            D[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    uint64_t v3 = 0;
    if (top) v3 = recip_3by2(D[VPL - 1], D[VPL - 2], recip_limb(D[VPL - 1]));

    const int nq = (int)MU - (int)K + 1;          // quotient limbs
    const int pad = (KB - nq % KB) % KB;          // zero quotient limbs on top that fill the first block
    const int nblk = (nq + pad) / KB;
    const int x0 = (int)MU + pad - MX - KB + 1;   // window position p holds limb x0 + p of u 2^s
    auto raw = [&](int t) -> uint64_t { return (t >= 0 && t < (int)MU) ? load_u((uint32_t)t) : 0; };
    auto shl = [&](int t) -> uint64_t { return (raw(t) << s) | ((raw(t - 1) >> 1) >> rs); };
    uint64_t X[VPL + KB];
    {
        const int t0 = x0 + gl * VPL;
        uint64_t prev = raw(t0 - 1);
#pragma unroll
        for (int i = 0; i < VPL + KB; i++) {   // X[VPL ..]: the top lane's limbs above the divisor
            const uint64_t cur = (i < VPL || top) ? raw(t0 + i) : 0;
            X[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    // dividend limbs still to enter, highest first: element k is limb x0 - 1 - k
    // of u 2^s; warp 0 keeps elements of two 32-element chunks, one a lane
    uint64_t chunk = 0, chunk_next = 0;
    if (w == 0) {
        chunk = shl(x0 - 1 - lane);
        chunk_next = shl(x0 - 33 - lane);
    }

    for (int b = 0; b < nblk; b++) {
        // 1. the block's quotient, in the top lane
        uint64_t Q[KB];
        if (top) {
            blk_estimate<KB>(*reinterpret_cast<uint64_t(*)[2 * KB + 1]>(&X[VPL - KB - 1]),
                             *reinterpret_cast<const uint64_t(*)[KB + 1]>(&D[VPL - KB - 1]), v3, Q);
            if constexpr (NW > 1) {
#pragma unroll
                for (int k = 0; k < KB; k++) sh->q[k] = Q[k];
            }
        }
        if constexpr (NW > 1) {
            __syncthreads();
#pragma unroll
            for (int k = 0; k < KB; k++) Q[k] = sh->q[k];
            if (b > 0 && lane == 0 && w > 0) {   // the limbs the last slide brought from the warp below
#pragma unroll
                for (int i = 0; i < KB; i++) X[i] = sh->slide[w - 1][i];
            }
        } else {
#pragma unroll
            for (int k = 0; k < KB; k++) Q[k] = __shfl_sync(FULL, Q[k], 31);
        }
        // 2. rows: the top lane's top KB + 1 divisor limbs were handled by step 1
        uint64_t S[KB + 1];
#pragma unroll
        for (int k = 0; k <= KB; k++) S[k] = 0;
        auto dm = [&](int c) -> uint64_t { return (c >= VPL - KB - 1 && top) ? 0ull : D[c]; };
        blk_rows<VPL, KB, 0>(X, S, dm, Q);
        const uint64_t tl = X[VPL] - S[0];   // top lane: what lands at position MX (its spill is borrows only)
        // 3. the spill of the lane below
        uint64_t Sin[KB + 1];
#pragma unroll
        for (int k = 0; k <= KB; k++) {
            const uint64_t t = __shfl_up_sync(FULL, S[k], 1);
            Sin[k] = lane == 0 ? 0 : t;
        }
        if constexpr (NW > 1) {
            if (lane == 31) {
#pragma unroll
                for (int k = 0; k <= KB; k++) sh->spill[w][k] = S[k];
            }
            __syncthreads();
            if (lane == 0 && w > 0) {
#pragma unroll
                for (int k = 0; k <= KB; k++) Sin[k] = sh->spill[w - 1][k];
            }
        }
        uint32_t g = chain_sub_gen<KB + 1>(X, [&](int k) { return Sin[k]; }, 0u);
        if (g) {   // rare: the borrow runs on through the lane
#pragma unroll
            for (int i = KB + 1; i < VPL; i++) {
                const uint64_t y = X[i];
                X[i] = y - g;
                g &= y == 0 ? 1u : 0u;
            }
        }
        const bool p = lane_is_zero<VPL>(*reinterpret_cast<const uint64_t(*)[VPL]>(&X[0]));
        // 4. lane-to-lane borrows
        const uint32_t A = __ballot_sync(FULL, g != 0 || p), Bm = __ballot_sync(FULL, g != 0);
        uint32_t cin = 0, cout;
        uint64_t tv;
        if constexpr (NW > 1) {
            if (lane == 0)
                sh->gp[w] = (uint32_t)(((uint64_t)A + Bm) >> 32) | ((uint32_t)(((uint64_t)A + Bm + 1) >> 32) << 1);
            if (top) sh->tv = tl;
            __syncthreads();
            uint32_t c = 0;
#pragma unroll
            for (int x = 0; x < NW; x++) {
                if (x == w) cin = c;
                c = (sh->gp[x] >> c) & 1u;
            }
            cout = c;
            tv = sh->tv;
        } else {
            cout = (uint32_t)(((uint64_t)A + Bm) >> 32);
            tv = __shfl_sync(FULL, tl, 31);
        }
        {
            const uint64_t sum = (uint64_t)A + Bm + cin;
            const uint32_t bin = (uint32_t)(((sum ^ A ^ Bm) >> lane) & 1u);
            lane_borrow_in<VPL>(*reinterpret_cast<uint64_t(*)[VPL]>(&X[0]), bin);
        }
        if (tv != (uint64_t)cout) {   // the window went negative: Q-hat was one too large (rare)
            uint32_t br = 1;
#pragma unroll
            for (int k = 0; k < KB; k++) {
                const uint64_t y = Q[k];
                Q[k] = y - br;
                br &= y == 0 ? 1u : 0u;
            }
            uint64_t cy = 0;
            bool allo = true;
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t x = X[i] + D[i];
                const uint64_t c1 = x < D[i] ? 1 : 0;
                const uint64_t y = x + cy;
                cy = c1 | (y < x ? 1 : 0);
                X[i] = y;
                allo &= y == ~0ull;
            }
            const uint32_t A2 = __ballot_sync(FULL, cy != 0 || allo), B2 = __ballot_sync(FULL, cy != 0);
            uint32_t cin2 = 0;
            if constexpr (NW > 1) {
                if (lane == 0)
                    sh->gp2[w] =
                        (uint32_t)(((uint64_t)A2 + B2) >> 32) | ((uint32_t)(((uint64_t)A2 + B2 + 1) >> 32) << 1);
                __syncthreads();
                uint32_t c = 0;
#pragma unroll
                for (int x = 0; x < NW; x++) {
                    if (x == w) cin2 = c;
                    c = (sh->gp2[x] >> c) & 1u;
                }
            }
            const uint64_t sum = (uint64_t)A2 + B2 + cin2;
            uint64_t ci = ((sum ^ A2 ^ B2) >> lane) & 1u;
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t y = X[i];
                X[i] = y + ci;
                ci &= y == ~0ull ? 1u : 0u;
            }
        }
        // 5. the block's quotient limbs (the top pad limbs of the first block are zero)
        if (top) {
            const int qb = nq + pad - (b + 1) * KB;
#pragma unroll
            for (int k = 0; k < KB; k++)
                if (qb + k < nq) store_q((uint32_t)(qb + k), Q[k]);
        }
        // 6. slide the window up KB limbs; KB dividend limbs enter at the bottom
        if (b + 1 < nblk) {
            uint64_t up[KB];
#pragma unroll
            for (int i = 0; i < KB; i++) up[i] = __shfl_up_sync(FULL, X[VPL - KB + i], 1);
            if constexpr (NW > 1) {
                if (lane == 31) {
#pragma unroll
                    for (int i = 0; i < KB; i++) sh->slide[w][i] = X[VPL - KB + i];
                }
            }
            uint64_t nw[KB];
            if (w == 0) {   // elements b KB .. b KB + KB - 1; element b KB + KB - 1 - i goes to position i
                const int c0 = (b * KB) & 31;
#pragma unroll
                for (int i = 0; i < KB; i++) nw[i] = __shfl_sync(FULL, chunk, c0 + KB - 1 - i);
                if ((((b + 1) * KB) & 31) == 0) {
                    chunk = chunk_next;
                    chunk_next = shl(x0 - 1 - ((b + 1) * KB + 32) - lane);
                }
            }
#pragma unroll
            for (int i = VPL + KB - 1; i >= KB; i--) X[i] = X[i - KB];
#pragma unroll
            for (int i = 0; i < KB; i++) X[i] = lane != 0 ? up[i] : (w == 0 ? nw[i] : X[i]);
        }
    }
    // remainder: position p = gl VPL + i holds limb p of (r 2^s) B^zl
    {
        uint64_t above = __shfl_down_sync(FULL, X[0], 1);
        if constexpr (NW > 1) {
            if (lane == 0) sh->rnext[w] = X[0];
            __syncthreads();
            if (lane == 31) above = w + 1 < NW ? sh->rnext[w + 1] : 0;
        } else {
            if (lane == 31) above = 0;
        }
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const int j = gl * VPL + i - zl;
            const uint64_t hi = i + 1 < VPL ? X[i + 1 < VPL ? i + 1 : 0] : above;
            if (j >= 0 && j < (int)MV) store_r((uint32_t)j, (X[i] >> s) | ((hi << 1) << rs));
        }
    }
    for (uint32_t j = K + (uint32_t)gl; j < MV; j += NL) store_r(j, 0);
    for (uint32_t j = (uint32_t)nq + (uint32_t)gl; j < MU; j += NL) store_q(j, 0);
    if constexpr (NW > 1) __syncthreads();   // the shared area is the next division's
    return 0;
}


}  // namespace bi
