// mulwarp.cuh -- the warp-level full product of small operands on 32-bit
// words, shared by the uniform multiply (mul.cu) and the uneven batch
// (batch.cu): G lanes per instance (several instances per warp when G < 32), operands padded to
// M = 2G words in the warp's shared memory (b twice over, so that
// b[(c - i) mod M] is at a compile-time offset from a per-lane base), no
// CTA barrier.  The library routes full products of at most 64 32-bit words
// (32 64-bit limbs) here, for both limb types, and the uneven batch its
// small full products when its tuning says so.
//
// Lane t accumulates four product columns as 3-word sums: 2t and 2t + M
// (pair A: term a_i b_((2t - i) mod M) belongs to column 2t for i <= 2t and
// to column 2t + M above) and 2t + 1, 2t + 1 + M (pair B, likewise) -- M
// terms a pair, the same in every lane.  A term is three instructions,
// mad.lo.cc / madc.hi.cc / addc on the integer multiply-add pipe with the
// carry flag; each pair runs one accumulator over all M terms and a snapshot
// at i = 2t (2t + 1) splits it into the low column (the snapshot) and the
// high one (the rest).  Operands come two words a load: a_i, a_(i+1) are
// one broadcast 64-bit load, and b's two words for pairs A and B are one
// 64-bit load at the lane's base.  The columns then fold into 64-bit limbs:
// lane t's columns 2t and 2t + 1 make the value v0 + v1 B at limb t
// (B = 2^64, v1 < 2^39), likewise at limb t + G, and limb p of the product
// is v0_p + v1_(p-1) with the carries resolved by ballots in the instance.
#pragma once

#include "common.cuh"

namespace bi {

// (c0, c1, c2) += x * y over 32-bit words, carries in the condition code
__device__ __forceinline__ void mac3w(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t x, uint32_t y) {
    asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\tmadc.hi.cc.u32 %1, %3, %4, %1;\n\taddc.u32 %2, %2, 0;"
        : "+r"(c0), "+r"(c1), "+r"(c2)
        : "r"(x), "r"(y));
}

// carry into lane t of a G-lane group (lanes base..base+G-1) for per-lane
// (generate, propagate) and carry-in cin; cout = carry out of the group
__device__ __forceinline__ uint32_t group_carry(uint32_t g, uint32_t p, uint32_t cin, uint32_t G, uint32_t base,
                                                uint32_t t, uint32_t& cout) {
    const uint32_t Aw = __ballot_sync(0xffffffffu, g | p), Bw = __ballot_sync(0xffffffffu, g);
    const uint64_t gm = G == 32 ? 0xffffffffull : ((1ull << G) - 1);
    const uint64_t A = (Aw >> base) & gm, B = (Bw >> base) & gm;
    const uint64_t s = A + B + cin;
    cout = (uint32_t)(s >> G) & 1u;
    return (uint32_t)((s ^ A ^ B) >> t) & 1u;
}


// Small CTAs (4 warps): a batch that fills one wave spreads within a warp or
// so of evenly over the SMs.
constexpr int MUL_WARP_CTA = 128;

// Shared memory of one G-lane group: a (2G words), then b twice (4G words).
template <int G>
__host__ __device__ constexpr uint32_t mul_warp_group_words() { return 3 * 2 * G; }

// One full product on the G lanes base .. base + G - 1 of the warp (t = the
// lane's index in the group); every lane of the warp calls it, each group
// with its own instance (or none: a group with nothing to do loads zeros and
// stores nothing).  sw: the group's mul_warp_group_words<G>() words of
// shared memory.  load(x, wa, wb) gives the 32-bit words x of a and b for
// x < 2G (zero past the operands); store(c, v) receives 64-bit limb c of the
// 4G-word product, c < 2G.
template <int G, typename Load, typename Store>
__device__ __forceinline__ void mul_warp_group(uint32_t* sw, uint32_t t, uint32_t base, Load load, Store store) {
    constexpr uint32_t M = 2 * G;                      // padded words per operand
    uint32_t* sa = sw;
    uint32_t* sb = sw + M;
    {
        const uint32_t x0 = 2 * t, x1 = 2 * t + 1;
        uint32_t a0, a1, b0, b1;
        load(x0, a0, b0);
        load(x1, a1, b1);
        sa[x0] = a0;
        sa[x1] = a1;
        sb[x0] = b0;
        sb[x1] = b1;
        sb[x0 + M] = b0;
        sb[x1 + M] = b1;
    }
    __syncwarp();
    uint32_t A0 = 0, A1 = 0, A2 = 0, B0 = 0, B1 = 0, B2 = 0;
    uint32_t SA0 = 0, SA1 = 0, SA2 = 0, SB0 = 0, SB1 = 0, SB2 = 0;
    // pair A reads b[(2t - i) mod M] = sb[M + 2t - i], pair B the word above
    const uint32_t* bp = sb + M + 2 * t;
#pragma unroll
    for (int k = 0; k < (int)G; k++) {
        const int i = 2 * k;
        const uint2 av = *reinterpret_cast<const uint2*>(sa + i);        // a_i, a_(i+1)
        const uint2 bv = *reinterpret_cast<const uint2*>(bp - i);        // b for A at i, b for B at i
        // i: A takes b[2t - i], B takes b[2t + 1 - i]
        mac3w(A0, A1, A2, av.x, bv.x);
        mac3w(B0, B1, B2, av.x, bv.y);
        const bool snap = k == (int)t;
        if (snap) { SA0 = A0; SA1 = A1; SA2 = A2; }
        // i + 1: A takes b[2t - i - 1], B takes b[2t - i] (= bv.x)
        const uint32_t bA1 = bp[-i - 1];
        mac3w(A0, A1, A2, av.y, bA1);
        mac3w(B0, B1, B2, av.y, bv.x);
        if (snap) { SB0 = B0; SB1 = B1; SB2 = B2; }
    }
    __syncwarp();   // the shared operands are rewritten by the next round
    // high columns: the rest after the snapshots
    uint32_t HA0, HA1, HA2, HB0, HB1, HB2;
    asm("sub.cc.u32 %0, %3, %6;\n\tsubc.cc.u32 %1, %4, %7;\n\tsubc.u32 %2, %5, %8;"
        : "=r"(HA0), "=r"(HA1), "=r"(HA2)
        : "r"(A0), "r"(A1), "r"(A2), "r"(SA0), "r"(SA1), "r"(SA2));
    asm("sub.cc.u32 %0, %3, %6;\n\tsubc.cc.u32 %1, %4, %7;\n\tsubc.u32 %2, %5, %8;"
        : "=r"(HB0), "=r"(HB1), "=r"(HB2)
        : "r"(B0), "r"(B1), "r"(B2), "r"(SB0), "r"(SB1), "r"(SB2));
    // limb value v0 + v1 B from columns (x0, x1, x2) and (y0, y1, y2) one word apart
    auto limb = [](uint32_t x0, uint32_t x1, uint32_t x2, uint32_t y0, uint32_t y1, uint32_t y2, uint64_t& v1) {
        const uint64_t lo = ((uint64_t)x1 << 32) | x0;
        const uint64_t add = (uint64_t)y0 << 32;
        const uint64_t v0 = lo + add;
        v1 = (uint64_t)x2 + (((uint64_t)y2 << 32) | y1) + (v0 < add ? 1 : 0);
        return v0;
    };
    uint64_t v1r[2], v0r[2];
    v0r[0] = limb(SA0, SA1, SA2, SB0, SB1, SB2, v1r[0]);
    v0r[1] = limb(HA0, HA1, HA2, HB0, HB1, HB2, v1r[1]);
    // fold: row jj holds limb G jj + t
    uint32_t cy = 0;
    uint64_t prev = 0;   // v1 of the limb below this row's first
#pragma unroll
    for (int jj = 0; jj < 2; jj++) {
        uint64_t s1 = __shfl_up_sync(0xffffffffu, v1r[jj], 1, G);
        if (t == 0) s1 = prev;
        prev = __shfl_sync(0xffffffffu, v1r[jj], base + G - 1);
        const uint64_t y = v0r[jj] + s1;
        uint32_t co;
        const uint32_t k1 = group_carry(y < s1, y == ~0ull, cy, G, base, t, co);
        cy = co;
        store((uint32_t)(G * jj) + t, y + k1);
    }
}

}  // namespace bi
