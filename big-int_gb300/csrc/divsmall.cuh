// divsmall.cuh -- division of one instance by one thread, for divisors of at
// most 16 64-bit limbs: schoolbook long division (Knuth, TAOCP vol. 2,
// 4.3.1, Algorithm D) with 3-by-2 quotient estimates (Moller and Granlund's
// reciprocals, divlimb.cuh).  The quotient and remainder of u / v are unique,
// so the results are the ones the shifted-inverse division (divcore.cuh, the
// reference's algorithm) gives; what changes is the cost.  Long division does
// (MU - K + 1) K limb products for a K-limb divisor, about one multiply's
// worth, where the shifted inverse does several multiplies' worth plus a
// barrier per block operation -- at these sizes the barriers and the CTA
// bookkeeping are the whole cost, and one thread per instance has none.
//
// Registers: the divisor D and the (MX + 1)-limb window of the running
// remainder are register arrays of compile-time size MX with compile-time
// indices only.  The divisor is right-aligned in D (its K limbs at the top,
// zeros below), which divides u B^(MX-K) by v B^(MX-K): the same quotient, a
// remainder scaled by B^(MX-K), with no index that depends on K.
#pragma once

#include "chain.cuh"
#include "divlimb.cuh"

namespace bi {

constexpr int DIV_THREAD_MAX_MV = 16;   // 64-bit divisor limbs handled by div_thread
constexpr int DIV_THREAD_CTA = 64;      // threads per CTA of the one-thread-per-instance kernels
constexpr int DIV_WARP_MAX_MV = 1024;   // 64-bit divisor limbs handled by div_warp
constexpr int DIV_WARP_CTA = 128;       // threads per CTA of the one-warp-per-instance kernels
constexpr int DIV_LONG_MAX_MV = 4096;   // 64-bit divisor limbs handled by long division (divblock.cuh above 128)
// Long division on lane groups or the shifted inverse on CTAs, for a batch
// of n instances with MV-limb divisors (64-bit limbs) on a GPU of `sms` SMs.
// Long division does fewer limb products but runs one quotient limb after
// another (0.4 to 1.5 us a limb), so with few instances one CTA per instance
// finishes sooner; past a few instances per SM the groups' throughput wins.
// Measured crossovers (dividend 2 MV limbs, GB300, the shapes div.cu
// launches): long division always up to 64 limbs (with few instances on one
// warp each: 152 divisions of 128/64 limbs take 29 us, the shifted inverse
// 40); above that once n exceeds 2, 3, 5 and 4 instances per SM for divisors
// up to 128, 256, 512 and 1024 limbs.
__host__ __device__ inline bool div_use_long(uint32_t MV, uint64_t n, int sms) {
    if (MV <= 64) return true;
    if (MV > (uint32_t)DIV_WARP_MAX_MV) return MV <= (uint32_t)DIV_LONG_MAX_MV;
    const uint64_t per_sm = MV <= 128 ? 2 : MV <= 256 ? 3 : MV <= 512 ? 5 : 4;
    return n > per_sm * (uint64_t)sms;
}

// Divisors of 17..128 limbs in a batch of at most DIV_SMALL_WARP_PER_SM
// instances an SM divide on one warp each (div_warp with 1, 2 or 4 limbs a
// lane) instead of sharing warps as lane groups: a warp's quotient limbs are
// shorter, and with so few instances the GPU has warps to spare.  Measured
// on GB300 (2m/m limbs; warps vs groups): 64/32, 152 divisions 15.3 vs 19.9
// us, 3040 of them 27.3 vs 22.6; 128/64, 152: 28.1 vs 44.0, 1520: 39.2 vs
// 44.2, 3040: 58.3 vs 53.8; 256/128, 760: 70.9 vs 80.3, 3040: 133.9 vs 128.2.
constexpr int DIV_SMALL_WARP_PER_SM = 10;
__host__ __device__ inline bool div_small_on_warps(uint32_t MV, uint64_t n, int sms) {
    return MV > (uint32_t)DIV_THREAD_MAX_MV && MV <= 128 && n <= (uint64_t)DIV_SMALL_WARP_PER_SM * (uint64_t)sms;
}

// Divisors of 9..16 limbs in a batch of at most DIV_SMALL_GROUP_PER_SM
// instances an SM run on 8-lane groups (div_group<2, 8>, four instances a
// warp) instead of one thread each: so few instances leave the GPU short of
// warps, and one thread's quotient limbs are long.  Measured on GB300 (32/16
// limbs): 4096 divisions 16.7 us on threads, 11.1 on groups; 16384 of them
// 19.1 us on threads, 26.1 on groups (a group does about three times a
// thread's work per instance).
constexpr int DIV_SMALL_GROUP_PER_SM = 48;
__host__ __device__ inline bool div_small_on_groups(uint32_t MV, uint64_t n, int sms) {
    return MV > 8 && MV <= (uint32_t)DIV_THREAD_MAX_MV && n <= (uint64_t)DIV_SMALL_GROUP_PER_SM * (uint64_t)sms;
}

// The quotient limb estimate of long division: floor((u2 B^2 + u1 B + u0) /
// (d1 B + d2)) capped at B - 1, from the top three limbs of the running
// remainder and the top two of the normalised divisor (v3 = recip_3by2(d1,
// d2, .)).  It is what Knuth's 2-by-1 trial quotient becomes after the
// q-hat * d2 test (TAOCP 4.3.1, step D3) -- at most one too large -- in one
// 3-by-2 division; the remainder's invariant keeps (u2, u1) <= (d1, d2), and
// equality means a quotient of B or more, capped.
__device__ __forceinline__ uint64_t qhat_3by2(uint64_t u2, uint64_t u1, uint64_t u0, uint64_t d1, uint64_t d2,
                                              uint64_t v3) {
    const uint64_t q = div_3by2(u2, u1, u0, d1, d2, v3);   // plain arithmetic whatever the inputs
    return (u2 > d1 || (u2 == d1 && u1 >= d2)) ? ~0ull : q;
}

// One instance: u (MU 64-bit limbs through load_u), v (MV <= MX limbs through
// load_v); writes MU quotient limbs and MV remainder limbs.  Returns the
// status: 0, or 1 when v == 0 (then q = r = 0).
template <int MX, typename LoadU, typename LoadV, typename StoreQ, typename StoreR>
__device__ __forceinline__ uint8_t div_thread(uint32_t MU, uint32_t MV, LoadU load_u, LoadV load_v, StoreQ store_q,
                                              StoreR store_r) {
    static_assert(MX >= 2, "the quotient estimate reads two divisor limbs");
    uint64_t D[MX];
#pragma unroll
    for (int k = 0; k < MX; k++) {
        const int i = k - (MX - (int)MV);
        D[k] = i >= 0 ? load_v((uint32_t)i) : 0;
    }
    // move the top nonzero limb to D[MX-1]: K = the divisor's precision
    int K = (int)MV;
    for (int z = 0; z < MX && D[MX - 1] == 0; z++) {
#pragma unroll
        for (int k = MX - 1; k > 0; k--) D[k] = D[k - 1];
        D[0] = 0;
        K--;
    }
    if (K <= 0) {
        for (uint32_t i = 0; i < MU; i++) store_q(i, 0);
        for (uint32_t i = 0; i < MV; i++) store_r(i, 0);
        return 1;
    }
    const int s = __clzll((long long)D[MX - 1]);
    const int rs = 63 - s;   // x >> (64 - s) written as (x >> 1) >> rs: 0 when s == 0
#pragma unroll
    for (int k = MX - 1; k > 0; k--) D[k] = (D[k] << s) | ((D[k - 1] >> 1) >> rs);
    D[0] <<= s;
    const int zl = MX - K;   // zero limbs below the divisor

    // the shifted dividend: sh(t) = limb t of u 2^s, t in [0, MU]
    auto raw = [&](int t) -> uint64_t { return (t >= 0 && t < (int)MU) ? load_u((uint32_t)t) : 0; };
    // window R[0..MX] = limbs MU - MX .. MU of u 2^s (zeros below limb 0)
    uint64_t R[MX + 1];
    uint64_t below = raw((int)MU - MX - 1);   // raw limb under the window
    {
        uint64_t prev = below;
#pragma unroll
        for (int k = 0; k <= MX; k++) {
            const uint64_t cur = raw((int)MU - MX + k);
            R[k] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    const uint64_t d1 = D[MX - 1], d2 = D[MX - 2];
    const uint64_t v3 = recip_3by2(d1, d2, recip_limb(d1));
    int tn = (int)MU - MX - 1;   // shifted-dividend limb that enters the window next
    for (int j = (int)MU - K; j >= 0; j--) {
        // the raw limb this step's slide needs, loaded first so that its
        // latency overlaps the step's arithmetic
        const uint64_t lower = j > 0 ? raw(tn - 1) : 0;
        const uint64_t u2 = R[MX], u1 = R[MX - 1], u0 = R[MX - 2];
        uint64_t qh = qhat_3by2(u2, u1, u0, d1, d2, v3);
        // R -= q-hat * D on the carry flag: the high halves one limb up (R[1..MX]),
        // then the low halves (R[0..MX-1], the borrow out taken from R[MX]);
        // the result is negative iff one of the two wrapped
        const uint32_t bA = chain_sub_from<MX>(*reinterpret_cast<uint64_t(*)[MX]>(&R[1]),
                                               [&](int k) { return __umul64hi(qh, D[k]); }, 0);
        const uint32_t bo = chain_sub_from<MX>(*reinterpret_cast<uint64_t(*)[MX]>(&R[0]),
                                               [&](int k) { return qh * D[k]; }, 0);
        const bool bB = R[MX] < bo;
        R[MX] -= bo;
        const bool borrow = bA != 0 || bB;
        if (borrow) {                          // one too large after all: add D back
            qh -= 1;
            uint64_t c = 0;
#pragma unroll
            for (int k = 0; k < MX; k++) {
                const uint64_t x = R[k] + D[k];
                const uint64_t c1 = x < D[k] ? 1 : 0;
                R[k] = x + c;
                c = c1 | (R[k] < x ? 1 : 0);
            }
            R[MX] += c;
        }
        store_q((uint32_t)j, qh);
        if (j > 0) {                           // slide the window down one limb
#pragma unroll
            for (int k = MX; k > 0; k--) R[k] = R[k - 1];
            R[0] = (below << s) | ((lower >> 1) >> rs);   // below = raw(tn)
            below = lower;
            tn--;
        }
    }
    for (uint32_t i = (uint32_t)((int)MU - K + 1); i < MU; i++) store_q(i, 0);
    // remainder: R[0..MX-1] = (r 2^s) B^zl
    for (int z = 0; z < zl; z++) {
#pragma unroll
        for (int k = 0; k < MX - 1; k++) R[k] = R[k + 1];
        R[MX - 1] = 0;
    }
#pragma unroll
    for (int k = 0; k < MX; k++) {
        const uint64_t hi = k + 1 < MX ? R[k + 1] : 0;
        const uint64_t x = (R[k] >> s) | ((hi << 1) << rs);
        if (k < (int)MV) store_r((uint32_t)k, x);
    }
    return 0;
}

// The lane's block is zero (the borrow chain's propagate bit): a random block
// almost never is, and its first and last limbs settle that; the OR of all
// limbs only when both are zero.
template <int VPL>
__device__ __forceinline__ bool lane_is_zero(const uint64_t (&R)[VPL]) {
    if ((R[0] | R[VPL - 1]) != 0) return false;
    uint64_t o = 0;
#pragma unroll
    for (int i = 0; i < VPL; i++) o |= R[i];
    return o == 0;
}

// R -= bin (0 or 1) over a lane's block: the borrow stops at R[0] unless
// R[0] was zero, so the chain through the other limbs is a rare branch.
template <int VPL>
__device__ __forceinline__ void lane_borrow_in(uint64_t (&R)[VPL], uint32_t bin) {
    const uint64_t y0 = R[0];
    R[0] = y0 - bin;
    if (bin && y0 == 0) {
        uint64_t b = 1;
#pragma unroll
        for (int i = 1; i < VPL; i++) {
            const uint64_t y = R[i];
            R[i] = y - b;
            b &= y == 0 ? 1 : 0;
        }
    }
}

// Borrow (or carry) into this lane of a warp-wide chain, from each lane's
// generate g (out with nothing in) and propagate p (out only with one in):
// bit l of (A + B) ^ A ^ B with A = ballot(g | p), B = ballot(g).  cout gets
// the borrow out of lane 31.
__device__ __forceinline__ uint64_t warp_chain_in(bool g, bool p, uint64_t& cout) {
    const uint32_t A = __ballot_sync(0xffffffffu, g || p), Bm = __ballot_sync(0xffffffffu, g);
    const uint64_t s = (uint64_t)A + Bm;
    cout = s >> 32;
    return ((s ^ A ^ Bm) >> (threadIdx.x & 31)) & 1u;
}

// One instance on one warp (all 32 lanes call with the same arguments): the
// long division of div_thread with the divisor and the window spread over
// the lanes, VPL limbs each (lane l holds positions l VPL .. l VPL + VPL - 1,
// MX = 32 VPL), the top window limb R[MX] uniform in every lane.  Each
// quotient limb costs the uniform 3-by-2 estimate, two in-lane borrow chains
// (the high halves of q-hat D, then the low halves) resolved across lanes by
// two ballots each, and a one-limb slide; the dividend streams in through a
// 32-limb buffer loaded by the whole warp every 32 quotient limbs.
template <int VPL, typename LoadU, typename LoadV, typename StoreQ, typename StoreR>
__device__ __forceinline__ uint8_t div_warp(uint32_t MU, uint32_t MV, LoadU load_u, LoadV load_v, StoreQ store_q,
                                            StoreR store_r) {
    constexpr int MX = 32 * VPL;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31);
    uint64_t D[VPL];
#pragma unroll
    for (int i = 0; i < VPL; i++) {
        const int idx = lane * VPL + i - (MX - (int)MV);
        D[i] = idx >= 0 ? load_v((uint32_t)idx) : 0;
    }
    int top_i = -1;
#pragma unroll
    for (int i = 0; i < VPL; i++)
        if (D[i] != 0) top_i = i;
    const uint32_t nz = __ballot_sync(FULL, top_i >= 0);
    if (nz == 0) {
        for (uint32_t i = lane; i < MU; i += 32) store_q(i, 0);
        for (uint32_t i = lane; i < MV; i += 32) store_r(i, 0);
        return 1;
    }
    const int tl = 31 - __clz((int)nz);
    const int ptop = tl * VPL + __shfl_sync(FULL, top_i, tl);   // top nonzero position
    const int K = ptop - (MX - (int)MV) + 1;
    const int zl = MX - K;
    for (int z = ptop; z < MX - 1; z++) {                      // one-limb shifts up
        const uint64_t from_below = __shfl_up_sync(FULL, D[VPL - 1], 1);
#pragma unroll
        for (int i = VPL - 1; i > 0; i--) D[i] = D[i - 1];
        D[0] = lane == 0 ? 0 : from_below;
    }
    const int s = __clzll((long long)__shfl_sync(FULL, D[VPL - 1], 31));
    const int rs = 63 - s;   // x >> (64 - s) written as (x >> 1) >> rs: 0 when s == 0
    {
        const uint64_t below = __shfl_up_sync(FULL, D[VPL - 1], 1);
        uint64_t prev = lane == 0 ? 0 : below;
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t cur = D[i];
            D[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    const uint64_t d1 = __shfl_sync(FULL, D[VPL - 1], 31);
    const uint64_t d2 = VPL >= 2 ? __shfl_sync(FULL, D[VPL >= 2 ? VPL - 2 : 0], 31) : __shfl_sync(FULL, D[0], 30);
    auto Dv = [&](int i) -> uint64_t { return D[i]; };
    const uint64_t v3 = recip_3by2(d1, d2, recip_limb(d1));

    // the shifted dividend: sh(t) = limb t of u 2^s, t in [0, MU]
    auto raw = [&](int t) -> uint64_t { return (t >= 0 && t < (int)MU) ? load_u((uint32_t)t) : 0; };
    auto sh = [&](int t) -> uint64_t { return (raw(t) << s) | ((raw(t - 1) >> 1) >> rs); };
    // window positions 0..MX-1 = limbs MU - MX .. MU - 1 of u 2^s, R[MX] = limb MU
    uint64_t R[VPL];
    {
        const int t0 = (int)MU - MX + lane * VPL;
        uint64_t prev = raw(t0 - 1);
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t cur = raw(t0 + i);
            R[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    uint64_t rtop = (raw((int)MU - 1) >> 1) >> rs;
    // stream buffer: lane l holds sh(base - l); limb c of it enters at the c-th slide
    int base = (int)MU - MX - 1, c = 0;
    uint64_t shb = sh(base - lane);
    for (int j = (int)MU - K; j >= 0; j--) {
        const uint64_t u2 = rtop;
        const uint64_t u1 = __shfl_sync(FULL, R[VPL - 1], 31);
        const uint64_t u0 = VPL >= 2 ? __shfl_sync(FULL, R[VPL >= 2 ? VPL - 2 : 0], 31) : __shfl_sync(FULL, R[0], 30);
        uint64_t qh = qhat_3by2(u2, u1, u0, d1, d2, v3);
        // pass A: R -= (high halves of q-hat D) shifted up one position, in
        // lane, borrows across lanes resolved by two ballots; the borrow into
        // each lane is applied by pass B's chain
        uint64_t coutA, coutB;
        bool neg;
        {
            const uint64_t htop = __umul64hi(qh, Dv(VPL - 1));
            const uint64_t hb = __shfl_up_sync(FULL, htop, 1);
            const uint64_t h0 = lane == 0 ? 0 : hb;
            const uint32_t gA = chain_sub_from<VPL>(
                R, [&](int i) { return i == 0 ? h0 : __umul64hi(qh, Dv(i > 0 ? i - 1 : 0)); }, 0);
            const bool zA = lane_is_zero<VPL>(R);
            const uint32_t binA = (uint32_t)warp_chain_in(gA != 0, zA, coutA);
            const uint64_t th = __shfl_sync(FULL, htop, 31);
            const uint64_t x = rtop - th;
            const bool bA = (rtop < th) || (x < coutA);
            rtop = x - coutA;
            // pass B: R -= low halves of q-hat D and the borrow from pass A;
            // a lane of zeros that took A's borrow wrapped to all ones, which
            // A's ballots already carried on, so it generates no B borrow
            const uint32_t gB = chain_sub_from<VPL>(R, [&](int i) { return qh * Dv(i); }, binA) &
                                (zA && binA ? 0u : 1u);
            const bool zB = lane_is_zero<VPL>(R);
            uint32_t bin = (uint32_t)warp_chain_in(gB != 0, zB, coutB);
            lane_borrow_in<VPL>(R, bin);
            const bool bB = rtop < coutB;
            rtop -= coutB;
            neg = bA || bB;                    // at most one of the two wraps
        }
        if (neg) {                             // one too large after all: add D back
            qh -= 1;
            uint64_t cy = 0;
            bool allo = true;
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t di = Dv(i);
                const uint64_t x = R[i] + di;
                const uint64_t c1 = x < di ? 1 : 0;
                const uint64_t y = x + cy;
                cy = c1 | (y < x ? 1 : 0);
                R[i] = y;
                allo &= y == ~0ull;
            }
            uint64_t cout;
            uint64_t cin = warp_chain_in(cy != 0, allo, cout);
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t y = R[i];
                R[i] = y + cin;
                cin &= y == ~0ull ? 1 : 0;
            }
            rtop += cout;
        }
        if (lane == 0) store_q((uint32_t)j, qh);
        if (j > 0) {                           // slide the window down one limb
            const uint64_t next = __shfl_sync(FULL, shb, c);
            rtop = __shfl_sync(FULL, R[VPL - 1], 31);
            const uint64_t from_below = __shfl_up_sync(FULL, R[VPL - 1], 1);
#pragma unroll
            for (int i = VPL - 1; i > 0; i--) R[i] = R[i - 1];
            R[0] = lane == 0 ? next : from_below;
            if (++c == 32) {
                base -= 32;
                c = 0;
                shb = sh(base - lane);
            }
        }
    }
    for (uint32_t i = (uint32_t)((int)MU - K + 1) + lane; i < MU; i += 32) store_q(i, 0);
    // remainder: positions 0..MX-1 hold (r 2^s) B^zl
    for (int z = 0; z < zl; z++) {
        const uint64_t from_above = __shfl_down_sync(FULL, R[0], 1);
#pragma unroll
        for (int i = 0; i < VPL - 1; i++) R[i] = R[i + 1];
        R[VPL - 1] = lane == 31 ? 0 : from_above;
    }
    {
        const uint64_t ab = __shfl_down_sync(FULL, R[0], 1);
        const uint64_t above = lane == 31 ? 0 : ab;
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t hi = i + 1 < VPL ? R[i + 1 < VPL ? i + 1 : 0] : above;
            const uint64_t x = (R[i] >> s) | ((hi << 1) << rs);
            const int p = lane * VPL + i;
            if (p < (int)MV) store_r((uint32_t)p, x);
        }
    }
    return 0;
}

// Carry (or borrow) into this lane of a chain over a G-lane group (lanes
// gbase .. gbase + G - 1 of the warp), as warp_chain_in; cout = out of the
// group's top lane.  Every lane of the warp calls it.
template <int G>
__device__ __forceinline__ uint64_t group_chain_in(bool g, bool p, uint64_t& cout) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gbase = lane & ~(uint32_t)(G - 1), r = lane & (G - 1);
    const uint32_t Aw = __ballot_sync(0xffffffffu, g || p), Bw = __ballot_sync(0xffffffffu, g);
    const uint64_t gm = G == 32 ? 0xffffffffull : ((1ull << G) - 1);
    const uint64_t A = (Aw >> gbase) & gm, B = (Bw >> gbase) & gm;
    const uint64_t s = A + B;
    cout = (s >> G) & 1u;
    return ((s ^ A ^ B) >> r) & 1u;
}

// div_warp on a G-lane group (G = 8, 16 or 32), 32 / G instances a warp: the
// steps of a quotient limb whose cost does not grow with the divisor -- the
// estimate, the ballots, the shuffles, the slide -- are shared by the warp's
// instances, so small and medium divisors (where they are most of the work)
// divide several times faster per instance.  All 32 lanes call it; each
// group passes its own instance (valid = false: no instance, nothing read or
// written).  Loops whose trip count differs between groups run to the warp's
// maximum with the work of the finished (or not yet started) groups masked:
// the quotient loop is aligned at its end, a group's first quotient limb
// waiting for the warp's longest; a group that is not yet active uses
// q-hat = 0, which leaves its window as it is.  Returns the status as
// div_warp does.
template <int VPL, int G, typename LoadU, typename LoadV, typename StoreQ, typename StoreR>
__device__ __forceinline__ uint8_t div_group(bool valid, uint32_t MU, uint32_t MV, LoadU load_u, LoadV load_v,
                                             StoreQ store_q, StoreR store_r) {
    static_assert(G == 8 || G == 16 || G == 32, "div_group: G is 8, 16 or 32");
    constexpr int MX = G * VPL;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = (int)(threadIdx.x & 31);
    const int r = lane & (G - 1);
    const uint32_t gbase = (uint32_t)(lane & ~(G - 1));
    const uint32_t gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << gbase);
    uint64_t D[VPL];
#pragma unroll
    for (int i = 0; i < VPL; i++) {
        const int idx = r * VPL + i - (MX - (int)MV);
        D[i] = (valid && idx >= 0) ? load_v((uint32_t)idx) : 0;
    }
    int top_i = -1;
#pragma unroll
    for (int i = 0; i < VPL; i++)
        if (D[i] != 0) top_i = i;
    const uint32_t nz = __ballot_sync(FULL, top_i >= 0) & gmask;
    const bool zero = nz == 0;                       // a zero divisor, or no instance
    const int tl = zero ? 0 : 31 - __clz((int)nz) - (int)gbase;
    const int ti = __shfl_sync(FULL, top_i, tl, G);
    const int ptop = zero ? MX - 1 : tl * VPL + ti;  // top nonzero position
    const int K = zero ? (int)MU + 1 : ptop - (MX - (int)MV) + 1;
    const int zl = zero ? 0 : MX - K;
    {
        const int nsh = MX - 1 - ptop;               // one-limb shifts up
        const int nsh_max = (int)__reduce_max_sync(FULL, (unsigned)nsh);
        for (int z = 0; z < nsh_max; z++) {
            const uint64_t from_below = __shfl_up_sync(FULL, D[VPL - 1], 1, G);
            if (z < nsh) {
#pragma unroll
                for (int i = VPL - 1; i > 0; i--) D[i] = D[i - 1];
                D[0] = r == 0 ? 0 : from_below;
            }
        }
    }
    const uint64_t dtop = __shfl_sync(FULL, D[VPL - 1], G - 1, G);
    const int s = zero ? 0 : __clzll((long long)dtop);
    const int rs = 63 - s;   // x >> (64 - s) written as (x >> 1) >> rs: 0 when s == 0
    {
        const uint64_t below = __shfl_up_sync(FULL, D[VPL - 1], 1, G);
        uint64_t prev = r == 0 ? 0 : below;
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t cur = D[i];
            D[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    const uint64_t d1 = __shfl_sync(FULL, D[VPL - 1], G - 1, G);
    const uint64_t d2 = VPL >= 2 ? __shfl_sync(FULL, D[VPL >= 2 ? VPL - 2 : 0], G - 1, G)
                                 : __shfl_sync(FULL, D[0], G - 2, G);
    const uint64_t d1n = zero ? (1ull << 63) : d1;   // a group without a division gets a normalised stand-in
    const uint64_t v3 = recip_3by2(d1n, zero ? 0 : d2, recip_limb(d1n));

    auto raw = [&](int t) -> uint64_t { return (valid && t >= 0 && t < (int)MU) ? load_u((uint32_t)t) : 0; };
    auto sh = [&](int t) -> uint64_t { return (raw(t) << s) | ((raw(t - 1) >> 1) >> rs); };
    uint64_t R[VPL];
    {
        const int t0 = (int)MU - MX + r * VPL;
        uint64_t prev = raw(t0 - 1);
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t cur = raw(t0 + i);
            R[i] = (cur << s) | ((prev >> 1) >> rs);
            prev = cur;
        }
    }
    uint64_t rtop = (raw((int)MU - 1) >> 1) >> rs;
    int base = (int)MU - MX - 1, c = 0;   // stream buffer: rank r holds sh(base - r)
    uint64_t shb = sh(base - r);
    const int nsteps = zero ? 0 : (int)MU - K + 1;
    const int nmax = (int)__reduce_max_sync(FULL, (unsigned)nsteps);
    for (int j = nmax - 1; j >= 0; j--) {            // this group's quotient limb j while j < nsteps
        const bool act = j < nsteps;
        const uint64_t u2 = rtop;
        const uint64_t u1 = __shfl_sync(FULL, R[VPL - 1], G - 1, G);
        const uint64_t u0 = VPL >= 2 ? __shfl_sync(FULL, R[VPL >= 2 ? VPL - 2 : 0], G - 1, G)
                                     : __shfl_sync(FULL, R[0], G - 2, G);
        uint64_t qh = act ? qhat_3by2(u2, u1, u0, d1, d2, v3) : 0;
        // R -= q-hat D in two passes as div_warp (q-hat = 0 leaves R as it is)
        uint64_t coutA, coutB;
        bool neg;
        {
            const uint64_t htop = __umul64hi(qh, D[VPL - 1]);
            const uint64_t hb = __shfl_up_sync(FULL, htop, 1, G);
            const uint64_t h0 = r == 0 ? 0 : hb;
            const uint32_t gA = chain_sub_from<VPL>(
                R, [&](int i) { return i == 0 ? h0 : __umul64hi(qh, D[i > 0 ? i - 1 : 0]); }, 0);
            const bool zA = lane_is_zero<VPL>(R);
            const uint32_t binA = (uint32_t)group_chain_in<G>(gA != 0, zA, coutA);
            const uint64_t th = __shfl_sync(FULL, htop, G - 1, G);
            const uint64_t x = rtop - th;
            const bool bA = (rtop < th) || (x < coutA);
            rtop = x - coutA;
            const uint32_t gB = chain_sub_from<VPL>(R, [&](int i) { return qh * D[i]; }, binA) &
                                (zA && binA ? 0u : 1u);
            const bool zB = lane_is_zero<VPL>(R);
            const uint32_t bin = (uint32_t)group_chain_in<G>(gB != 0, zB, coutB);
            lane_borrow_in<VPL>(R, bin);
            const bool bB = rtop < coutB;
            rtop -= coutB;
            neg = bA || bB;
        }
        if (__any_sync(FULL, neg)) {                 // rare: add D back where q-hat was one too large
            if (neg) qh -= 1;
            uint64_t cy = 0;
            bool allo = true;
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t di = neg ? D[i] : 0;
                const uint64_t x = R[i] + di;
                const uint64_t c1 = x < di ? 1 : 0;
                const uint64_t y = x + cy;
                cy = c1 | (y < x ? 1 : 0);
                R[i] = y;
                allo &= y == ~0ull;
            }
            uint64_t cout;
            uint64_t cin = group_chain_in<G>(cy != 0, allo && neg, cout);
#pragma unroll
            for (int i = 0; i < VPL; i++) {
                const uint64_t y = R[i];
                R[i] = y + cin;
                cin &= y == ~0ull ? 1 : 0;
            }
            rtop += cout;
        }
        if (act && r == 0) store_q((uint32_t)j, qh);
        if (j > 0) {                                 // slide the window down one limb (active groups)
            const uint64_t next = __shfl_sync(FULL, shb, c, G);
            const uint64_t newtop = __shfl_sync(FULL, R[VPL - 1], G - 1, G);
            const uint64_t from_below = __shfl_up_sync(FULL, R[VPL - 1], 1, G);
            if (act) {
                rtop = newtop;
#pragma unroll
                for (int i = VPL - 1; i > 0; i--) R[i] = R[i - 1];
                R[0] = r == 0 ? next : from_below;
                if (++c == G) {
                    base -= G;
                    c = 0;
                    shb = sh(base - r);
                }
            }
        }
    }
    if (valid)
        for (uint32_t i = (uint32_t)((int)MU - K + 1) + (uint32_t)r; i < MU; i += G) store_q(i, 0);
    // remainder: positions 0..MX-1 hold (r 2^s) B^zl
    {
        const int zl_max = (int)__reduce_max_sync(FULL, (unsigned)zl);
        for (int z = 0; z < zl_max; z++) {
            const uint64_t from_above = __shfl_down_sync(FULL, R[0], 1, G);
            if (z < zl) {
#pragma unroll
                for (int i = 0; i < VPL - 1; i++) R[i] = R[i + 1];
                R[VPL - 1] = r == G - 1 ? 0 : from_above;
            }
        }
    }
    {
        const uint64_t ab = __shfl_down_sync(FULL, R[0], 1, G);
        const uint64_t above = r == G - 1 ? 0 : ab;
#pragma unroll
        for (int i = 0; i < VPL; i++) {
            const uint64_t hi = i + 1 < VPL ? R[i + 1 < VPL ? i + 1 : 0] : above;
            const uint64_t x = zero ? 0 : (R[i] >> s) | ((hi << 1) << rs);
            const int p = r * VPL + i;
            if (valid && p < (int)MV) store_r((uint32_t)p, x);
        }
    }
    return zero ? 1 : 0;
}

}  // namespace bi
