// mulcore.cuh -- the CTA-level classical multiply shared by the uniform
// batch kernel (mul.cu) and the uneven-batch kernel (batch.cu).  See mul.cu
// for the design.
#pragma once

#include "blockops.cuh"   // row_mac8, block_carry_in

namespace bi {

constexpr int MUL_C = 8;

// skewed shared-memory position of limb x: 2 limbs of padding after every C
template <int C>
__device__ __forceinline__ uint32_t skew(uint32_t x) {
    return x + 2 * (x / C);
}

__device__ __forceinline__ void lds128(const uint64_t* p, uint64_t& x, uint64_t& y) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
    x = v.x;
    y = v.y;
}

struct MulGeom {
    uint32_t L;      // limbs per operand in the u64 view
    uint32_t Lp;     // L rounded up to a multiple of 2C
    uint32_t tpi;    // threads per instance
    uint32_t ipc;    // instances per CTA
    uint32_t SA;     // skewed span of a_s (limbs)
    uint32_t IS;     // per-instance shared-memory stride (limbs)
    uint32_t m;      // limbs per operand in the caller's type
    uint32_t out_limbs;   // result limbs per instance in the u64 view
    uint32_t out_words;   // result limbs per instance in the caller's type
    uint32_t S, lgS;      // slices per thread's rows (a power of two; 1 = none)
};

// The CTA-level multiply of g.ipc instances held in shared memory.  `load`
// supplies limb x of instance li's operands (zero past the operand), `store`
// receives limb x of instance li's result for x < g.out_limbs.  Every thread
// of the CTA calls it; it ends with the CTA synchronised.  The caller
// provides g.ipc * g.IS limbs of shared memory and 96 words of scratch.
//
// With g.S > 1 each window pair's rows are cut into S slices run by S
// consecutive lanes, whose partial windows are summed with warp shuffles
// before the merge: shorter serial carry chains for one instance that has a
// whole CTA to itself (the serving loop); the extra lanes pass carries
// through unchanged in the merge's lookahead.
template <int C, typename Load, typename Store>
__device__ __forceinline__ void mul_cta(const MulGeom& g, uint64_t* smem, uint32_t* scratch,
                                        const FastDiv& lpdiv, Load load, Store store) {
    const uint32_t tid = threadIdx.x;
    const uint32_t Lp = g.Lp;
    const uint32_t nwin_half = Lp / C;      // windows in one half of the product

    // ---- stage operands: a_s[x], b_s[x + C] (zero padded), per instance
    {
        // U limbs a thread in flight: all U loads issue before the first
        // shared-memory store waits on one
        constexpr int U = 4;
        const uint32_t total = g.ipc * Lp, step = blockDim.x;
        for (uint32_t idx0 = tid; idx0 < total; idx0 += U * step) {
            uint64_t va[U], vb[U];
            uint32_t li[U], x[U];
#pragma unroll
            for (int k = 0; k < U; k++) {
                const uint32_t idx = idx0 + k * step;
                li[k] = lpdiv.div(idx);
                x[k] = idx - li[k] * Lp;
                va[k] = 0;
                vb[k] = 0;
                if (idx < total && x[k] < g.L) load(li[k], x[k], va[k], vb[k]);
            }
#pragma unroll
            for (int k = 0; k < U; k++) {
                if (idx0 + k * step < total) {
                    uint64_t* base = smem + (size_t)li[k] * g.IS;
                    base[skew<C>(x[k])] = va[k];
                    base[g.SA + skew<C>(x[k] + C)] = vb[k];
                }
            }
        }
        // zero pads of b_s: logical [0, C) and [Lp + C, Lp + 2C)
        for (uint32_t idx = tid; idx < g.ipc * 2 * C; idx += blockDim.x) {
            const uint32_t li = idx / (2 * C), q = idx % (2 * C);
            const uint32_t y = q < C ? q : Lp + q;
            smem[(size_t)li * g.IS + g.SA + skew<C>(y)] = 0;
        }
    }
    __syncthreads();

    const uint32_t grp = tid >> g.lgS;            // (instance, rank) group of S lanes
    const uint32_t sl = tid & (g.S - 1);          // slice within the group
    const uint32_t li = grp / g.tpi;
    const uint32_t rank = grp - li * g.tpi;
    const bool active = li < g.ipc;
    const bool merger = active && sl == 0;
    uint64_t R[C + 2], R1[C + 2];
#pragma unroll
    for (int e = 0; e < C + 2; e++) { R[e] = 0; R1[e] = 0; }
    uint32_t w1 = 0, w2 = 0;

    if (active) {
        const uint64_t* as = smem + (size_t)li * g.IS;
        const uint64_t* bs = as + g.SA;
        // window pair and the (a, b) bases of each phase; row r of a phase
        // multiplies a[abase + r] by b[bbase - r + c], c = 0..C-1
        uint32_t nblk1, a1, b1, a2, b2;
        const uint32_t half_threads = nwin_half / 2;
        if (rank < half_threads) {               // low half: windows j and L/C-1-j
            w1 = rank;
            w2 = nwin_half - 1 - rank;
            nblk1 = rank + 1;
            a1 = 0; b1 = w1 * C;
            a2 = 0; b2 = w2 * C;
        } else {                                 // high half: windows L/C+u and 2L/C-1-u
            const uint32_t u = rank - half_threads, u2 = nwin_half - 1 - u;
            w1 = nwin_half + u;
            w2 = nwin_half + u2;
            nblk1 = nwin_half - u;
            a1 = u * C; b1 = Lp;
            a2 = u2 * C; b2 = Lp;
        }
        const uint32_t nblk = nwin_half + 1;
        const uint32_t per = (nblk + g.S - 1) >> g.lgS;
        const uint32_t b_lo = sl * per < nblk ? sl * per : nblk;
        const uint32_t b_hi = b_lo + per < nblk ? b_lo + per : nblk;
        for (uint32_t blk = b_lo; blk < b_hi; blk++) {
            if (blk == nblk1) {
#pragma unroll
                for (int e = 0; e < C + 2; e++) { R1[e] = R[e]; R[e] = 0; }
            }
            const bool ph2 = blk >= nblk1;
            const uint32_t r0 = (ph2 ? blk - nblk1 : blk) * C;
            const uint32_t ab = (ph2 ? a2 : a1) + r0;
            const uint32_t yb = (ph2 ? b2 : b1) - r0;     // logical b_s index of ext[0]
            uint64_t av[C], ext[2 * C];
            const uint64_t* pa = as + skew<C>(ab);
            const uint64_t* pb0 = bs + skew<C>(yb);
            const uint64_t* pb1 = bs + skew<C>(yb + C);
#pragma unroll
            for (int h = 0; h < C / 2; h++) {
                lds128(pa + 2 * h, av[2 * h], av[2 * h + 1]);
                lds128(pb0 + 2 * h, ext[2 * h], ext[2 * h + 1]);
                lds128(pb1 + 2 * h, ext[C + 2 * h], ext[C + 2 * h + 1]);
            }
            static_assert(C == 8, "row_mac8 is written for 8-limb windows");
            row_mac8<8>(R, av[0], ext);
            row_mac8<7>(R, av[1], ext);
            row_mac8<6>(R, av[2], ext);
            row_mac8<5>(R, av[3], ext);
            row_mac8<4>(R, av[4], ext);
            row_mac8<3>(R, av[5], ext);
            row_mac8<2>(R, av[6], ext);
            row_mac8<1>(R, av[7], ext);
        }
        if (b_hi <= nblk1) {   // the slice ended among window w1's rows
#pragma unroll
            for (int e = 0; e < C + 2; e++) { R1[e] = R[e]; R[e] = 0; }
        }
    }
    // sum the S slices of each window pair onto slice 0
    for (uint32_t off = g.S >> 1; off > 0; off >>= 1) {
        uint64_t o1[C + 2], o2[C + 2];
#pragma unroll
        for (int e = 0; e < C + 2; e++) {
            o1[e] = __shfl_down_sync(0xffffffffu, R1[e], off);
            o2[e] = __shfl_down_sync(0xffffffffu, R[e], off);
        }
        if (sl < off) {
            add10(R1, o1);
            add10(R, o2);
        }
    }
    __syncthreads();   // every thread is done reading a_s / b_s

    // ---- window results into shared memory (over the operand area)
    if (merger) {
        uint64_t* racc = smem + (size_t)li * g.IS;
#pragma unroll
        for (int e = 0; e < C + 2; e++) {
            racc[w1 * (C + 2) + e] = R1[e];
            racc[w2 * (C + 2) + e] = R[e];
        }
    }
    __syncthreads();

    // ---- merge: thread takes windows 2*rank and 2*rank+1; D_u = P_u + O_{u-1}
    uint64_t D0[C], D1[C];
    uint32_t gq = 0, pq = active ? 1u : 0u;   // slice lanes pass carries through
    uint32_t g0 = 0, p0 = 0;
    if (merger) {
        const uint64_t* racc = smem + (size_t)li * g.IS;
        const uint32_t u0 = 2 * rank, u1 = u0 + 1;
        uint64_t o0 = 0, o1 = 0;
        if (u0 > 0) {
            o0 = racc[(u0 - 1) * (C + 2) + C];
            o1 = racc[(u0 - 1) * (C + 2) + C + 1];
        }
#pragma unroll
        for (int e = 0; e < C; e++) {
            D0[e] = racc[u0 * (C + 2) + e];
            D1[e] = racc[u1 * (C + 2) + e];
        }
        const uint64_t q0 = racc[u0 * (C + 2) + C], q1 = racc[u0 * (C + 2) + C + 1];
        // D0 += (o0, o1); D1 += (q0, q1) with carries out of the top limb
        uint32_t c0 = 0, c1 = 0;
        uint32_t all0 = 1, all1 = 1;
#pragma unroll
        for (int e = 0; e < C; e++) {
            const uint64_t add0 = (e == 0 ? o0 : (e == 1 ? o1 : 0));
            const uint64_t add1 = (e == 0 ? q0 : (e == 1 ? q1 : 0));
            uint64_t s = D0[e] + add0;
            uint32_t k = s < add0;
            uint64_t s2 = s + c0;
            k |= s2 < s;
            D0[e] = s2;
            c0 = k;
            s = D1[e] + add1;
            k = s < add1;
            s2 = s + c1;
            k |= s2 < s;
            D1[e] = s2;
            c1 = k;
            all0 &= D0[e] == ~0ull;
            all1 &= D1[e] == ~0ull;
        }
        g0 = c0;
        p0 = all0 & !c0;
        const uint32_t g1 = c1, p1 = all1 & !c1;
        gq = g1 | (p1 & g0);
        pq = p0 & p1;
    }
    const uint32_t cin = block_carry_in(gq, pq, !active || (rank == 0 && sl == 0), scratch);

    if (merger) {
        uint32_t c = cin;
#pragma unroll
        for (int e = 0; e < C; e++) {
            const uint64_t s = D0[e] + c;
            c = c & (s == 0);
            D0[e] = s;
        }
        c = g0 | (p0 & cin);
#pragma unroll
        for (int e = 0; e < C; e++) {
            const uint64_t s = D1[e] + c;
            c = c & (s == 0);
            D1[e] = s;
        }
        const uint32_t base = 2 * rank * C;   // first limb of window 2*rank
#pragma unroll
        for (int e = 0; e < 2 * C; e++) {
            const uint32_t x = base + e;
            if (x < g.out_limbs) store(li, x, e < C ? D0[e] : D1[e - C]);
        }
    }
    __syncthreads();
}


// Geometry of a CTA that multiplies up to `ipc_cap` instances of L 64-bit
// limbs (full product when `full`).  IS is the per-instance shared stride.
__host__ __device__ inline MulGeom mul_geometry(uint32_t L, bool full, uint32_t ipc_cap) {
    constexpr int C = MUL_C;
    MulGeom g;
    g.L = L;
    g.m = L;
    g.Lp = (L + 2 * C - 1) / (2 * C) * (2 * C);
    g.tpi = full ? g.Lp / C : g.Lp / (2 * C);
    g.ipc = g.tpi >= 256 ? 1 : 256 / g.tpi;
    if (g.ipc > ipc_cap) g.ipc = ipc_cap;
    if (g.ipc < 1) g.ipc = 1;
    g.SA = g.Lp + 2 * (g.Lp / C) + 2;
    const uint32_t SB = (g.Lp + 2 * C) + 2 * ((g.Lp + 2 * C) / C) + 2;
    const uint32_t nwin = 2 * g.tpi;
    g.IS = g.SA + SB;
    if (g.IS < nwin * (C + 2)) g.IS = nwin * (C + 2);
    g.IS = (g.IS + 1) & ~1u;                    // 16-byte aligned instance base
    if ((g.IS / 2) % 2 == 0) g.IS += 2;         // odd 16-byte stride spreads banks across instances
    g.out_limbs = full ? 2 * L : L;
    g.out_words = g.out_limbs;
    g.S = 1;
    g.lgS = 0;
    return g;
}

// One instance with its rows cut into S slices: S = the largest power of two
// up to `threads` / tpi and up to one row block per slice.
__host__ __device__ inline MulGeom mul_geometry_single_sliced(uint32_t L, bool full, uint32_t threads) {
    MulGeom g = mul_geometry(L, full, 1);
    const uint32_t nblk = g.Lp / MUL_C + 1;
    uint32_t lg = 0;
    while (lg < 5 && (g.tpi << (lg + 1)) <= threads && (2u << lg) <= nblk) lg++;
    g.S = 1u << lg;
    g.lgS = lg;
    return g;
}

__host__ __device__ inline uint32_t mul_threads(const MulGeom& g) { return (g.ipc * g.tpi * g.S + 31) / 32 * 32; }
__host__ __device__ inline size_t mul_smem_bytes(const MulGeom& g) { return (size_t)g.ipc * g.IS * 8 + 3 * 32 * 4; }

}  // namespace bi
