// blockops.cuh -- CTA-cooperative big-integer primitives on shared memory.
//
// Every function here is called by all threads of a cooperating group (the
// whole CTA: CtaGroup, the default) with the same arguments, and synchronises
// that group.  Limbs are 64-bit, little-endian.  These are the batched-division building blocks:
// the reference's division prototype composes the same primitives (shift,
// compare, findk, add, sub, mult; prototypes/div.c:49-218, and their parallel
// forms in futhark/helper.fut:101-124 and futhark/div.fut:21-69).
#pragma once

#include "common.cuh"

namespace bi {

// R[0..10) += a * (e[T0 .. T0+8)): one row of a window product (see mul.cu)
template <int T0>
__device__ __forceinline__ void row_mac8(uint64_t (&R)[10], uint64_t a, const uint64_t (&e)[16]) {
    asm volatile(
        "{\n\t.reg .u64 t;\n\t"
        "mul.lo.u64 t, %10, %11;\n\tadd.cc.u64  %0, %0, t;\n\t"
        "mul.lo.u64 t, %10, %12;\n\taddc.cc.u64 %1, %1, t;\n\t"
        "mul.lo.u64 t, %10, %13;\n\taddc.cc.u64 %2, %2, t;\n\t"
        "mul.lo.u64 t, %10, %14;\n\taddc.cc.u64 %3, %3, t;\n\t"
        "mul.lo.u64 t, %10, %15;\n\taddc.cc.u64 %4, %4, t;\n\t"
        "mul.lo.u64 t, %10, %16;\n\taddc.cc.u64 %5, %5, t;\n\t"
        "mul.lo.u64 t, %10, %17;\n\taddc.cc.u64 %6, %6, t;\n\t"
        "mul.lo.u64 t, %10, %18;\n\taddc.cc.u64 %7, %7, t;\n\t"
        "addc.cc.u64 %8, %8, 0;\n\t"
        "addc.u64    %9, %9, 0;\n\t"
        "mul.hi.u64 t, %10, %11;\n\tadd.cc.u64  %1, %1, t;\n\t"
        "mul.hi.u64 t, %10, %12;\n\taddc.cc.u64 %2, %2, t;\n\t"
        "mul.hi.u64 t, %10, %13;\n\taddc.cc.u64 %3, %3, t;\n\t"
        "mul.hi.u64 t, %10, %14;\n\taddc.cc.u64 %4, %4, t;\n\t"
        "mul.hi.u64 t, %10, %15;\n\taddc.cc.u64 %5, %5, t;\n\t"
        "mul.hi.u64 t, %10, %16;\n\taddc.cc.u64 %6, %6, t;\n\t"
        "mul.hi.u64 t, %10, %17;\n\taddc.cc.u64 %7, %7, t;\n\t"
        "mul.hi.u64 t, %10, %18;\n\taddc.cc.u64 %8, %8, t;\n\t"
        "addc.u64    %9, %9, 0;\n\t}"
        : "+l"(R[0]), "+l"(R[1]), "+l"(R[2]), "+l"(R[3]), "+l"(R[4]), "+l"(R[5]), "+l"(R[6]),
          "+l"(R[7]), "+l"(R[8]), "+l"(R[9])
        : "l"(a), "l"(e[T0 + 0]), "l"(e[T0 + 1]), "l"(e[T0 + 2]), "l"(e[T0 + 3]), "l"(e[T0 + 4]),
          "l"(e[T0 + 5]), "l"(e[T0 + 6]), "l"(e[T0 + 7]));
}

// Shared scratch needed by the functions below: 128 32-bit words.
constexpr int BLOCKOPS_SCRATCH_WORDS = 128;

__device__ __forceinline__ uint32_t block_max_u32(uint32_t v, uint32_t* scratch) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    uint32_t x = lane < nw ? scratch[lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
    __syncthreads();
    return x;
}

// The threads that cooperate on one number.  CtaGroup: the whole CTA, with
// __syncthreads and shared-memory exchanges through `scratch`.  (Work on one
// warp -- small products, long division -- has its own kernels.)
struct CtaGroup {
    static __device__ __forceinline__ int rank() { return (int)threadIdx.x; }
    static __device__ __forceinline__ int size() { return (int)blockDim.x; }
    static __device__ __forceinline__ void sync() { __syncthreads(); }
    static __device__ __forceinline__ uint32_t carry_in(uint32_t g, uint32_t p, bool seg, uint32_t* scratch) {
        return block_carry_in(g, p, seg, scratch);
    }
    static __device__ __forceinline__ uint32_t max_u32(uint32_t v, uint32_t* scratch) {
        return block_max_u32(v, scratch);
    }
    // v as held by rank src
    static __device__ __forceinline__ uint32_t bcast(uint32_t v, int src, uint32_t* scratch) {
        if ((int)threadIdx.x == src) scratch[100] = v;
        __syncthreads();
        const uint32_t r = scratch[100];
        __syncthreads();
        return r;
    }
};

template <typename Grp = CtaGroup>
__device__ __forceinline__ void chunk_of(int len, int& lo, int& hi) {
    const int T = Grp::size();
    const int cw = (len + T - 1) / T;
    lo = Grp::rank() * cw;
    hi = lo + cw < len ? lo + cw : len;
    if (lo > len) lo = len;
}

// number of limbs up to and including the top nonzero one (0 for zero) -- findk + 1
// (prototypes/div.c:92-101; futhark/div.fut:38-39)
template <typename Grp = CtaGroup>
__device__ __forceinline__ int block_prec(const uint64_t* X, int len, uint32_t* scratch) {
    uint32_t best = 0;
    for (int i = Grp::rank(); i < len; i += Grp::size())
        if (X[i] != 0) best = max(best, (uint32_t)(i + 1));
    return (int)Grp::max_u32(best, scratch);
}

template <typename Grp = CtaGroup>
__device__ __forceinline__ void block_zero(uint64_t* X, int len) {
    for (int i = Grp::rank(); i < len; i += Grp::size()) X[i] = 0;
}

template <typename Grp = CtaGroup>
__device__ __forceinline__ void block_copy(uint64_t* dst, const uint64_t* src, int len) {
    for (int i = Grp::rank(); i < len; i += Grp::size()) dst[i] = src[i];
}

// out[0..len) = (X << s bits) over len limbs of X (zero above lx); s in [0, 64).  out != X.
template <typename Grp = CtaGroup>
__device__ __forceinline__ void block_shl_bits(uint64_t* out, const uint64_t* X, int lx, int len, int s) {
    for (int i = Grp::rank(); i < len; i += Grp::size()) {
        const uint64_t cur = i < lx ? X[i] : 0;
        const uint64_t prev = (i > 0 && i - 1 < lx) ? X[i - 1] : 0;
        out[i] = s ? ((cur << s) | (prev >> (64 - s))) : cur;
    }
}

// out[0..len) = X >> s bits (X has lx limbs); s in [0, 64).  out != X.
template <typename Grp = CtaGroup>
__device__ __forceinline__ void block_shr_bits(uint64_t* out, const uint64_t* X, int lx, int len, int s) {
    for (int i = Grp::rank(); i < len; i += Grp::size()) {
        const uint64_t cur = i < lx ? X[i] : 0;
        const uint64_t next = i + 1 < lx ? X[i + 1] : 0;
        out[i] = s ? ((cur >> s) | (next << (64 - s))) : cur;
    }
}

// out = X + Y (sub=false) or X - Y (sub=true) mod B^len, X and Y zero-extended
// from lx / ly limbs.  out may alias X or Y.  Returns the carry (borrow) out.
// The carries are resolved by block_carry_in over per-thread chunks, i.e. the
// carry-propagation scan of the reference's badd/bsub (ker-add.cu.h:121-149,
// futhark/sub.fut:14-26) applied to a single instance held by the whole CTA.
template <typename Grp = CtaGroup>
__device__ __forceinline__ uint32_t block_addsub(uint64_t* out, const uint64_t* X, int lx, const uint64_t* Y,
                                                 int ly, int len, bool sub, uint32_t* scratch) {
    int lo, hi;
    chunk_of<Grp>(len, lo, hi);
    uint32_t G = 0, P = 1;
    for (int i = lo; i < hi; i++) {
        const uint64_t x = i < lx ? X[i] : 0, y = i < ly ? Y[i] : 0;
        uint32_t g, p;
        if (!sub) { const uint64_t s = x + y; g = s < x; p = s == ~0ull; }
        else      { g = x < y; p = x == y; }
        G = g | (p & G);
        P = p & P;
    }
    if (lo >= hi) { G = 0; P = 1; }
    const uint32_t cin = Grp::carry_in(G, P, Grp::rank() == 0, scratch);
    uint32_t c = cin;
    for (int i = lo; i < hi; i++) {
        const uint64_t x = i < lx ? X[i] : 0, y = i < ly ? Y[i] : 0;
        uint64_t s;
        uint32_t g, p;
        if (!sub) { s = x + y; g = s < x; p = s == ~0ull; out[i] = s + c; }
        else      { s = x - y; g = x < y; p = x == y; out[i] = s - c; }
        c = g | (p & c);
    }
    // carry out of the whole number: the last nonempty chunk's final carry
    const int T = Grp::size();
    const int cw = (len + T - 1) / T;
    const int last = cw ? (len - 1) / cw : 0;
    return Grp::bcast(c, last, scratch);
}

// -1, 0, 1 as X <, ==, > Y (both zero-extended to len limbs) -- the reference's
// lt/eq (prototypes/div.c:49-62; futhark/helper.fut:109-115)
template <typename Grp = CtaGroup>
__device__ __forceinline__ int block_cmp(const uint64_t* X, int lx, const uint64_t* Y, int ly, int len,
                                        uint32_t* scratch) {
    uint32_t best = 0;
    for (int i = Grp::rank(); i < len; i += Grp::size()) {
        const uint64_t x = i < lx ? X[i] : 0, y = i < ly ? Y[i] : 0;
        if (x != y) best = max(best, ((uint32_t)(i + 1) << 1) | (x > y ? 1u : 0u));
    }
    const uint32_t m = Grp::max_u32(best, scratch);
    if (m == 0) return 0;
    return (m & 1u) ? 1 : -1;
}

// Limbs per 8-column window in block_mul's window buffer: the 10-limb window
// plus one, an odd stride so consecutive windows fall on different banks.
constexpr int BLOCK_MUL_WS = 11;

// R[0..10) += O[0..10) with the carry chain.
__device__ __forceinline__ void add10(uint64_t (&R)[10], const uint64_t (&O)[10]) {
    asm("add.cc.u64 %0, %0, %10;\n\taddc.cc.u64 %1, %1, %11;\n\taddc.cc.u64 %2, %2, %12;\n\t"
        "addc.cc.u64 %3, %3, %13;\n\taddc.cc.u64 %4, %4, %14;\n\taddc.cc.u64 %5, %5, %15;\n\t"
        "addc.cc.u64 %6, %6, %16;\n\taddc.cc.u64 %7, %7, %17;\n\taddc.cc.u64 %8, %8, %18;\n\t"
        "addc.u64 %9, %9, %19;"
        : "+l"(R[0]), "+l"(R[1]), "+l"(R[2]), "+l"(R[3]), "+l"(R[4]), "+l"(R[5]), "+l"(R[6]), "+l"(R[7]),
          "+l"(R[8]), "+l"(R[9])
        : "l"(O[0]), "l"(O[1]), "l"(O[2]), "l"(O[3]), "l"(O[4]), "l"(O[5]), "l"(O[6]), "l"(O[7]), "l"(O[8]),
          "l"(O[9]));
}

// out[c..olen) for c >= floor(c_lo / 8) * 8: the limbs of (A[0..la) *
// Bm[0..lb)) mod B^olen, exact when c_lo = 0.  With c_lo > 0 only the column
// windows from floor(c_lo / 8) up are summed (a short product): the limbs
// below are not written, and the value of out above c_lo falls short of the
// true product's by less than min(la, lb) * B^(c_lo + 1) -- under one unit
// two limbs above c_lo.  out must not alias A, Bm or wbuf; wbuf holds
// ceil(olen/8)*BLOCK_MUL_WS limbs.
//
// Column windows of 8 limbs are accumulated with row_mac8 (as in mul.cu).  The
// rows of each window are cut into S slices (S a power of two up to 32, the
// one that minimises rounds x rows per slice for the CTA's size), computed by
// S consecutive lanes and summed with warp shuffles, so a product with few
// windows still occupies the CTA.  The windows are then merged with a carry
// lookahead across windows.
template <typename Grp = CtaGroup>
__device__ __forceinline__ void block_mul(const uint64_t* A, int la, const uint64_t* Bm, int lb, uint64_t* out,
                                          int olen, uint64_t* wbuf, uint32_t* scratch, int c_lo = 0) {
    constexpr int C = 8;
    constexpr int WS = BLOCK_MUL_WS;   // window stride in wbuf: odd, so lanes' 64-bit accesses spread over the banks
    const int T = Grp::size(), t = Grp::rank(), lane = t & 31;
    const int W = (olen + C - 1) / C;
    const int w0 = c_lo / C < W ? c_lo / C : W;
    const int NW = W - w0;
    int S = 1, lgS = 0;
    const int mr = la < lb + C - 1 ? la : lb + C - 1;   // most rows of any window
    if (NW < T && mr > C) {
        uint32_t best = 0xffffffffu;
        for (int lg = 0; lg <= 5; lg++) {
            const uint32_t rounds = ((uint32_t)(NW << lg) + T - 1) / (uint32_t)T;
            const uint32_t rows = (uint32_t)((((mr + (1 << lg) - 1) >> lg) + C - 1) & ~(C - 1));
            const uint32_t cost = rounds * (rows + lg);
            if (cost < best) { best = cost; S = 1 << lg; lgS = lg; }
        }
    }
    for (int base = t & ~31; base < NW * S; base += T) {
        const int j = base + lane;
        const int w = w0 + (j >> lgS), sl = j & (S - 1);
        uint64_t R[C + 2];
#pragma unroll
        for (int e = 0; e < C + 2; e++) R[e] = 0;
        if (j < NW * S) {
            const int k0 = w * C;
            int ilo = k0 - lb + 1;
            if (ilo < 0) ilo = 0;
            int ihi = k0 + C;
            if (ihi > la) ihi = la;
            const int len = ihi > ilo ? ihi - ilo : 0;
            const int span = (((len + S - 1) >> lgS) + C - 1) & ~(C - 1);
            const int lo = ilo + sl * span;
            const int hi = lo + span < ihi ? lo + span : ihi;
            for (int i0 = lo; i0 < hi; i0 += C) {
                uint64_t av[C], ext[2 * C];
#pragma unroll
                for (int k = 0; k < C; k++) av[k] = (i0 + k < hi) ? A[i0 + k] : 0;
#pragma unroll
                for (int q = 0; q < 2 * C; q++) {
                    const int bi = k0 - i0 - C + q;
                    ext[q] = (bi >= 0 && bi < lb) ? Bm[bi] : 0;
                }
                // rows past hi are zero: skip them (each row extends R's carry chain)
                const int nr = hi - i0;
                row_mac8<8>(R, av[0], ext);
                if (nr > 1) row_mac8<7>(R, av[1], ext);
                if (nr > 2) row_mac8<6>(R, av[2], ext);
                if (nr > 3) row_mac8<5>(R, av[3], ext);
                if (nr > 4) row_mac8<4>(R, av[4], ext);
                if (nr > 5) row_mac8<3>(R, av[5], ext);
                if (nr > 6) row_mac8<2>(R, av[6], ext);
                if (nr > 7) row_mac8<1>(R, av[7], ext);
            }
        }
        // sum the S slices of a window (consecutive lanes) onto its slice 0
        for (int off = S >> 1; off > 0; off >>= 1) {
            uint64_t o[C + 2];
#pragma unroll
            for (int e = 0; e < C + 2; e++) o[e] = __shfl_down_sync(0xffffffffu, R[e], off);
            if (sl < off) add10(R, o);
        }
        if (j < NW * S && sl == 0) {
#pragma unroll
            for (int e = 0; e < C + 2; e++) wbuf[w * WS + e] = R[e];
        }
    }
    Grp::sync();
    // merge: thread takes windows [u_lo, u_hi); D_u = P_u + O_{u-1} (in place in wbuf)
    const int cw = (NW + T - 1) / T;
    int u_lo = w0 + t * cw, u_hi = u_lo + cw;
    if (u_lo > W) u_lo = W;
    if (u_hi > W) u_hi = W;
    uint32_t G = 0, P = 1;
    uint32_t gs = 0, ps = 0;   // per-window bits (cw <= 32 assumed: NW <= 32 * T)
    for (int u = u_lo; u < u_hi; u++) {
        uint64_t o0 = 0, o1 = 0;
        if (u > w0) {
            o0 = wbuf[(u - 1) * WS + C];
            o1 = wbuf[(u - 1) * WS + C + 1];
        }
        uint32_t c = 0, all = 1;
        for (int e = 0; e < C; e++) {
            const uint64_t add = e == 0 ? o0 : (e == 1 ? o1 : 0);
            const uint64_t x = wbuf[u * WS + e];
            const uint64_t s = x + add;
            uint32_t k = s < add;
            const uint64_t s2 = s + c;
            k |= s2 < s;
            c = k;
            all &= s2 == ~0ull;
        }
        const uint32_t g = c, p = all & !c;
        gs |= g << (u - u_lo);
        ps |= p << (u - u_lo);
        G = g | (p & G);
        P = p & P;
    }
    // the D values are recomputed below (the O limbs are never overwritten)
    const uint32_t cin = Grp::carry_in(G, P, t == 0, scratch);
    uint32_t c_win = cin;
    for (int u = u_lo; u < u_hi; u++) {
        uint64_t o0 = 0, o1 = 0;
        if (u > w0) {
            o0 = wbuf[(u - 1) * WS + C];
            o1 = wbuf[(u - 1) * WS + C + 1];
        }
        uint32_t c = 0;
        uint32_t cc = c_win;
        for (int e = 0; e < C; e++) {
            const uint64_t add = e == 0 ? o0 : (e == 1 ? o1 : 0);
            const uint64_t x = wbuf[u * WS + e];
            const uint64_t s = x + add;
            uint32_t k = s < add;
            const uint64_t s2 = s + c;
            k |= s2 < s;
            c = k;
            const uint64_t d = s2 + cc;
            cc = cc & (d == 0);
            const int pos = u * C + e;
            if (pos < olen) out[pos] = d;
        }
        const uint32_t g = (gs >> (u - u_lo)) & 1u, p = (ps >> (u - u_lo)) & 1u;
        c_win = g | (p & c_win);
    }
    Grp::sync();
}

}  // namespace bi
