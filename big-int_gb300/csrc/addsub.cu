// addsub.cu -- batched addition and sign-magnitude subtraction.
//
// Semantics follow the reference: r = (a + b) mod B^m with the carry-out
// dropped (cuda/ker-add.cu.h:121-149, 212-243), and r = |a - b| with
// sign = (a < b) (futhark/sub.fut:14-26).
//
// Design (HBM-bound; every limb is read once and written once):
//   * A CTA owns a tile of whole instances, ipt = floor(TILE / m) of them,
//     laid out contiguously in the flat [n][m] array.  Instances never cross
//     a tile, so no carry ever crosses a CTA.
//   * The tile is cut into warp rows of 32 x 16 bytes.  Lane t of a warp
//     loads bytes [16t, 16t+16) of each row, so every load and store
//     instruction is a fully coalesced 512-byte transaction.
//   * Carries are resolved with warp ballots (WarpCarry): one 32-bit
//     addition resolves the carries of a whole row; rows of a warp are
//     chained with a scalar carry; warps of a CTA exchange one (generate,
//     propagate) pair each through shared memory, and each warp resolves its
//     own carry-in with one more ballot -- a single __syncthreads per tile.
//   * Subtraction runs the borrow chains of a - b and b - a side by side;
//     the instance's final a - b borrow is its sign (a < b), published
//     through shared memory, and selects which difference is stored.
//
// When m is a multiple of 64 bytes and the buffers are 32-byte aligned (every
// size of the reference's benchmarks), a leaner chunked kernel runs instead:
// each lane owns 64 consecutive bytes of one instance, so instance
// boundaries fall only between lanes and the lane's limbs are added or
// subtracted on the hardware carry chain (chain.cuh).
#include "chain.cuh"
#include "common.cuh"

namespace bi {

enum AddSubOp { OP_ADD = 0, OP_SUB = 1 };

template <typename T, int VEC>
__device__ __forceinline__ void load_limbs(const T* p, T (&v)[VEC]) {
    if constexpr (VEC * sizeof(T) == 16) {
        uint4 x;
        asm("ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];"
            : "=r"(x.x), "=r"(x.y), "=r"(x.z), "=r"(x.w) : "l"(p));
        if constexpr (sizeof(T) == 8) {
            v[0] = ((uint64_t)x.y << 32) | x.x;
            v[1] = ((uint64_t)x.w << 32) | x.z;
        } else {
            v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) v[e] = __ldcs(p + e);
    }
}

template <typename T, int VEC>
__device__ __forceinline__ void store_limbs(T* p, const T (&v)[VEC]) {
    if constexpr (VEC * sizeof(T) == 16) {
        uint4 x;
        if constexpr (sizeof(T) == 8) {
            x.x = (uint32_t)v[0]; x.y = (uint32_t)(v[0] >> 32);
            x.z = (uint32_t)v[1]; x.w = (uint32_t)(v[1] >> 32);
        } else {
            x.x = v[0]; x.y = v[1]; x.z = v[2]; x.w = v[3];
        }
        asm volatile("st.global.cs.v4.u32 [%0], {%1,%2,%3,%4};"
                     :: "l"(p), "r"(x.x), "r"(x.y), "r"(x.z), "r"(x.w) : "memory");
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) __stcs(p + e, v[e]);
    }
}

// Composite (generate, propagate) of a sequence of carry stages: applying
// stage (g, p) after (G, P) gives (g | (p & G), p & P).
struct GP {
    uint32_t g, p;
};

// Per-row position bookkeeping of a lane's VEC limbs: which limbs start an
// instance (seg), which end one (last), and the instance index (within the
// tile) of the lane's first valid limb.  One division per row and lane.
template <int VEC>
__device__ __forceinline__ void row_positions(int li0, int len, uint32_t m, const FastDiv& mdiv, uint32_t& seg,
                                              uint32_t& last, uint32_t& valid, uint32_t& q0, uint32_t& wrapbits) {
    seg = last = valid = wrapbits = 0;
    q0 = 0;
    if (li0 + VEC <= 0 || li0 >= len) return;
    if (m >= (uint32_t)VEC && li0 >= 0) {
        q0 = mdiv.div((uint32_t)li0);
        uint32_t pos = (uint32_t)li0 - q0 * m;
#pragma unroll
        for (int e = 0; e < VEC; e++) {
            if (e > 0) {
                pos++;
                if (pos == m) { pos = 0; wrapbits |= 1u << e; }
            }
            if (li0 + e < len) {
                valid |= 1u << e;
                if (pos == 0) seg |= 1u << e;
                if (pos == m - 1) last |= 1u << e;
            }
        }
    } else {
        // tiny m or a lane straddling the tile start: per-limb division
        bool first = true;
#pragma unroll
        for (int e = 0; e < VEC; e++) {
            const int li = li0 + e;
            if (li < 0 || li >= len) continue;
            const uint32_t q = mdiv.div((uint32_t)li);
            const uint32_t pos = (uint32_t)li - q * m;
            if (first) { q0 = q; first = false; }
            else if (q != q0) wrapbits |= 1u << e;   // (only used when m >= VEC)
            valid |= 1u << e;
            if (pos == 0) seg |= 1u << e;
            if (pos == m - 1) last |= 1u << e;
        }
    }
}

template <typename T, int WARPS, int ROWS, int VEC, int OP>
__global__ void __launch_bounds__(WARPS * 32, 1024 / (WARPS * 32))
addsub_kernel(const T* a, const T* b, T* r, uint8_t* sign_out, uint32_t m, uint64_t n,
              uint32_t ipt, FastDiv mdiv, uint64_t ntiles) {
    constexpr int ROWL = 32 * VEC;              // limbs per warp row
    constexpr int TILE = WARPS * ROWS * ROWL;   // limbs per CTA tile
    constexpr int NCH = (OP == OP_SUB) ? 2 : 1; // carry chains (sub: a-b and b-a)
    constexpr T HI = Limb<T>::HIGHEST;
    static_assert(ROWS * VEC <= 32, "per-limb bit masks hold 32 limbs");

    __shared__ uint32_t s_gp[NCH][WARPS];       // per-warp composite, bit0 = g, bit1 = p
    __shared__ uint32_t s_first[WARPS];         // 1 if the warp's first limb starts an instance
    __shared__ uint8_t s_sign[(OP == OP_SUB) ? TILE : 1];

    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = threadIdx.x >> 5;

    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t inst0 = tile * (uint64_t)ipt;
        const uint64_t left = n - inst0;
        const uint32_t ninst = left < ipt ? (uint32_t)left : ipt;
        const uint64_t start = inst0 * (uint64_t)m;     // flat limb index of the tile
        const int len = (int)(ninst * m);
        const int off = (int)(start & (VEC - 1));       // limbs before start in the first vector
        const uint64_t abase = start - off;

        // d = a + b (add) or a - b (sub), both without carries; gbits = carry
        // (borrow) generated by each limb on its own
        T d[ROWS][VEC], y[ROWS][VEC];
        uint32_t gbits = 0, segbits = 0, lastbits = 0, validbits = 0;

        // issue every load of the tile before using any of them
#pragma unroll
        for (int rr = 0; rr < ROWS; rr++) {
            const int vi = (int)((warp * ROWS + rr) * 32 + lane);
            const int li0 = vi * VEC - off;
            const uint64_t gi = abase + (uint64_t)vi * VEC;
            if (li0 >= 0 && li0 + VEC <= len) {
                load_limbs<T, VEC>(a + gi, d[rr]);
                load_limbs<T, VEC>(b + gi, y[rr]);
            } else {
#pragma unroll
                for (int e = 0; e < VEC; e++) {
                    const int li = li0 + e;
                    const bool ok = li >= 0 && li < len;
                    d[rr][e] = ok ? __ldcs(a + gi + e) : (T)0;
                    y[rr][e] = ok ? __ldcs(b + gi + e) : (T)0;
                }
            }
        }
#pragma unroll
        for (int rr = 0; rr < ROWS; rr++) {
            const int vi = (int)((warp * ROWS + rr) * 32 + lane);
            const int li0 = vi * VEC - off;
#pragma unroll
            for (int e = 0; e < VEC; e++) {
                const T x = d[rr][e];
                uint32_t g;
                if (OP == OP_ADD) { d[rr][e] = x + y[rr][e]; g = d[rr][e] < x; }
                else              { d[rr][e] = x - y[rr][e]; g = x < y[rr][e]; }
                gbits |= g << (rr * VEC + e);
            }
            uint32_t sg, la, va, q0, wr;
            row_positions<VEC>(li0, len, m, mdiv, sg, la, va, q0, wr);
            segbits |= sg << (rr * VEC);
            lastbits |= la << (rr * VEC);
            validbits |= va << (rr * VEC);
        }

        // ---- per-row lane classes and row ballots
        uint32_t rowA[NCH][ROWS], rowB[NCH][ROWS];
        uint32_t rowS0 = 0;   // bit rr: lane 0 of row rr starts an instance
#pragma unroll
        for (int rr = 0; rr < ROWS; rr++) {
            GP lg[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++) { lg[c].g = 0; lg[c].p = 1; }
#pragma unroll
            for (int e = 0; e < VEC; e++) {
                const int bit = rr * VEC + e;
                const uint32_t ok = (validbits >> bit) & 1u;
                const uint32_t seg = (segbits >> bit) & 1u;
                const uint32_t g0 = ok & (gbits >> bit);
                const uint32_t p = ok & (uint32_t)(OP == OP_ADD ? d[rr][e] == HI : d[rr][e] == 0);
#pragma unroll
                for (int c = 0; c < NCH; c++) {
                    if (e > 0 && seg) { lg[c].g = 0; lg[c].p = 0; }
                    // b - a borrows where a - b neither borrows nor is zero
                    const uint32_t ge = (c == 0) ? g0 : (ok & ~g0 & ~p & 1u);
                    lg[c].g = ge | (p & lg[c].g);
                    lg[c].p = p & lg[c].p;
                }
            }
            const uint32_t S = __ballot_sync(0xffffffffu, segbits >> (rr * VEC) & 1u);
            const uint32_t kill = S >> 1;   // lane t+1 starts an instance: no carry out of lane t
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                rowA[c][rr] = __ballot_sync(0xffffffffu, lg[c].g | lg[c].p) & ~kill;
                rowB[c][rr] = __ballot_sync(0xffffffffu, lg[c].g) & ~kill;
            }
            rowS0 |= (S & 1u) << rr;
        }

        // ---- warp composite over rows -> shared memory
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                GP w = {0u, 1u};
#pragma unroll
                for (int rr = 0; rr < ROWS; rr++) {
                    if ((rowS0 >> rr) & 1u) { w.g = 0; w.p = 0; }
                    const uint32_t g = warp_carry_resolve(rowA[c][rr], rowB[c][rr], 0).cout;
                    const uint32_t gp = warp_carry_resolve(rowA[c][rr], rowB[c][rr], 1).cout;
                    const uint32_t p = gp & ~g;
                    w.g = g | (p & w.g);
                    w.p = p & w.p;
                }
                s_gp[c][warp] = w.g | (w.p << 1);
            }
            s_first[warp] = rowS0 & 1u;
        }
        __syncthreads();

        // ---- carry into this warp: ballot over the preceding warps
        uint32_t cin[NCH];
        {
            const bool before = lane < warp;
            // a carry leaving warp j is killed if warp j+1 starts an instance
            const bool killed = before && s_first[lane + 1 < WARPS ? lane + 1 : 0];
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                const uint32_t gp = before ? s_gp[c][lane] : 0u;
                const bool live = before && !killed;
                const uint32_t A = __ballot_sync(0xffffffffu, live && (gp & 3u));
                const uint32_t B = __ballot_sync(0xffffffffu, live && (gp & 1u));
                cin[c] = (warp_carry_resolve(A, B, 0).carries >> warp) & 1u;
            }
        }

        // ---- replay rows with the resolved carries
        uint32_t c1bits = 0, c2bits = 0;   // sub: borrow into each limb for a-b and b-a
#pragma unroll
        for (int rr = 0; rr < ROWS; rr++) {
            uint32_t c_in[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                if ((rowS0 >> rr) & 1u) cin[c] = 0;
                const WarpCarry wc = warp_carry_resolve(rowA[c][rr], rowB[c][rr], cin[c]);
                c_in[c] = (wc.carries >> lane) & 1u;
                cin[c] = wc.cout;
            }
#pragma unroll
            for (int e = 0; e < VEC; e++) {
                const int bit = rr * VEC + e;
                const uint32_t seg = (segbits >> bit) & 1u;
                const uint32_t g0 = (gbits >> bit) & 1u;
                if (OP == OP_ADD) {
                    if (e > 0 && seg) c_in[0] = 0;
                    const uint32_t p = d[rr][e] == HI;
                    const T s = d[rr][e];
                    d[rr][e] = s + (T)c_in[0];
                    c_in[0] = g0 | (p & c_in[0]);
                } else {
                    if (e > 0 && seg) { c_in[0] = 0; c_in[1] = 0; }
                    const uint32_t p = d[rr][e] == 0;
                    c1bits |= c_in[0] << bit;
                    c2bits |= c_in[1] << bit;
                    c_in[0] = g0 | (p & c_in[0]);
                    c_in[1] = (~g0 & ~p & 1u) | (p & c_in[1]);
                    if ((lastbits >> bit) & 1u) {
                        // instance index of this limb within the tile
                        const int li = ((int)((warp * ROWS + rr) * 32 + lane)) * VEC - off + e;
                        s_sign[mdiv.div((uint32_t)li)] = (uint8_t)c_in[0];
                    }
                }
            }
        }

        if (OP == OP_SUB) __syncthreads();

        // ---- store
#pragma unroll
        for (int rr = 0; rr < ROWS; rr++) {
            const int vi = (int)((warp * ROWS + rr) * 32 + lane);
            const int li0 = vi * VEC - off;
            const uint64_t gi = abase + (uint64_t)vi * VEC;
            T out[VEC];
            if (OP == OP_ADD) {
#pragma unroll
                for (int e = 0; e < VEC; e++) out[e] = d[rr][e];
            } else {
                uint32_t q = 0;
                const uint32_t rowvalid = (validbits >> (rr * VEC)) & ((1u << VEC) - 1u);
                if (rowvalid) {
                    const int lfirst = li0 + (int)(__ffs(rowvalid) - 1);
                    q = mdiv.div((uint32_t)lfirst);
                }
#pragma unroll
                for (int e = 0; e < VEC; e++) {
                    const int bit = rr * VEC + e;
                    const bool ok = (validbits >> bit) & 1u;
                    if (e > 0 && ((segbits >> bit) & 1u) && ((validbits >> (bit - 1)) & 1u)) q++;
                    const bool neg = ok && s_sign[q];
                    const T c1 = (T)((c1bits >> bit) & 1u), c2 = (T)((c2bits >> bit) & 1u);
                    out[e] = neg ? (T)(0 - d[rr][e] - c2) : (T)(d[rr][e] - c1);
                    if (ok && sign_out != nullptr && ((segbits >> bit) & 1u)) sign_out[inst0 + q] = s_sign[q];
                }
            }
            if (li0 >= 0 && li0 + VEC <= len) {
                store_limbs<T, VEC>(r + gi, out);
            } else {
#pragma unroll
                for (int e = 0; e < VEC; e++) {
                    const int li = li0 + e;
                    if (li >= 0 && li < len) __stcs(r + gi + e, out[e]);
                }
            }
        }
        __syncthreads();   // shared state is rewritten by the next tile
    }
}

// ---------------------------------------------------------------------------
// Chunked kernel (m a multiple of K = 64 bytes / limb size, 32-byte aligned
// buffers).  A tile is W warps x 32 lanes x one chunk of K limbs, holding
// ipt = floor(32 W / (m / K)) whole instances.  Lane t owns chunk t of the
// tile (two 32-byte loads per operand), which lies inside one instance, so:
//   * pass 1 runs the lane's K-limb add (subtract) on the carry chain with
//     carry-in 0 to get its generate bit g, and compares the chunks for its
//     propagate bit p (add: x = ~y limb by limb; sub: x = y);
//   * the warp resolves the lanes' carries with ballots (WarpCarry), instance
//     starts killing the carry from the lane before; warps exchange one
//     (g, p) pair each through shared memory (one barrier);
//   * pass 2 reruns the chain with the lane's resolved carry-in and stores.
// Subtraction also resolves the chain of b - a, whose lane classes follow
// from pass 1 (b - a borrows out of a lane iff a > b there: !g & !p).  The
// lane holding an instance's last chunk publishes the sign (a < b) through
// shared memory; a negative instance stores b - a - c2 = ~(a - b - (1 - c2))
// with c2 its lane's b - a borrow-in, so pass 2 is one chain either way.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ld32B(const void* p, uint64_t& w0, uint64_t& w1, uint64_t& w2, uint64_t& w3) {
    asm("ld.global.cs.v4.u64 {%0,%1,%2,%3}, [%4];" : "=l"(w0), "=l"(w1), "=l"(w2), "=l"(w3) : "l"(p));
}
__device__ __forceinline__ void st32B(void* p, uint64_t w0, uint64_t w1, uint64_t w2, uint64_t w3) {
    asm volatile("st.global.cs.v4.u64 [%0], {%1,%2,%3,%4};" ::"l"(p), "l"(w0), "l"(w1), "l"(w2), "l"(w3)
                 : "memory");
}

template <typename T, int K>
__device__ __forceinline__ void load_chunk(const T* p, T (&x)[K]) {
    uint64_t w[8];
    ld32B(p, w[0], w[1], w[2], w[3]);
    ld32B(reinterpret_cast<const char*>(p) + 32, w[4], w[5], w[6], w[7]);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        if constexpr (sizeof(T) == 8) {
            x[i] = w[i];
        } else {
            x[2 * i] = (uint32_t)w[i];
            x[2 * i + 1] = (uint32_t)(w[i] >> 32);
        }
    }
}

template <typename T, int K>
__device__ __forceinline__ void store_chunk(T* p, const T (&x)[K]) {
    uint64_t w[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        if constexpr (sizeof(T) == 8) w[i] = x[i];
        else w[i] = (uint64_t)x[2 * i] | ((uint64_t)x[2 * i + 1] << 32);
    }
    st32B(p, w[0], w[1], w[2], w[3]);
    st32B(reinterpret_cast<char*>(p) + 32, w[4], w[5], w[6], w[7]);
}

template <int OP, typename T, int K>
__device__ __forceinline__ uint32_t chunk_chain(T (&x)[K], const T (&y)[K], uint32_t c) {
#pragma unroll
    for (int g = 0; g < K / 8; g++) {
        T(&xg)[8] = *reinterpret_cast<T(*)[8]>(x + 8 * g);
        const T(&yg)[8] = *reinterpret_cast<const T(*)[8]>(y + 8 * g);
        c = OP == OP_ADD ? chain_add8(xg, yg, c) : chain_sub8(xg, yg, c);
    }
    return c;
}

template <typename T, int W, int OP>
__global__ void __launch_bounds__(W * 32, 1024 / (W * 32))
addsub_chunk_kernel(const T* a, const T* b, T* r, uint8_t* sign_out, uint32_t cpi, uint64_t n, uint32_t ipt,
                    uint64_t ntiles) {
    constexpr int K = 64 / sizeof(T);
    constexpr int NCH = (OP == OP_SUB) ? 2 : 1;
    __shared__ uint32_t s_gp[NCH][W];   // per-warp composite, bit0 = g, bit1 = p
    __shared__ uint32_t s_first[W];     // 1 if the warp's first chunk starts an instance
    __shared__ uint8_t s_sign[(OP == OP_SUB) ? W * 32 : 1];

    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t q = threadIdx.x / cpi;          // instance within the tile
    const uint32_t pos = threadIdx.x - q * cpi;    // chunk within the instance

    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t inst0 = tile * (uint64_t)ipt;
        const uint64_t left = n - inst0;
        const uint32_t ninst = left < ipt ? (uint32_t)left : ipt;
        const bool valid = q < ninst;
        const uint64_t off = (inst0 * cpi + threadIdx.x) * (uint64_t)K;

        T x[K], y[K];
        if (valid) {
            load_chunk<T, K>(a + off, x);
            load_chunk<T, K>(b + off, y);
        } else {
#pragma unroll
            for (int e = 0; e < K; e++) x[e] = y[e] = 0;
        }

        // pass 1: the lane's carry out with carry-in 0, and whether a carry-in passes
        uint32_t g, p;
        {
            T t[K];
#pragma unroll
            for (int e = 0; e < K; e++) t[e] = x[e];
            g = chunk_chain<OP, T, K>(t, y, 0u);
            T acc = OP == OP_ADD ? (T)~(T)0 : (T)0;
#pragma unroll
            for (int e = 0; e < K; e++) {
                if (OP == OP_ADD) acc &= x[e] ^ y[e];
                else acc |= x[e] ^ y[e];
            }
            p = OP == OP_ADD ? (acc == (T)~(T)0) : (acc == 0);
            if (!valid) g = p = 0;
        }

        const uint32_t S = __ballot_sync(0xffffffffu, valid && pos == 0);
        const uint32_t kill = S >> 1;   // lane t+1 starts an instance: no carry out of lane t
        uint32_t A[NCH], B[NCH];
        A[0] = __ballot_sync(0xffffffffu, g | p) & ~kill;
        B[0] = __ballot_sync(0xffffffffu, g) & ~kill;
        if constexpr (OP == OP_SUB) {
            const uint32_t g2 = (valid && !g && !p) ? 1u : 0u;   // b - a borrows out of this lane
            A[1] = __ballot_sync(0xffffffffu, g2 | p) & ~kill;
            B[1] = __ballot_sync(0xffffffffu, g2) & ~kill;
        }
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                const uint32_t g0 = warp_carry_resolve(A[c], B[c], 0).cout;
                const uint32_t g1 = warp_carry_resolve(A[c], B[c], 1).cout;
                s_gp[c][warp] = g0 | ((g1 & ~g0) << 1);
            }
            s_first[warp] = S & 1u;
        }
        __syncthreads();

        // carry into this warp (ballot over the preceding warps), then into this lane
        uint32_t cl[NCH];
        {
            const bool before = lane < warp;
            const bool killed = before && s_first[lane + 1 < W ? lane + 1 : 0];
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                const uint32_t gp = before ? s_gp[c][lane] : 0u;
                const bool live = before && !killed;
                const uint32_t A2 = __ballot_sync(0xffffffffu, live && (gp & 3u));
                const uint32_t B2 = __ballot_sync(0xffffffffu, live && (gp & 1u));
                uint32_t cin = (warp_carry_resolve(A2, B2, 0).carries >> warp) & 1u;
                if (S & 1u) cin = 0;
                cl[c] = (warp_carry_resolve(A[c], B[c], cin).carries >> lane) & 1u;
            }
        }

        if constexpr (OP == OP_SUB) {
            if (valid && pos == cpi - 1) {
                const uint8_t sg = (uint8_t)(g | (p & cl[0]));
                s_sign[q] = sg;
                if (sign_out) sign_out[inst0 + q] = sg;
            }
            __syncthreads();
        }

        // pass 2: the chain with the resolved carry-in
        if (valid) {
            if constexpr (OP == OP_ADD) {
                chunk_chain<OP_ADD, T, K>(x, y, cl[0]);
            } else {
                const bool neg = s_sign[q] != 0;
                chunk_chain<OP_SUB, T, K>(x, y, neg ? 1u - cl[1] : cl[0]);
                if (neg) {
#pragma unroll
                    for (int e = 0; e < K; e++) x[e] = ~x[e];
                }
            }
            store_chunk<T, K>(r + off, x);
        }
        __syncthreads();   // shared state is rewritten by the next tile
    }
}

// ---------------------------------------------------------------------------
// Fused add chain, the reference's "ten additions" benchmark
// (baddKer1Bench, cuda/ker-add.cu.h:88-112; the thesis's 10(u+v),
// thesis/sections/performance.tex:28-36): r1 = a + b, then p-1 times
// r = r1 + r, i.e. r = p (a + b) mod B^m.  Each step is a full addition with
// its own carry resolution; r1 and r stay in registers between steps and
// touch HBM once each way.  Chunked layout as addsub_chunk_kernel.
// ---------------------------------------------------------------------------
template <typename T, int W>
__global__ void __launch_bounds__(W * 32, 1024 / (W * 32))
addchain_chunk_kernel(const T* a, const T* b, T* r, uint32_t cpi, uint64_t n, uint32_t ipt, uint64_t ntiles,
                      uint32_t steps) {
    constexpr int K = 64 / sizeof(T);
    __shared__ uint32_t s_gp[W];
    __shared__ uint32_t s_first[W];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t q = threadIdx.x / cpi;
    const uint32_t pos = threadIdx.x - q * cpi;

    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t inst0 = tile * (uint64_t)ipt;
        const uint64_t left = n - inst0;
        const uint32_t ninst = left < ipt ? (uint32_t)left : ipt;
        const bool valid = q < ninst;
        const uint64_t off = (inst0 * cpi + threadIdx.x) * (uint64_t)K;
        T x[K], y[K];
        if (valid) {
            load_chunk<T, K>(a + off, x);
            load_chunk<T, K>(b + off, y);
        } else {
#pragma unroll
            for (int e = 0; e < K; e++) x[e] = y[e] = 0;
        }
        const uint32_t S = __ballot_sync(0xffffffffu, valid && pos == 0);
        const uint32_t kill = S >> 1;
        for (uint32_t step = 0; step < steps; step++) {
            if (step == 1) {   // y = r1 = a + b from now on
#pragma unroll
                for (int e = 0; e < K; e++) y[e] = x[e];
            }
            uint32_t g, p;
            {
                T t[K];
#pragma unroll
                for (int e = 0; e < K; e++) t[e] = x[e];
                g = chunk_chain<OP_ADD, T, K>(t, y, 0u);
                T acc = (T)~(T)0;
#pragma unroll
                for (int e = 0; e < K; e++) acc &= x[e] ^ y[e];
                p = acc == (T)~(T)0;
                if (!valid) g = p = 0;
            }
            const uint32_t A = __ballot_sync(0xffffffffu, g | p) & ~kill;
            const uint32_t B = __ballot_sync(0xffffffffu, g) & ~kill;
            if (lane == 0) {
                const uint32_t g0 = warp_carry_resolve(A, B, 0).cout;
                const uint32_t g1 = warp_carry_resolve(A, B, 1).cout;
                s_gp[warp] = g0 | ((g1 & ~g0) << 1);
                s_first[warp] = S & 1u;
            }
            __syncthreads();
            const bool before = lane < warp;
            const bool killed = before && s_first[lane + 1 < W ? lane + 1 : 0];
            const uint32_t gp = before ? s_gp[lane] : 0u;
            const bool live = before && !killed;
            const uint32_t A2 = __ballot_sync(0xffffffffu, live && (gp & 3u));
            const uint32_t B2 = __ballot_sync(0xffffffffu, live && (gp & 1u));
            uint32_t cin = (warp_carry_resolve(A2, B2, 0).carries >> warp) & 1u;
            if (S & 1u) cin = 0;
            const uint32_t cl = (warp_carry_resolve(A, B, cin).carries >> lane) & 1u;
            if (valid) chunk_chain<OP_ADD, T, K>(x, y, cl);
            __syncthreads();   // s_gp is rewritten by the next step
        }
        if (valid) store_chunk<T, K>(r + off, x);
    }
}

template <typename T, int W>
static bi_status launch_addchain_cfg(const T* a, const T* b, T* r, uint32_t m, uint64_t n, uint32_t steps,
                                     cudaStream_t st) {
    constexpr uint32_t K = 64 / sizeof(T);
    const uint32_t cpi = m / K;
    const uint32_t ipt = (W * 32) / cpi;
    const uint64_t ntiles = (n + ipt - 1) / ipt;
    const unsigned grid = (unsigned)(ntiles < (1ull << 30) ? ntiles : (1ull << 30));
    addchain_chunk_kernel<T, W><<<grid, W * 32, 0, st>>>(a, b, r, cpi, n, ipt, ntiles, steps);
    return check_launch("add chain kernel");
}

template <typename T, int W, int OP>
static bi_status launch_chunk_cfg(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                                  cudaStream_t st) {
    constexpr uint32_t K = 64 / sizeof(T);
    const uint32_t cpi = m / K;
    const uint32_t ipt = (W * 32) / cpi;
    if (ipt == 0) return set_error(BI_EUNSUPPORTED, "m=%u exceeds the add/sub tile", m);
    const uint64_t ntiles = (n + ipt - 1) / ipt;
    const uint64_t maxgrid = 1ull << 30;
    const unsigned grid = (unsigned)(ntiles < maxgrid ? ntiles : maxgrid);
    addsub_chunk_kernel<T, W, OP><<<grid, W * 32, 0, st>>>(a, b, r, sign, cpi, n, ipt, ntiles);
    return check_launch(OP == OP_ADD ? "add kernel" : "sub kernel");
}

template <typename T, int OP>
static bi_status launch_chunk(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                              cudaStream_t st) {
    constexpr uint32_t K = 64 / sizeof(T);
    if (m <= 8 * 32 * K) return launch_chunk_cfg<T, 8, OP>(a, b, r, sign, m, n, st);
    if (m <= 16 * 32 * K) return launch_chunk_cfg<T, 16, OP>(a, b, r, sign, m, n, st);
    return launch_chunk_cfg<T, 32, OP>(a, b, r, sign, m, n, st);
}

// ---------------------------------------------------------------------------
// Host launch: pick the tile shape for m (the tile must hold one instance).
// ---------------------------------------------------------------------------
template <typename T, int WARPS, int ROWS, int VEC, int OP>
static bi_status launch_cfg(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                            cudaStream_t st) {
    constexpr uint32_t TILE = WARPS * ROWS * 32 * VEC;
    // an unaligned instance start costs up to VEC-1 limbs of slack in the tile
    const bool aligned_starts = (m % VEC) == 0;
    const uint32_t room = aligned_starts ? TILE : TILE - (VEC - 1);
    uint32_t ipt = room / m;
    if (ipt == 0) return set_error(BI_EUNSUPPORTED, "m=%u exceeds the add/sub tile", m);
    const uint64_t ntiles = (n + ipt - 1) / ipt;
    const uint64_t maxgrid = 1ull << 30;
    const unsigned grid = (unsigned)(ntiles < maxgrid ? ntiles : maxgrid);
    addsub_kernel<T, WARPS, ROWS, VEC, OP><<<grid, WARPS * 32, 0, st>>>(a, b, r, sign, m, n, ipt,
                                                                         FastDiv(m), ntiles);
    return check_launch(OP == OP_ADD ? "add kernel" : "sub kernel");
}

template <typename T, int VEC, int OP>
static bi_status launch_vec(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                            cudaStream_t st) {
    constexpr uint32_t ROWL = 32 * VEC;
    const uint32_t need = m + (m % VEC ? VEC - 1 : 0);
    if (need <= 8 * 4 * ROWL) return launch_cfg<T, 8, 4, VEC, OP>(a, b, r, sign, m, n, st);
    if (need <= 16 * 4 * ROWL) return launch_cfg<T, 16, 4, VEC, OP>(a, b, r, sign, m, n, st);
    return launch_cfg<T, 16, 8, VEC, OP>(a, b, r, sign, m, n, st);
}

// Largest instance of the 16-byte path: a 16-warp x 8-row tile.
template <typename T>
static uint32_t max_limbs() {
    return 16 * 8 * 32 * (16 / sizeof(T));
}

// host_link: the buffers are pinned host memory read over the CPU-GPU link,
// where the 16-byte row kernel's fully coalesced 512-byte warp accesses run
// about twice as fast as the chunked kernel's strided 32-byte ones.
template <typename T, int OP>
static bi_status addsub(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                        bi_stream s, bool host_link = false) {
    if (n == 0) return BI_OK;
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    if ((uint64_t)n * m / m != n || n * (uint64_t)m > (1ull << 46))
        return set_error(BI_EINVAL, "n*m too large");
    cudaStream_t st = (cudaStream_t)s;
    const bool vec32 = ((uintptr_t)a | (uintptr_t)b | (uintptr_t)r) % 32 == 0;
    constexpr uint32_t KC = 64 / sizeof(T);
    if (!host_link && vec32 && m % KC == 0 && m <= 32 * 32 * KC)
        return launch_chunk<T, OP>(a, b, r, sign, m, n, st);
    const bool vec16 = ((uintptr_t)a | (uintptr_t)b | (uintptr_t)r) % 16 == 0;
    if (vec16) {
        if (m > max_limbs<T>()) return set_error(BI_EUNSUPPORTED, "m=%u above %u limbs", m, max_limbs<T>());
        return launch_vec<T, 16 / sizeof(T), OP>(a, b, r, sign, m, n, st);
    }
    if (m > max_limbs<T>() / (16 / sizeof(T)))
        return set_error(BI_EUNSUPPORTED, "m=%u above the unaligned-buffer limit", m);
    return launch_vec<T, 1, OP>(a, b, r, sign, m, n, st);
}

// r = p (a + b) mod B^m by p chained additions (see addchain_chunk_kernel);
// sizes the chunked kernel cannot take run as p separate launches into r
// (which then must not alias a or b).
template <typename T>
static bi_status add_chain(const T* a, const T* b, T* r, uint32_t m, uint64_t n, uint32_t steps, bi_stream s) {
    if (n == 0) return BI_OK;
    if (steps == 0) return set_error(BI_EINVAL, "add chain: p must be >= 1");
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    if ((uint64_t)n * m > (1ull << 46)) return set_error(BI_EINVAL, "n*m too large");
    constexpr uint32_t KC = 64 / sizeof(T);
    cudaStream_t st = (cudaStream_t)s;
    if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)r) % 32 == 0 && m % KC == 0 && m <= 32 * 32 * KC) {
        if (m <= 8 * 32 * KC) return launch_addchain_cfg<T, 8>(a, b, r, m, n, steps, st);
        if (m <= 16 * 32 * KC) return launch_addchain_cfg<T, 16>(a, b, r, m, n, steps, st);
        return launch_addchain_cfg<T, 32>(a, b, r, m, n, steps, st);
    }
    if (steps > 1 && (r == a || r == b)) return set_error(BI_EINVAL, "add chain: r must not alias a or b at this size");
    BI_RETURN_IF((addsub<T, OP_ADD>(a, b, r, nullptr, m, n, s)));   // r1
    for (uint32_t k = 1; k < steps; k++) {
        // r = r1 + r with r1 = a + b recomputed on the fly: r += a, then r += b
        BI_RETURN_IF((addsub<T, OP_ADD>(r, a, r, nullptr, m, n, s)));
        BI_RETURN_IF((addsub<T, OP_ADD>(r, b, r, nullptr, m, n, s)));
    }
    return BI_OK;
}

bi_status add_link_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return addsub<uint64_t, OP_ADD>(a, b, r, nullptr, m, n, s, true);
}
bi_status add_link_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return addsub<uint32_t, OP_ADD>(a, b, r, nullptr, m, n, s, true);
}
bi_status sub_link_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m, uint64_t n,
                       bi_stream s) {
    return addsub<uint64_t, OP_SUB>(a, b, r, sign, m, n, s, true);
}
bi_status sub_link_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* sign, uint32_t m, uint64_t n,
                       bi_stream s) {
    return addsub<uint32_t, OP_SUB>(a, b, r, sign, m, n, s, true);
}

}  // namespace bi

using namespace bi;

extern "C" {

uint32_t bi_max_limbs_addsub_u64(void) { return max_limbs<uint64_t>(); }
uint32_t bi_max_limbs_addsub_u32(void) { return max_limbs<uint32_t>(); }

bi_status bi_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n,
                     bi_stream s) {
    return addsub<uint64_t, OP_ADD>(a, b, r, nullptr, m, n, s);
}
bi_status bi_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n,
                     bi_stream s) {
    return addsub<uint32_t, OP_ADD>(a, b, r, nullptr, m, n, s);
}
bi_status bi_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m,
                     uint64_t n, bi_stream s) {
    return addsub<uint64_t, OP_SUB>(a, b, r, sign, m, n, s);
}
bi_status bi_sub_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* sign, uint32_t m,
                     uint64_t n, bi_stream s) {
    return addsub<uint32_t, OP_SUB>(a, b, r, sign, m, n, s);
}
bi_status bi_add_chain_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, uint32_t p,
                           bi_stream s) {
    return add_chain<uint64_t>(a, b, r, m, n, p, s);
}
bi_status bi_add_chain_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, uint32_t p,
                           bi_stream s) {
    return add_chain<uint32_t>(a, b, r, m, n, p, s);
}

}  // extern "C"
