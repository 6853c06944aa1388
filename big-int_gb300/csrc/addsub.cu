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

template <typename T, int OP>
static bi_status addsub(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, uint64_t n,
                        bi_stream s) {
    if (n == 0) return BI_OK;
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    if ((uint64_t)n * m / m != n || n * (uint64_t)m > (1ull << 46))
        return set_error(BI_EINVAL, "n*m too large");
    cudaStream_t st = (cudaStream_t)s;
    const bool vec16 = ((uintptr_t)a | (uintptr_t)b | (uintptr_t)r) % 16 == 0;
    if (vec16) {
        if (m > max_limbs<T>()) return set_error(BI_EUNSUPPORTED, "m=%u above %u limbs", m, max_limbs<T>());
        return launch_vec<T, 16 / sizeof(T), OP>(a, b, r, sign, m, n, st);
    }
    if (m > max_limbs<T>() / (16 / sizeof(T)))
        return set_error(BI_EUNSUPPORTED, "m=%u above the unaligned-buffer limit", m);
    return launch_vec<T, 1, OP>(a, b, r, sign, m, n, st);
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

}  // extern "C"
