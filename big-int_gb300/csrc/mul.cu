// mul.cu -- batched classical (quadratic) multiplication.
//
// Semantics: bi_mul_* keeps the reference's truncated product
// r = (a * b) mod B^m (convMul1..5, cuda/ker-mul.cu.h:147-666, whose result
// array has the inputs' size m, cuda/main.cu:291); bi_mulfull_* writes the
// full 2m-limb product, which the reference can only obtain by zero-padding
// its inputs to 2m limbs and launching at size 2m.
//
// Design (integer-pipe bound):
//   * Arithmetic is on 64-bit limbs (a u32 batch is viewed as pairs of u32
//     words): the probe in probe.cu measures mul.lo.u64 + mul.hi.u64 as the
//     fastest way to form word products on this GPU, and the additions of
//     the products go to the ALU pipe, which is otherwise idle.
//   * Each instance's operands are staged in shared memory (16 bytes of skew
//     after every C limbs keeps strided 16-byte loads conflict-free).
//   * The product's 2L columns are cut into windows of C columns.  A thread
//     accumulates one window at a time as a (C+2)-limb integer: every row i
//     adds a_i * (b_{k0-i}, ..., b_{k0-i+C-1}) with two add.cc carry chains
//     (low words, then high words), so each word product costs 2 multiplies
//     and 2 adds, with no per-column overflow bookkeeping.
//   * Load balance: low-half window w needs (w+1)*C rows, its mirror
//     L/C-1-w needs L-w*C; each thread takes such a pair (and likewise in
//     the high half), so every thread runs exactly L+C rows in lockstep --
//     the reference balances the same way with columns k and m-1-k
//     (ker-mul.cu.h:160-184), here at window granularity.
//   * The windows overlap by two limbs; a carry-lookahead across windows
//     (block_carry_in) merges them, as the reference's final baddKer3Run
//     merges its low/high/carry vectors (ker-mul.cu.h:588-645).
#include "mulcore.cuh"

namespace bi {

template <typename T, int C, bool FULL>
__global__ void __launch_bounds__(512)
mul_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ r, uint64_t n, MulGeom g,
           FastDiv lpdiv) {
    extern __shared__ __align__(16) uint64_t smem[];
    uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + (size_t)g.ipc * g.IS);
    const uint64_t inst0 = (uint64_t)blockIdx.x * g.ipc;
    auto load = [&](uint32_t li, uint32_t x, uint64_t& va, uint64_t& vb) {
        const uint64_t gi = inst0 + li;
        if (gi >= n) return;
        if constexpr (sizeof(T) == 8) {
            va = a[gi * g.m + x];
            vb = b[gi * g.m + x];
        } else {
            const uint64_t w0 = gi * g.m + 2 * x;
            va = a[w0];
            vb = b[w0];
            if (2 * x + 1 < g.m) {
                va |= (uint64_t)a[w0 + 1] << 32;
                vb |= (uint64_t)b[w0 + 1] << 32;
            }
        }
    };
    auto store = [&](uint32_t li, uint32_t x, uint64_t v) {
        const uint64_t gi = inst0 + li;
        if (gi >= n) return;
        if constexpr (sizeof(T) == 8) {
            r[gi * g.out_words + x] = v;
        } else {
            if (2 * x < g.out_words) r[gi * g.out_words + 2 * x] = (uint32_t)v;
            if (2 * x + 1 < g.out_words) r[gi * g.out_words + 2 * x + 1] = (uint32_t)(v >> 32);
        }
    };
    mul_cta<C>(g, smem, scratch, lpdiv, load, store);
}

// Fused multiply chain, the reference's "six multiplications" benchmark
// kernel (convMul5Bench, cuda/ker-mul.cu.h:668-695): r1 = a*b, then p-1
// times r = r1*r, every product truncated to m limbs -- (a*b)^p mod B^m.
// The first product and the running one stay in shared memory (`first`,
// `cur`, after the multiply's own area); only a, b and the final r touch HBM.
template <typename T>
__global__ void __launch_bounds__(512)
mulchain_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ r, uint64_t n, MulGeom g,
                FastDiv lpdiv, uint32_t steps) {
    extern __shared__ __align__(16) uint64_t smem[];
    uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + (size_t)g.ipc * g.IS);
    uint64_t* first = smem + (size_t)g.ipc * g.IS + 48;   // after 96 words of scratch
    uint64_t* cur = first + (size_t)g.ipc * g.L;
    const uint64_t inst0 = (uint64_t)blockIdx.x * g.ipc;
    // an odd u32 m: the u64 view's top limb keeps only its low word (mod B^m)
    const uint64_t topmask = (sizeof(T) == 4 && (g.m & 1)) ? 0xffffffffull : ~0ull;
    // step 0 reads a, b from global memory and fills first and cur; later
    // steps read first and cur and rewrite cur (one inlined multiply)
    for (uint32_t k = 0; k < steps; k++) {
        auto load = [&](uint32_t li, uint32_t x, uint64_t& va, uint64_t& vb) {
            if (k > 0) {
                va = first[(size_t)li * g.L + x];
                vb = cur[(size_t)li * g.L + x];
                return;
            }
            const uint64_t gi = inst0 + li;
            if (gi >= n) return;
            if constexpr (sizeof(T) == 8) {
                va = a[gi * g.m + x];
                vb = b[gi * g.m + x];
            } else {
                const uint64_t w0 = gi * g.m + 2 * x;
                va = a[w0];
                vb = b[w0];
                if (2 * x + 1 < g.m) {
                    va |= (uint64_t)a[w0 + 1] << 32;
                    vb |= (uint64_t)b[w0 + 1] << 32;
                }
            }
        };
        auto store = [&](uint32_t li, uint32_t x, uint64_t v) {
            if (x == g.L - 1) v &= topmask;
            if (k == 0) first[(size_t)li * g.L + x] = v;
            cur[(size_t)li * g.L + x] = v;
        };
        mul_cta<MUL_C>(g, smem, scratch, lpdiv, load, store);
    }
    // the final value to global memory
    for (uint32_t idx = threadIdx.x; idx < g.ipc * g.L; idx += blockDim.x) {
        const uint32_t li = idx / g.L, x = idx - li * g.L;
        const uint64_t gi = inst0 + li;
        if (gi >= n) continue;
        const uint64_t v = cur[idx];
        if constexpr (sizeof(T) == 8) {
            r[gi * g.m + x] = v;
        } else {
            r[gi * g.m + 2 * x] = (uint32_t)v;
            if (2 * x + 1 < g.m) r[gi * g.m + 2 * x + 1] = (uint32_t)(v >> 32);
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-level full product for small operands: G lanes per instance (G = the
// power of two >= L, several instances per warp when L < 32; written for
// P = Lpad / G column pairs per lane, which also covers L up to 128 with
// G = 32), no CTA barrier.  The library routes full products of
// L <= MUL_WARP_MAX_L = 32 here: faster than the CTA kernel at L = 32
// (2048 bits), slower at L = 64, where each lane's column loop costs more
// instructions per word product than the CTA kernel's row windows.  Operands padded to Lpad = G*P limbs sit in the
// warp's shared memory; lane t of an instance accumulates the product
// columns t + G*j, j < 2P, as 3-word sums (mul.lo/hi + add.cc chain),
// pairing low column j with high column 2P-1-j so every lane does
// G(2j+1) terms in phase j.  The column sums s_c = c0 + c1 B + c2 B^2 are
// folded into limbs by two additions row by row (c0 + c1 shifted one column,
// then + c2 shifted two), carries resolved with ballots within the instance.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mac3(uint64_t& c0, uint64_t& c1, uint64_t& c2, uint64_t x, uint64_t y) {
    asm("{\n\t.reg .u64 lo, hi;\n\t"
        "mul.lo.u64 lo, %3, %4;\n\tmul.hi.u64 hi, %3, %4;\n\t"
        "add.cc.u64 %0, %0, lo;\n\taddc.cc.u64 %1, %1, hi;\n\taddc.u64 %2, %2, 0;\n\t}"
        : "+l"(c0), "+l"(c1), "+l"(c2)
        : "l"(x), "l"(y));
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

template <typename T, int P, int G>
__global__ void __launch_bounds__(256)
mul_warp_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ r, uint64_t n, uint32_t m,
                uint32_t L) {
    extern __shared__ __align__(16) uint64_t smem[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t Lpad = G * P;
    const uint32_t ipw = 32 / G;                       // instances per warp
    const uint32_t lg = lane / G, t = lane - lg * G;   // instance within the warp, lane within it
    const uint32_t base = lg * G;
    uint64_t* sa = smem + ((size_t)warp * ipw + lg) * 2 * Lpad;
    uint64_t* sb = sa + Lpad;
    const uint32_t out_limbs = 2 * L;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t wi = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp; wi * ipw < n; wi += nwarps) {
        const uint64_t inst = wi * ipw + lg;
        const bool valid = inst < n;
        for (uint32_t x = t; x < Lpad; x += G) {
            uint64_t va = 0, vb = 0;
            if (valid && x < L) {
                if constexpr (sizeof(T) == 8) {
                    va = a[inst * m + x];
                    vb = b[inst * m + x];
                } else {
                    const uint64_t w0 = inst * m + 2 * x;
                    va = a[w0];
                    vb = b[w0];
                    if (2 * x + 1 < m) {
                        va |= (uint64_t)a[w0 + 1] << 32;
                        vb |= (uint64_t)b[w0 + 1] << 32;
                    }
                }
            }
            sa[x] = va;
            sb[x] = vb;
        }
        __syncwarp();
        uint64_t acc[2 * P][3];
#pragma unroll
        for (int j = 0; j < P; j++) {
            const uint32_t lo = t + G * j;                  // a low column ...
            const uint32_t hi = t + G * (2 * P - 1 - j);    // ... and its high partner (>= Lpad)
            const uint32_t hi_i0 = hi - Lpad + 1;           // first row of the high column
            const uint32_t len = G * (2 * j + 1);           // terms of both, the same in every lane
            uint64_t c0 = 0, c1 = 0, c2 = 0;
#pragma unroll
            for (uint32_t rr = 0; rr < len; rr++) {
                const bool low = rr <= lo;
                const uint32_t i = low ? rr : hi_i0 + (rr - lo - 1);
                const uint32_t col = low ? lo : hi;
                mac3(c0, c1, c2, sa[i], sb[col - i]);
                if (rr == lo) {
                    acc[j][0] = c0; acc[j][1] = c1; acc[j][2] = c2;
                    c0 = c1 = c2 = 0;
                }
            }
            acc[2 * P - 1 - j][0] = c0; acc[2 * P - 1 - j][1] = c1; acc[2 * P - 1 - j][2] = c2;
        }
        __syncwarp();   // the shared operands are rewritten by the next round
        // fold: row jj holds columns G*jj + t
        uint32_t cy1 = 0, cy2 = 0;                  // carries between rows (both additions)
        uint64_t prev1 = 0, prev2a = 0, prev2b = 0;  // c1 of column G*jj-1; c2 of columns G*jj-2, G*jj-1
#pragma unroll
        for (int jj = 0; jj < 2 * P; jj++) {
            // c1 of column c-1 and c2 of column c-2
            uint64_t s1 = __shfl_up_sync(0xffffffffu, acc[jj][1], 1, G);
            if (t == 0) s1 = prev1;
            uint64_t s2 = __shfl_up_sync(0xffffffffu, acc[jj][2], 2, G);
            if (t == 0) s2 = prev2a;
            else if (t == 1) s2 = prev2b;
            prev1 = __shfl_sync(0xffffffffu, acc[jj][1], base + G - 1);
            prev2a = __shfl_sync(0xffffffffu, acc[jj][2], base + G - 2);
            prev2b = __shfl_sync(0xffffffffu, acc[jj][2], base + G - 1);
            // y = c0 + s1
            const uint64_t y = acc[jj][0] + s1;
            uint32_t co;
            const uint32_t k1 = group_carry(y < s1, y == ~0ull, cy1, G, base, t, co);
            cy1 = co;
            const uint64_t y2 = y + k1;
            // v = y2 + s2
            const uint64_t v = y2 + s2;
            const uint32_t k2 = group_carry(v < s2, v == ~0ull, cy2, G, base, t, co);
            cy2 = co;
            const uint32_t c = G * jj + t;
            if (valid && c < out_limbs) {
                const uint64_t out = v + k2;
                if constexpr (sizeof(T) == 8) {
                    r[inst * out_limbs + c] = out;
                } else {
                    const uint64_t w0 = inst * (2ull * m) + 2 * c;
                    if (2 * c < 2 * m) r[w0] = (uint32_t)out;
                    if (2 * c + 1 < 2 * m) r[w0 + 1] = (uint32_t)(out >> 32);
                }
            }
        }
    }
}

template <typename T, int P, int G>
static bi_status mul_warp_launch(const T* a, const T* b, T* r, uint32_t m, uint64_t n, uint32_t L, cudaStream_t st) {
    constexpr uint32_t ipw = 32 / G;
    const uint64_t warps = (n + ipw - 1) / ipw;
    const uint64_t blocks = (warps + 7) / 8;
    const uint64_t cap = (uint64_t)num_sms() * 32;
    const size_t smem = (size_t)8 * ipw * 2 * G * P * 8;
    mul_warp_kernel<T, P, G><<<(unsigned)(blocks < cap ? blocks : cap), 256, smem, st>>>(a, b, r, n, m, L);
    return check_launch("mulfull warp kernel");
}

// Full products of u64-view size L <= MUL_WARP_MAX_L go to the warp kernel.
template <typename T>
static bi_status mul_warp(const T* a, const T* b, T* r, uint32_t m, uint64_t n, uint32_t L, cudaStream_t st) {
    if (L <= 2) return mul_warp_launch<T, 1, 2>(a, b, r, m, n, L, st);
    if (L <= 4) return mul_warp_launch<T, 1, 4>(a, b, r, m, n, L, st);
    if (L <= 8) return mul_warp_launch<T, 1, 8>(a, b, r, m, n, L, st);
    if (L <= 16) return mul_warp_launch<T, 1, 16>(a, b, r, m, n, L, st);
    return mul_warp_launch<T, 1, 32>(a, b, r, m, n, L, st);
}

// ---------------------------------------------------------------------------

constexpr uint32_t MUL_MAX_L = 4096;   // u64-view limbs per operand
constexpr uint32_t MUL_WARP_MAX_L = 32;    // full products up to here take the warp kernel

template <typename T, bool FULL>
static bi_status mul_launch(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    constexpr int C = MUL_C;
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    if (L > MUL_MAX_L) return set_error(BI_EUNSUPPORTED, "mul: m=%u above the supported size", m);
    if (FULL && L <= MUL_WARP_MAX_L) return mul_warp<T>(a, b, r, m, n, L, st);
    // at least two CTAs per SM when the batch is small: fewer instances per CTA
    const uint64_t fill = (n + 2ull * num_sms() - 1) / (2ull * num_sms());
    MulGeom g = mul_geometry(L, FULL, fill < 256 ? (uint32_t)(fill ? fill : 1) : 256u);
    g.m = m;
    g.out_words = FULL ? 2 * m : m;
    const uint32_t threads = (g.ipc * g.tpi + 31) / 32 * 32;
    const size_t smem = (size_t)g.ipc * g.IS * 8 + 3 * 32 * 4;
    if (smem > 227 * 1024) return set_error(BI_EUNSUPPORTED, "mul: m=%u needs too much shared memory", m);
    auto kern = mul_kernel<T, C, FULL>;
    cudaError_t e = smem_opt_in((const void*)kern, smem);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "mul: %s", cudaGetErrorString(e));
    const uint64_t blocks = (n + g.ipc - 1) / g.ipc;
    if (blocks > 0x7fffffffull) return set_error(BI_EINVAL, "mul: n too large");
    kern<<<(unsigned)blocks, threads, smem, st>>>(a, b, r, n, g, FastDiv(g.Lp));
    return check_launch(FULL ? "mulfull kernel" : "mul kernel");
}

template <typename T, bool FULL>
static bi_status mul_entry(const T* a, const T* b, T* r, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    return mul_launch<T, FULL>(a, b, r, m, n, (cudaStream_t)s);
}

template <typename T>
static bi_status mul_chain(const T* a, const T* b, T* r, uint32_t m, uint64_t n, uint32_t steps, bi_stream s) {
    if (n == 0) return BI_OK;
    if (steps == 0) return set_error(BI_EINVAL, "mul chain: p must be >= 1");
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    if (L > MUL_MAX_L) return set_error(BI_EUNSUPPORTED, "mul chain: m=%u above the supported size", m);
    const uint64_t fill = (n + 2ull * num_sms() - 1) / (2ull * num_sms());
    MulGeom g = mul_geometry(L, false, fill < 256 ? (uint32_t)(fill ? fill : 1) : 256u);
    g.m = m;
    g.out_words = m;
    const uint32_t threads = (g.ipc * g.tpi + 31) / 32 * 32;
    const size_t smem = (size_t)g.ipc * g.IS * 8 + 3 * 32 * 4 + 2 * (size_t)g.ipc * g.L * 8;
    if (smem > 227 * 1024) return set_error(BI_EUNSUPPORTED, "mul chain: m=%u needs too much shared memory", m);
    auto kern = mulchain_kernel<T>;
    cudaError_t e = smem_opt_in((const void*)kern, smem);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "mul chain: %s", cudaGetErrorString(e));
    const uint64_t blocks = (n + g.ipc - 1) / g.ipc;
    if (blocks > 0x7fffffffull) return set_error(BI_EINVAL, "mul chain: n too large");
    kern<<<(unsigned)blocks, threads, smem, (cudaStream_t)s>>>(a, b, r, n, g, FastDiv(g.Lp), steps);
    return check_launch("mul chain kernel");
}

}  // namespace bi

using namespace bi;

extern "C" {

bi_status bi_mul_chain_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, uint32_t p,
                           bi_stream s) {
    return mul_chain<uint64_t>(a, b, r, m, n, p, s);
}
bi_status bi_mul_chain_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, uint32_t p,
                           bi_stream s) {
    return mul_chain<uint32_t>(a, b, r, m, n, p, s);
}

uint32_t bi_max_limbs_mul_u64(void) { return MUL_MAX_L; }
uint32_t bi_max_limbs_mul_u32(void) { return 2 * MUL_MAX_L; }

bi_status bi_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return mul_entry<uint64_t, false>(a, b, r, m, n, s);
}
bi_status bi_mul_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return mul_entry<uint32_t, false>(a, b, r, m, n, s);
}
bi_status bi_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n,
                         bi_stream s) {
    return mul_entry<uint64_t, true>(a, b, r, m, n, s);
}
bi_status bi_mulfull_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n,
                         bi_stream s) {
    return mul_entry<uint32_t, true>(a, b, r, m, n, s);
}

}  // extern "C"
