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
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "mulcore.cuh"
#include "multhread.cuh"
#include "mulwarp.cuh"

namespace bi {

constexpr uint32_t MUL_CTA_MAX_THREADS = 512;   // the CTA multiply's launch bound

template <typename T, int C, bool FULL>
__global__ void __launch_bounds__(MUL_CTA_MAX_THREADS)
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
// Warp-level full product for small operands on 32-bit words (mulwarp.cuh):
// the library routes full products of 25 to 32 64-bit limbs (49 to 64
// 32-bit words) here, for both limb types, unless a tuning says otherwise;
// smaller ones go to the thread kernel above.
// ---------------------------------------------------------------------------

// word x (32-bit) of operand row p with `words` words
template <typename T>
__device__ __forceinline__ uint32_t word32(const T* p, uint32_t words, uint32_t x) {
    if (x >= words) return 0;
    if constexpr (sizeof(T) == 8) return (uint32_t)(p[x >> 1] >> (32 * (x & 1)));
    else return p[x];
}

template <typename T, int G>
__global__ void __launch_bounds__(MUL_WARP_CTA)
mul_warp_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ r, uint64_t n, uint32_t m) {
    constexpr uint32_t ipw = 32 / G;                   // instances per warp
    extern __shared__ __align__(16) uint32_t smw[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lg = lane / G, t = lane - lg * G;   // instance within the warp, lane within it
    uint32_t* sw = smw + ((size_t)warp * ipw + lg) * mul_warp_group_words<G>();
    const uint32_t words = sizeof(T) == 8 ? 2 * m : m;        // operand words
    const uint32_t out_words = 2 * words;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t wi = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp; wi * ipw < n; wi += nwarps) {
        const uint64_t inst = wi * ipw + lg;
        const bool valid = inst < n;
        const T* pa = a + inst * m;
        const T* pb = b + inst * m;
        mul_warp_group<G>(
            sw, t, lg * G,
            [&](uint32_t x, uint32_t& wa, uint32_t& wb) {
                wa = valid ? word32(pa, words, x) : 0;
                wb = valid ? word32(pb, words, x) : 0;
            },
            [&](uint32_t c, uint64_t out) {   // 64-bit limb c of the product
                if (!valid) return;
                if constexpr (sizeof(T) == 8) {
                    if (c < m * 2) r[inst * (2ull * m) + c] = out;
                } else {
                    const uint64_t w0 = inst * (2ull * m) + 2 * c;
                    if (2 * c < out_words) r[w0] = (uint32_t)out;
                    if (2 * c + 1 < out_words) r[w0 + 1] = (uint32_t)(out >> 32);
                }
            });
    }
}

template <typename T, int G>
static bi_status mul_warp_launch(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    constexpr uint32_t ipw = 32 / G;
    constexpr uint32_t WPB = MUL_WARP_CTA / 32;   // warps per CTA
    const uint64_t warps = (n + ipw - 1) / ipw;
    const uint64_t blocks = (warps + WPB - 1) / WPB;
    const uint64_t cap = (uint64_t)num_sms() * 64;
    const size_t smem = (size_t)WPB * ipw * mul_warp_group_words<G>() * 4;
    mul_warp_kernel<T, G><<<(unsigned)(blocks < cap ? blocks : cap), MUL_WARP_CTA, smem, st>>>(a, b, r, n, m);
    return check_launch("mulfull warp kernel");
}

// Full products of at most 64 32-bit words per operand go to the warp kernel;
// G = the power of two >= half the operand's words.
template <typename T>
static bi_status mul_warp(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    const uint32_t half = sizeof(T) == 8 ? m : (m + 1) / 2;
    if (half <= 2) return mul_warp_launch<T, 2>(a, b, r, m, n, st);
    if (half <= 4) return mul_warp_launch<T, 4>(a, b, r, m, n, st);
    if (half <= 8) return mul_warp_launch<T, 8>(a, b, r, m, n, st);
    if (half <= 16) return mul_warp_launch<T, 16>(a, b, r, m, n, st);
    return mul_warp_launch<T, 32>(a, b, r, m, n, st);
}

// ---------------------------------------------------------------------------
// One thread per instance for products (full or truncated) of at most
// MUL_THREAD_MAX_L 64-bit limbs (multhread.cuh): the library's default
// there, for both limb types.  A CTA moves mul_thread_cta<M>() instances' operands into shared memory
// with coalesced loads, each thread multiplies its own row in registers and
// leaves the product in shared memory, and the CTA writes the tile back with
// coalesced stores.  64-bit limbs (u64, and u32 batches of an even word count
// on 8-byte-aligned buffers, which are the same bytes): rows at an odd stride
// of P limbs, so that consecutive threads' 8-byte reads of their own rows hit
// distinct banks.  u32 batches of an odd word count m = 2M - 1: the tile is
// kept as the words arrive (row stride m, odd, so each thread's 32-bit reads
// are conflict-free too) and the product at stride 2m words.
// ---------------------------------------------------------------------------
template <typename T, int M, bool FULL>
__global__ void __launch_bounds__(mul_thread_cta<M>())
mul_thread_kernel(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ r, uint64_t n, uint32_t m) {
    constexpr uint32_t CT = mul_thread_cta<M>();
    constexpr uint32_t P = (M % 2 == 0) ? M + 1 : M;    // operand row stride (limbs)
    constexpr uint32_t OL = FULL ? 2 * M : M;          // product limbs
    constexpr uint32_t Q = FULL ? 2 * M + 1 : P;       // product row stride (limbs)
    constexpr uint32_t S = (2 * P > Q ? 2 * P : Q);
    __shared__ uint64_t s[CT * S];                     // operands a | b, then the products
    uint32_t* sw = reinterpret_cast<uint32_t*>(s);     // the same, as 32-bit words
    const uint32_t tid = threadIdx.x;
    for (uint64_t base = (uint64_t)blockIdx.x * CT; base < n; base += (uint64_t)gridDim.x * CT) {
        const uint32_t rows = (uint32_t)(n - base < CT ? n - base : CT);
        uint64_t x[M], y[M];
        if constexpr (sizeof(T) == 8) {
            const T* ga = a + base * M;
            const T* gb = b + base * M;
            for (uint32_t k = tid; k < rows * M; k += CT) {
                const uint32_t row = k / M, col = k - row * M;
                s[row * P + col] = ga[k];
                s[CT * P + row * P + col] = gb[k];
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < M; ++i) {
                x[i] = s[tid * P + i];
                y[i] = s[CT * P + tid * P + i];
            }
        } else {
            constexpr uint32_t BOFF = CT * 2 * M;      // word offset of the b tile (m <= 2M words a row)
            const T* ga = a + base * m;
            const T* gb = b + base * m;
            for (uint32_t k = tid; k < rows * m; k += CT) {
                sw[k] = ga[k];
                sw[BOFF + k] = gb[k];
            }
            __syncthreads();
            const uint32_t* ra = sw + tid * m;
            const uint32_t* rb = sw + BOFF + tid * m;
#pragma unroll
            for (int i = 0; i < M; ++i) {
                const bool hi = i < M - 1 || 2 * M == m;   // word 2i + 1 exists
                x[i] = ra[2 * i] | (hi ? (uint64_t)ra[2 * i + 1] << 32 : 0ull);
                y[i] = rb[2 * i] | (hi ? (uint64_t)rb[2 * i + 1] << 32 : 0ull);
            }
        }
        __syncthreads();
        if constexpr (sizeof(T) == 8) {
            mul_thread_product<M, FULL>(x, y, [&](int c, uint64_t v) { s[tid * Q + c] = v; });
            __syncthreads();
            T* gr = r + base * OL;
            for (uint32_t k = tid; k < rows * OL; k += CT) {
                const uint32_t row = k / OL, col = k - row * OL;
                gr[k] = s[row * Q + col];
            }
        } else {
            const uint32_t ow = FULL ? 2 * m : m;      // product words
            uint32_t* rw = sw + tid * ow;
            mul_thread_product<M, FULL>(x, y, [&](int c, uint64_t v) {
                if (2u * c < ow) rw[2 * c] = (uint32_t)v;
                if (2u * c + 1 < ow) rw[2 * c + 1] = (uint32_t)(v >> 32);
            });
            __syncthreads();
            T* gr = r + base * ow;
            for (uint32_t k = tid; k < rows * ow; k += CT) gr[k] = sw[k];
        }
        __syncthreads();
    }
}

template <typename T, int M, bool FULL>
static bi_status mul_thread_launch(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    constexpr uint32_t CT = mul_thread_cta<M>();
    static const int occ = [] {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, mul_thread_kernel<T, M, FULL>, CT, 0) != cudaSuccess) {
            cudaGetLastError();                // not the launch's error: clear it, grid one CTA an SM
            o = 1;
        }
        return o > 0 ? o : 1;
    }();
    const uint64_t tiles = (n + CT - 1) / CT;
    const uint64_t cap = (uint64_t)num_sms() * (uint64_t)occ;
    mul_thread_kernel<T, M, FULL><<<(unsigned)(tiles < cap ? tiles : cap), CT, 0, st>>>(a, b, r, n, m);
    return check_launch(FULL ? "mulfull thread kernel" : "mul thread kernel");
}

// Products of at most MUL_THREAD_MAX_L (full) or MUL_THREAD_TRUNC_MAX_L
// (truncated) 64-bit limbs, one thread each.
template <typename T, bool FULL>
static bi_status mul_thread(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        // an even word count on 8-byte-aligned buffers: the same bytes as m/2 64-bit limbs
        if (m % 2 == 0 && ((uintptr_t)a | (uintptr_t)b | (uintptr_t)r) % 8 == 0)
            return mul_thread<uint64_t, FULL>(reinterpret_cast<const uint64_t*>(a), reinterpret_cast<const uint64_t*>(b),
                                              reinterpret_cast<uint64_t*>(r), m / 2, n, st);
    }
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    switch (L) {
        case 1: return mul_thread_launch<T, 1, FULL>(a, b, r, m, n, st);
        case 2: return mul_thread_launch<T, 2, FULL>(a, b, r, m, n, st);
        case 3: return mul_thread_launch<T, 3, FULL>(a, b, r, m, n, st);
        case 4: return mul_thread_launch<T, 4, FULL>(a, b, r, m, n, st);
        case 5: return mul_thread_launch<T, 5, FULL>(a, b, r, m, n, st);
        case 6: return mul_thread_launch<T, 6, FULL>(a, b, r, m, n, st);
        case 7: return mul_thread_launch<T, 7, FULL>(a, b, r, m, n, st);
        case 8: return mul_thread_launch<T, 8, FULL>(a, b, r, m, n, st);
        case 9: return mul_thread_launch<T, 9, FULL>(a, b, r, m, n, st);
        case 10: return mul_thread_launch<T, 10, FULL>(a, b, r, m, n, st);
        case 11: return mul_thread_launch<T, 11, FULL>(a, b, r, m, n, st);
        case 12: return mul_thread_launch<T, 12, FULL>(a, b, r, m, n, st);
        case 13: return mul_thread_launch<T, 13, FULL>(a, b, r, m, n, st);
        case 14: return mul_thread_launch<T, 14, FULL>(a, b, r, m, n, st);
        case 15: return mul_thread_launch<T, 15, FULL>(a, b, r, m, n, st);
        case 16: return mul_thread_launch<T, 16, FULL>(a, b, r, m, n, st);
        case 17: return mul_thread_launch<T, 17, FULL>(a, b, r, m, n, st);
        case 18: return mul_thread_launch<T, 18, FULL>(a, b, r, m, n, st);
        case 19: return mul_thread_launch<T, 19, FULL>(a, b, r, m, n, st);
        case 20: return mul_thread_launch<T, 20, FULL>(a, b, r, m, n, st);
        case 21: return mul_thread_launch<T, 21, FULL>(a, b, r, m, n, st);
        case 22: return mul_thread_launch<T, 22, FULL>(a, b, r, m, n, st);
        case 23: return mul_thread_launch<T, 23, FULL>(a, b, r, m, n, st);
        case 24: return mul_thread_launch<T, 24, FULL>(a, b, r, m, n, st);
        default: break;
    }
    if constexpr (!FULL) {
        switch (L) {
            case 25: return mul_thread_launch<T, 25, false>(a, b, r, m, n, st);
            case 26: return mul_thread_launch<T, 26, false>(a, b, r, m, n, st);
            case 27: return mul_thread_launch<T, 27, false>(a, b, r, m, n, st);
            case 28: return mul_thread_launch<T, 28, false>(a, b, r, m, n, st);
            case 29: return mul_thread_launch<T, 29, false>(a, b, r, m, n, st);
            case 30: return mul_thread_launch<T, 30, false>(a, b, r, m, n, st);
            case 31: return mul_thread_launch<T, 31, false>(a, b, r, m, n, st);
            case 32: return mul_thread_launch<T, 32, false>(a, b, r, m, n, st);
            default: break;
        }
    }
    return set_error(BI_EUNSUPPORTED, "mul thread kernel: m=%u above its size", m);
}

// ---------------------------------------------------------------------------

constexpr uint32_t MUL_MAX_L = 4096;   // u64-view limbs per operand
constexpr uint32_t MUL_WARP_MAX_L = 32;    // full products above MUL_THREAD_MAX_L up to here: the warp kernel

// ---------------------------------------------------------------------------
// Tiling of the CTA multiply: instances per CTA (ipc) and row slices per
// window pair (S).  Without a tuning entry the library's own choice applies
// (as many instances as fill MUL_CTA_THREADS threads, fewer when the batch is
// small, no slicing); bi_mul_autotune_* times the candidates on the caller's data and
// records the fastest here, per device, limb width, product kind and size.
// ---------------------------------------------------------------------------
struct MulTune {
    uint32_t ipc, S;
};

// The default CTA size: the autotuner's sweep on GB300 (full products, m =
// 64..2048 64-bit limbs) found 128-thread CTAs best or within 1 % of best at
// every size, 256-thread CTAs 2-7 % slower.
constexpr uint32_t MUL_CTA_THREADS = 128;

static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, uint32_t>, MulTune> g_tune;   // (device, limb bytes, full, L)

static bool mul_tuning_lookup(int limb_bytes, bool full, uint32_t L, MulTune* t) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(std::make_tuple(dev, limb_bytes, full ? 1 : 0, L));
    if (it == g_tune.end()) return false;
    *t = it->second;
    return true;
}

// The geometry of a tiling; false if it does not fit a CTA.
static bool mul_geom_tiled(uint32_t L, bool full, uint32_t ipc, uint32_t S, MulGeom* out) {
    if (ipc < 1 || S < 1 || S > 32 || (S & (S - 1))) return false;
    MulGeom g = mul_geometry(L, full, ipc);
    if (g.ipc != ipc) return false;              // more instances than 256 threads hold
    g.S = S;
    g.lgS = 0;
    while ((1u << g.lgS) < S) g.lgS++;
    if ((uint64_t)g.ipc * g.tpi * g.S > MUL_CTA_MAX_THREADS) return false;
    if (mul_smem_bytes(g) > 227 * 1024) return false;
    *out = g;
    return true;
}

template <typename T, bool FULL>
static MulGeom mul_geom_for(uint32_t L, uint64_t n) {
    MulTune t;
    MulGeom g;
    if (mul_tuning_lookup((int)sizeof(T), FULL, L, &t) && mul_geom_tiled(L, FULL, t.ipc, t.S, &g)) return g;
    // CTAs of about MUL_CTA_THREADS threads (as many instances as fill them),
    // fewer instances when the batch is small: at least two CTAs per SM
    const uint32_t tpi = mul_geometry(L, FULL, 1).tpi;
    uint32_t cap = MUL_CTA_THREADS / tpi;
    if (cap < 1) cap = 1;
    const uint64_t fill = (n + 2ull * num_sms() - 1) / (2ull * num_sms());
    if (fill < cap) cap = fill ? (uint32_t)fill : 1u;
    return mul_geometry(L, FULL, cap);
}

template <typename T, bool FULL>
static bi_status mul_launch_geom(const T* a, const T* b, T* r, uint32_t m, uint64_t n, MulGeom g, cudaStream_t st) {
    constexpr int C = MUL_C;
    g.m = m;
    g.out_words = FULL ? 2 * m : m;
    const uint32_t threads = mul_threads(g);
    const size_t smem = mul_smem_bytes(g);
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
static bi_status mul_launch(const T* a, const T* b, T* r, uint32_t m, uint64_t n, cudaStream_t st) {
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    if (L > MUL_MAX_L) return set_error(BI_EUNSUPPORTED, "mul: m=%u above the supported size", m);
    constexpr uint32_t THREAD_MAX = FULL ? MUL_THREAD_MAX_L : MUL_THREAD_TRUNC_MAX_L;
    if (L <= THREAD_MAX || (FULL && L <= MUL_WARP_MAX_L)) {
        // the thread kernel (L <= MUL_THREAD_MAX_L) or, for full products, the
        // warp kernel, unless a tuning picked one of them ({0, 1}, {0, 0}) or
        // a CTA tiling
        MulTune t;
        const bool tuned = mul_tuning_lookup((int)sizeof(T), FULL, L, &t);
        if (!tuned || t.ipc == 0) {
            const bool thread = tuned ? t.S == 1 : L <= THREAD_MAX;
            if (thread) return mul_thread<T, FULL>(a, b, r, m, n, st);
            if constexpr (FULL) return mul_warp<T>(a, b, r, m, n, st);
        }
    }
    return mul_launch_geom<T, FULL>(a, b, r, m, n, mul_geom_for<T, FULL>(L, n), st);
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
    MulGeom g = mul_geom_for<T, false>(L, n);   // the uniform multiply's tiling (128-thread CTAs unless tuned)
    g.S = 1;                                     // the chain kernel does not slice rows
    g.lgS = 0;
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

// Time every tiling that fits (ipc in 1, 2, 4, ..., S in 1, 2, 4) on the
// caller's operands, median of `reps` runs each, and record the fastest.
// For full products of at most MUL_WARP_MAX_L 64-bit limbs the warp kernel
// (32-bit words: mad.lo/madc.hi column sums) is a candidate too, recorded as
// {0, 0}, and for products (full or truncated) of at most MUL_THREAD_MAX_L
// limbs the thread kernel (64-bit limbs, one thread an instance), recorded
// as {0, 1}, beside the CTA
// kernel's tilings (64-bit limbs: row_mac8) -- the arithmetic's word width
// and the threads an instance are part of what is tuned.
template <typename T, bool FULL>
static bi_status mul_autotune(const T* a, const T* b, T* r, uint32_t m, uint64_t n, int reps, int* chosen,
                              cudaStream_t st) {
    if (chosen) chosen[0] = chosen[1] = 0;
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    const bool warp_ok = FULL && L <= MUL_WARP_MAX_L;
    std::vector<std::pair<uint32_t, uint32_t>> cands;
    if (warp_ok) cands.push_back({0, 0});
    if (L <= (FULL ? MUL_THREAD_MAX_L : MUL_THREAD_TRUNC_MAX_L)) cands.push_back({0, 1});
    for (uint32_t ipc = 1; ipc <= 64; ipc *= 2)
        for (uint32_t S = 1; S <= 4; S *= 2) {
            MulGeom g;
            if (mul_geom_tiled(L, FULL, ipc, S, &g) && (uint64_t)ipc <= n) cands.push_back({ipc, S});
        }
    if (cands.empty()) return set_error(BI_EUNSUPPORTED, "mul autotune: no tiling fits m=%u", m);
    // one run of a candidate: the warp kernel {0, 0}, the thread kernel {0, 1} or a CTA tiling
    auto run = [&](uint32_t ipc, uint32_t S) -> bi_status {
        if (ipc == 0) {
            if (S == 1) return mul_thread<T, FULL>(a, b, r, m, n, st);
            if constexpr (FULL) return mul_warp<T>(a, b, r, m, n, st);
            return set_error(BI_EINVAL, "mul autotune: no warp kernel for truncated products");
        }
        MulGeom g;
        mul_geom_tiled(L, FULL, ipc, S, &g);
        return mul_launch_geom<T, FULL>(a, b, r, m, n, g, st);
    };
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return set_error(BI_ECUDA, "mul autotune: %s", cudaGetErrorString(cudaGetLastError()));
    float best = 1e30f;
    MulTune pick = {cands[0].first, cands[0].second};
    bi_status st_out = BI_OK;
    for (const auto& c : cands) {
        std::vector<float> ts;
        for (int k = 0; k <= reps && st_out == BI_OK; k++) {   // the first run warms up
            cudaEventRecord(e0, st);
            st_out = run(c.first, c.second);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) st_out = set_error(BI_ECUDA, "mul autotune: %s",
                                                                            cudaGetErrorString(cudaGetLastError()));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (k > 0) ts.push_back(ms);
        }
        if (st_out != BI_OK) break;
        std::sort(ts.begin(), ts.end());
        const float med = ts[ts.size() / 2];
        if (med < best) {
            best = med;
            pick = {c.first, c.second};
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st_out != BI_OK) return st_out;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[std::make_tuple(dev, (int)sizeof(T), FULL ? 1 : 0, L)] = pick;
    }
    // leave r as one plain call with the chosen tiling writes it
    BI_RETURN_IF(run(pick.ipc, pick.S));
    if (chosen) {
        chosen[0] = (int)pick.ipc;
        chosen[1] = (int)pick.S;
    }
    return BI_OK;
}

template <typename T>
static bi_status mul_autotune_entry(const T* a, const T* b, T* r, uint32_t m, uint64_t n, int full, int reps,
                                    int* chosen, bi_stream s) {
    if (n == 0) return set_error(BI_EINVAL, "mul autotune: n must be >= 1");
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (reps < 1 || reps > 100) return set_error(BI_EINVAL, "mul autotune: reps must be in 1..100");
    if (!a || !b || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;
    if (L > MUL_MAX_L) return set_error(BI_EUNSUPPORTED, "mul: m=%u above the supported size", m);
    return full ? mul_autotune<T, true>(a, b, r, m, n, reps, chosen, (cudaStream_t)s)
                : mul_autotune<T, false>(a, b, r, m, n, reps, chosen, (cudaStream_t)s);
}

static bi_status mul_set_tuning(int limb_bytes, uint32_t m, int full, int ipc, int slices) {
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    const uint32_t L = limb_bytes == 8 ? m : (m + 1) / 2;
    if (L > MUL_MAX_L) return set_error(BI_EUNSUPPORTED, "mul: m=%u above the supported size", m);
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, limb_bytes, full ? 1 : 0, L);
    if (ipc == 0) {                                   // back to the library's own choice
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune.erase(key);
        return BI_OK;
    }
    if (ipc == -1) {                                  // a per-instance kernel: slices 0 warp, 1 thread
        const bool ok = (slices == 0 && full && L <= MUL_WARP_MAX_L) ||
                        (slices == 1 && L <= (full ? MUL_THREAD_MAX_L : MUL_THREAD_TRUNC_MAX_L));
        if (!ok) return set_error(BI_EINVAL, "mul tuning: no per-instance kernel %d for m=%u (full=%d)", slices, m, full);
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = {0u, (uint32_t)slices};
        return BI_OK;
    }
    MulGeom g;
    if (ipc < 0 || slices < 1 || !mul_geom_tiled(L, full != 0, (uint32_t)ipc, (uint32_t)slices, &g))
        return set_error(BI_EINVAL, "mul tuning: ipc=%d slices=%d does not fit a CTA for m=%u", ipc, slices, m);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = {(uint32_t)ipc, (uint32_t)slices};
    return BI_OK;
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

bi_status bi_mul_autotune_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, int full,
                              int reps, int* chosen, bi_stream s) {
    return mul_autotune_entry<uint64_t>(a, b, r, m, n, full, reps, chosen, s);
}
bi_status bi_mul_autotune_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, int full,
                              int reps, int* chosen, bi_stream s) {
    return mul_autotune_entry<uint32_t>(a, b, r, m, n, full, reps, chosen, s);
}
bi_status bi_mul_set_tuning_u64(uint32_t m, int full, int ipc, int slices) {
    return mul_set_tuning(8, m, full, ipc, slices);
}
bi_status bi_mul_set_tuning_u32(uint32_t m, int full, int ipc, int slices) {
    return mul_set_tuning(4, m, full, ipc, slices);
}

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
