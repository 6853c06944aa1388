// batch.cu -- uneven batches: instances of different operations and sizes in
// one graph-captured launch.
//
// The reference launches one kernel per (operation, size) with the size a
// template parameter (cuda/main.cu:476-515), so a batch of mixed sizes costs
// one launch per distinct size.  Here a plan groups the descriptors once:
//   * add/sub instances, largest first, go to a persistent kernel in which
//     each warp takes one instance at a time (warp_addsub: rows of 32 lanes x
//     16 bytes, carries resolved by ballots, a subtraction first finds the
//     larger operand from the top limb down as the reference's bsub does,
//     futhark/sub.fut:14-16) -- no shared memory and no CTA barrier, so any
//     size mix keeps the warps busy;
//   * multiplications are bucketed by padded size; a persistent CTA takes a
//     bucket item (as many instances as fit one CTA, mulcore.cuh);
//   * divisions go to persistent kernels by divisor size class: schoolbook
//     long division (divsmall.cuh) on one thread per instance for divisors
//     up to 4, 8 and 16 limbs, on one lane group per instance up to 32, 64,
//     ..., 1024 limbs (8 lanes up to 64 limbs, 16 up to 128, a warp above:
//     the register arrays sized for the class, the group size measured
//     fastest in the batch), and the shifted
//     inverse (divcore.cuh) on one 512-thread CTA per instance above -- and
//     for a class above 128 limbs with too few divisions to fill the GPU,
//     the crossover a uniform batch uses (div_use_long); most expensive
//     first within a class.
// The persistent kernels run concurrently on forked streams; the fork,
// the launches, the counter reset and the join are captured once into a CUDA
// graph and replayed by every bi_plan_execute.  Work is handed out with one
// atomic counter per kernel (no waiting on other CTAs).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "descio.cuh"
#include "divblock.cuh"
#include "divcore.cuh"
#include "divsmall.cuh"
#include "mulcore.cuh"
#include "mulwarp.cuh"
#include "warpops.cuh"

namespace bi {

constexpr uint32_t BATCH_MAX_LIMBS = 2048;   // per operand (64-bit limbs), add/sub and multiplies
constexpr uint32_t BATCH_DIV_MAX_M = 8192;   // a division's dividend limbs
constexpr uint32_t BATCH_DIV_MAX_MB = DIV_LONG_MAX_MV;   // and divisor limbs
constexpr uint32_t BATCH_SHINV_MAX_M = 2048; // the shifted inverse keeps its operands in shared memory

struct MulItem {
    uint32_t first;   // index into the mul list
    uint32_t count;   // instances in this item
    uint32_t Lp;      // padded limbs (geometry)
    uint32_t full;    // 1 = full product, 0 = truncated
};

struct BatchTune {
    int addsub_rows;      // rows of 32 lanes loaded per step (limbs per lane = rows * VEC)
    int addsub_vec;       // limbs per lane per row: 2 (16-byte accesses) or 1
    int mul_ipc_div;      // divide the default instances-per-CTA by this
    int mul_small_bits;   // word width of the full products of at most 32 limbs: 32 (the
                          // warp kernel, mulwarp.cuh) or 64 (the CTA kernel, mulcore.cuh)
};

// Full products of at most MULW_MAX_M 64-bit limbs form MULW_CLASSES classes
// for the warp kernel: class c takes m <= 2 << c on groups of G = 2 << c lanes.
constexpr int MULW_CLASSES = 5;
constexpr uint32_t MULW_MAX_M = 32;
inline int mulw_class(uint32_t m) {
    int c = 0;
    while ((2u << c) < m) c++;
    return c;
}

template <int VEC, int R>
__global__ void __launch_bounds__(256)
batch_addsub_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                    uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(counter, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= count) break;
        const bi_desc d = descs[list[idx]];
        const bool sub = d.op == BI_OP_SUB;
        uint8_t* sg = (sub && flags) ? flags + d.flag : nullptr;
        if (desc_w32(d)) {
            if (((d.a | d.b | d.r | d.m) & 1ull) == 0) {   // whole 64-bit limbs: the same bytes as m / 2 limbs
                const bi_desc e = {d.op, d.m / 2, d.m / 2, 0, d.a / 2, d.b / 2, d.r / 2, 0, d.flag};
                if (VEC == 2 && ((e.a | e.b | e.r) & 1ull) == 0)
                    warp_addsub<VEC, R>(in + e.a, in + e.b, out + e.r, sg, e.m, sub);
                else
                    warp_addsub<1, R>(in + e.a, in + e.b, out + e.r, sg, e.m, sub);
            } else {
                const uint32_t* in32 = reinterpret_cast<const uint32_t*>(in);
                warp_addsub<1, R, uint32_t>(in32 + d.a, in32 + d.b, reinterpret_cast<uint32_t*>(out) + d.r, sg, d.m,
                                            sub);
            }
        } else if (VEC == 2 && ((d.a | d.b | d.r) & 1ull) == 0) {
            // 16-byte accesses need even limb offsets (the arenas are 16-byte aligned)
            warp_addsub<VEC, R>(in + d.a, in + d.b, out + d.r, sg, d.m, sub);
        } else {
            warp_addsub<1, R>(in + d.a, in + d.b, out + d.r, sg, d.m, sub);
        }
    }
}

// ---------------------------------------------------------------------------
// persistent multiply and divide kernels
// ---------------------------------------------------------------------------
constexpr int BATCH_CTA = 256;

__global__ void __launch_bounds__(BATCH_CTA, 2)
batch_mul_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list,
                 const MulItem* __restrict__ items, uint32_t nitems, uint32_t* counter, const uint64_t* in,
                 uint64_t* out, int ipc_div) {
    extern __shared__ __align__(16) uint64_t smem[];
    __shared__ uint32_t s_item;
    __shared__ uint64_t s_a[BATCH_CTA], s_b[BATCH_CTA], s_r[BATCH_CTA];
    __shared__ uint32_t s_m[BATCH_CTA];   // elements of an operand (limbs or words)
    __shared__ uint8_t s_w[BATCH_CTA];    // 1: 32-bit words
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= nitems) break;
        const MulItem item = items[it];
        for (uint32_t i = threadIdx.x; i < item.count; i += blockDim.x) {
            const bi_desc& d = descs[list[item.first + i]];
            s_a[i] = d.a;
            s_b[i] = d.b;
            s_r[i] = d.r;
            s_m[i] = d.m;
            s_w[i] = desc_w32(d) ? 1 : 0;
        }
        uint32_t cap = item.count;
        const MulGeom g0 = mul_geometry(item.Lp, item.full != 0, cap);
        const MulGeom g = ipc_div > 1 && g0.ipc > 1 ? mul_geometry(item.Lp, item.full != 0, (g0.ipc + ipc_div - 1) / ipc_div)
                                                    : g0;
        __syncthreads();
        uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + (size_t)g.ipc * g.IS);
        const FastDiv lpdiv(g.Lp);
        const uint32_t full = item.full;
        // the item's instances in rounds of g.ipc
        for (uint32_t base = 0; base < item.count; base += g.ipc) {
            auto load = [&](uint32_t li, uint32_t x, uint64_t& va, uint64_t& vb) {
                const uint32_t k = base + li;
                if (k >= item.count) return;
                const bool w = s_w[k] != 0;
                va = ld64(in, s_a[k], s_m[k], w, x);
                vb = ld64(in, s_b[k], s_m[k], w, x);
            };
            auto store = [&](uint32_t li, uint32_t x, uint64_t v) {
                const uint32_t k = base + li;
                if (k >= item.count) return;
                st64(out, s_r[k], full ? 2 * s_m[k] : s_m[k], s_w[k] != 0, x, v);
            };
            mul_cta<MUL_C>(g, smem, scratch, lpdiv, load, store);
        }
        __syncthreads();   // s_item and the descriptor cache are rewritten next round
    }
}

// Small full products (class of G, at most G 64-bit limbs) on the warp
// kernel's 32-bit word arithmetic (mulwarp.cuh): G-lane groups, 32 / G
// instances a warp; lane 0 takes that many list entries at a time.
template <int G>
__global__ void __launch_bounds__(MUL_WARP_CTA)
batch_mulwarp_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                     uint32_t* counter, const uint64_t* in, uint64_t* out) {
    constexpr uint32_t ipw = 32 / G;
    extern __shared__ __align__(16) uint32_t smw[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lg = lane / G, t = lane - lg * G;
    uint32_t* sw = smw + ((size_t)warp * ipw + lg) * mul_warp_group_words<G>();
    for (;;) {
        uint32_t idx0 = 0;
        if (lane == 0) idx0 = atomicAdd(counter, ipw);
        idx0 = __shfl_sync(0xffffffffu, idx0, 0);
        if (idx0 >= count) break;
        const uint32_t idx = idx0 + lg;
        bi_desc d = {};                       // a group past the list: m = 0, loads zeros, stores nothing
        if (idx < count) d = descs[list[idx]];
        const bool w32 = desc_w32(d);
        const uint32_t words = w32 ? d.m : 2 * d.m;   // 32-bit words of an operand
        const uint32_t* pa = reinterpret_cast<const uint32_t*>(in) + (w32 ? d.a : 2 * d.a);
        const uint32_t* pb = reinterpret_cast<const uint32_t*>(in) + (w32 ? d.b : 2 * d.b);
        mul_warp_group<G>(
            sw, t, lg * G,
            [&](uint32_t x, uint32_t& wa, uint32_t& wb) {
                wa = x < words ? pa[x] : 0u;
                wb = x < words ? pb[x] : 0u;
            },
            [&](uint32_t c, uint64_t v) { st64(out, d.r, 2 * d.m, w32, c, v); });
    }
}

// division classes by divisor limbs: long division on threads (divisors up
// to 4, 8, 16 limbs), on warps or lane groups (up to 32, 64, 128, 256, 384,
// 512, 768, 1024 limbs: a divisor is right-aligned in its lanes' blocks,
// whose rows below it are zeros, so 384 takes 16-lane groups of 24 limbs
// and 768 a warp of 24 limbs a lane where 512 and 1024 take warps of 16 and
// 32; finer classes, of 20 and 28 limbs a lane, were 2 % slower on the
// 100000-instance batch: two more persistent kernels sharing the SMs),
// block long division on two warps (up
// to 2048 limbs) and four warps (up to 4096); the shifted inverse on
// 512-thread CTAs is the class that a size class above 128 limbs with few
// divisions runs as
constexpr int DIV_THREAD_CLASSES = 3, DIV_WARP_CLASSES = 8;
constexpr uint32_t DIV_WARP_CLASS_MAX_MV[DIV_WARP_CLASSES] = {32, 64, 128, 256, 384, 512, 768, 1024};
constexpr int DIV_CTA_CLASS = DIV_THREAD_CLASSES + DIV_WARP_CLASSES;
constexpr int DIV_BLK2_CLASS = DIV_CTA_CLASS + 1, DIV_BLK4_CLASS = DIV_CTA_CLASS + 2;
constexpr int DIV_CLASSES = DIV_CTA_CLASS + 3;
constexpr int DIV_CTA_THREADS = 512;
// add/sub, multiply, one per division class, one per warp-multiply class
constexpr int PLAN_KERNELS = 2 + DIV_CLASSES + MULW_CLASSES;
constexpr int PLAN_MULW0 = 2 + DIV_CLASSES;      // index of the first warp-multiply kernel

static inline int div_class(uint32_t mv) {
    if (mv <= 4) return 0;
    if (mv <= 8) return 1;
    if (mv <= 16) return 2;
    if (mv > (uint32_t)DIV_WARP_MAX_MV) return mv <= 2048 ? DIV_BLK2_CLASS : DIV_BLK4_CLASS;
    int c = 0;
    while (DIV_WARP_CLASS_MAX_MV[c] < mv) c++;
    return DIV_THREAD_CLASSES + c;
}

template <int MX>
__global__ void __launch_bounds__(DIV_THREAD_CTA)
batch_divthread_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                       uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u);   // 32 instances a warp
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) break;
        const uint32_t idx = base + lane;
        if (idx >= count) continue;
        const bi_desc d = descs[list[idx]];
        const bool w32 = desc_w32(d);
        auto lu = [&](uint32_t i) { return ld64(in, d.a, d.m, w32, i); };
        auto lv = [&](uint32_t i) { return ld64(in, d.b, d.mb, w32, i); };
        auto sq = [&](uint32_t i, uint64_t x) { st64(out, d.r, d.m, w32, i, x); };
        auto sr = [&](uint32_t i, uint64_t x) { st64(out, d.r2, d.mb, w32, i, x); };
        const uint8_t st = div_thread<MX>(
            m64(d), mb64(d), lu, lv, sq, sr);
        if (flags) flags[d.flag] = st;
    }
}

template <int VPL>
__device__ __forceinline__ void batch_divwarp_items(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list,
                                                    uint32_t count, uint32_t* counter, const uint64_t* in, uint64_t* out,
                                                    uint8_t* flags) {
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(counter, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= count) break;
        const bi_desc d = descs[list[idx]];
        const bool w32 = desc_w32(d);
        auto lu = [&](uint32_t i) { return ld64(in, d.a, d.m, w32, i); };
        auto lv = [&](uint32_t i) { return ld64(in, d.b, d.mb, w32, i); };
        auto sq = [&](uint32_t i, uint64_t x) { st64(out, d.r, d.m, w32, i, x); };
        auto sr = [&](uint32_t i, uint64_t x) { st64(out, d.r2, d.mb, w32, i, x); };
        const uint8_t st = div_warp<VPL>(
            m64(d), mb64(d), lu, lv, sq, sr);
        if (flags && lane == 0) flags[d.flag] = st;
    }
}

template <int VPL>
__global__ void __launch_bounds__(DIV_WARP_CTA)
batch_divwarp_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                     uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    batch_divwarp_items<VPL>(descs, list, count, counter, in, out, flags);
}

// Held to three CTAs (12 warps) an SM, for 24 limbs a lane (as the uniform
// entry's div_warp3_kernel): 168 registers instead of 194.
template <int VPL>
__global__ void __launch_bounds__(DIV_WARP_CTA, 3)
batch_divwarp3_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                      uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    batch_divwarp_items<VPL>(descs, list, count, counter, in, out, flags);
}

// Several divisions a warp, one per G-lane group (div_group): lane 0 takes
// 32 / G list entries at a time.
template <int VPL, int G>
__global__ void __launch_bounds__(DIV_WARP_CTA)
batch_divgroup_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                      uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    constexpr uint32_t ipw = 32 / G;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, ipw);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) break;
        const uint32_t idx = base + lane / G;
        const bool valid = idx < count;
        bi_desc d = {};
        if (valid) d = descs[list[idx]];
        const bool w32 = desc_w32(d);
        auto lu = [&](uint32_t i) { return ld64(in, d.a, d.m, w32, i); };
        auto lv = [&](uint32_t i) { return ld64(in, d.b, d.mb, w32, i); };
        auto sq = [&](uint32_t i, uint64_t x) { st64(out, d.r, d.m, w32, i, x); };
        auto sr = [&](uint32_t i, uint64_t x) { st64(out, d.r2, d.mb, w32, i, x); };
        const uint8_t st = div_group<VPL, G>(
            valid, valid ? m64(d) : 1u, valid ? mb64(d) : 1u, lu, lv, sq, sr);
        if (flags && valid && (lane & (G - 1)) == 0) flags[d.flag] = st;
    }
}

// At most 128 registers a thread, so 512 / THREADS CTAs fit an SM's register file.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 512 / THREADS)
batch_div_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                 uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    extern __shared__ __align__(16) uint64_t smem[];
    __shared__ uint32_t s_idx;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const bi_desc d = descs[list[idx]];
        const DivGeom g = div_geom(m64(d), mb64(d), 8);
        const bool w32 = desc_w32(d);
        auto lu = [&](uint32_t i) { return ld64(in, d.a, d.m, w32, i); };
        auto lv = [&](uint32_t i) { return ld64(in, d.b, d.mb, w32, i); };
        auto sq = [&](uint32_t i, uint64_t x) { st64(out, d.r, d.m, w32, i, x); };
        auto sr = [&](uint32_t i, uint64_t x) { st64(out, d.r2, d.mb, w32, i, x); };
        div_cta(
            g, smem, lu, lv, sq, sr,
            [&](uint8_t code) { if (flags) flags[d.flag] = code; });
    }
}

// ---------------------------------------------------------------------------
// host side: the plan
// ---------------------------------------------------------------------------
template <typename T>
static bi_status dev_upload(T** dst, const std::vector<T>& v, cudaStream_t s) {
    *dst = nullptr;
    if (v.empty()) return BI_OK;
    cudaError_t e = cudaMallocAsync((void**)dst, v.size() * sizeof(T), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? BI_ENOMEM : BI_ECUDA, "plan upload: %s",
                         cudaGetErrorString(e));
    }
    return BI_OK;
}

}  // namespace bi

using namespace bi;

// Divisions by 1025..4096-limb divisors: block long division (divblock.cuh)
// on the CTA's NW warps, one division at a time.
template <int NW>
__global__ void __launch_bounds__(32 * NW)
batch_divblk_kernel(const bi_desc* __restrict__ descs, const uint32_t* __restrict__ list, uint32_t count,
                    uint32_t* counter, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    __shared__ DivBlkShared<8, NW> sh;
    __shared__ uint32_t s_idx;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t idx = s_idx;
        __syncthreads();
        if (idx >= count) break;
        const bi_desc d = descs[list[idx]];
        const bool w32 = desc_w32(d);
        auto lu = [&](uint32_t i) { return ld64(in, d.a, d.m, w32, i); };
        auto lv = [&](uint32_t i) { return ld64(in, d.b, d.mb, w32, i); };
        auto sq = [&](uint32_t i, uint64_t x) { st64(out, d.r, d.m, w32, i, x); };
        auto sr = [&](uint32_t i, uint64_t x) { st64(out, d.r2, d.mb, w32, i, x); };
        const uint8_t st = div_blk<32, 8, NW>(
            m64(d), mb64(d), lu, lv, sq, sr, &sh);
        if (flags && threadIdx.x == 0) flags[d.flag] = st;
    }
}

struct bi_plan {
    int device = 0;
    uint64_t count = 0;
    bi_desc* d_descs = nullptr;
    uint32_t* d_addsub = nullptr;
    uint32_t* d_mul = nullptr;
    uint32_t* d_div = nullptr;          // division list: class 0, then 1, then 2
    MulItem* d_items = nullptr;         // every multiply, on the CTA kernel
    MulItem* d_items_large = nullptr;   // the multiplies the warp classes do not take
    uint32_t* d_mulw = nullptr;         // small full products: warp class 0, then 1, ...
    uint32_t* d_counters = nullptr;     // one per kernel (PLAN_KERNELS)
    uint32_t n_addsub = 0, n_mul = 0, n_items = 0, n_div = 0, n_items_large = 0, n_mulw_total = 0;
    uint32_t mulw_off[MULW_CLASSES] = {}, n_mulw[MULW_CLASSES] = {};
    uint32_t div_off[DIV_CLASSES] = {}, n_divc[DIV_CLASSES] = {};
    uint32_t max_mul_Lp_full = 0, max_mul_Lp_trunc = 0;
    uint64_t nflags = 0;                // flag-arena bytes the descriptors were checked against
    size_t mul_smem = 0, div_smem = 0, divc_smem[DIV_CLASSES] = {};
    BatchTune tune = {4, 2, 1, 32};
    cudaGraphExec_t exec = nullptr;
    const void* g_in = nullptr;
    void* g_out = nullptr;
    void* g_flags = nullptr;
    BatchTune g_tune = {0, 0, 0, 0};
    cudaStream_t cap = nullptr;
    cudaStream_t side[PLAN_KERNELS] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[PLAN_KERNELS] = {};
    std::mutex mu;
};

namespace bi {

static size_t mul_smem_for(const bi_plan* p, int ipc_div) {
    size_t best = 0;
    for (int full = 0; full < 2; full++) {
        const uint32_t Lp = full ? p->max_mul_Lp_full : p->max_mul_Lp_trunc;
        if (!Lp) continue;
        // every padded size up to the largest can appear; smaller sizes pack more instances
        for (uint32_t L = 2 * MUL_C; L <= Lp; L += 2 * MUL_C) {
            MulGeom g = mul_geometry(L, full != 0, 256);
            if (ipc_div > 1 && g.ipc > 1) g = mul_geometry(L, full != 0, (g.ipc + ipc_div - 1) / ipc_div);
            best = std::max(best, mul_smem_bytes(g));
        }
    }
    return best;
}

// The class of each division: by divisor size (div_class), except that a
// band of divisor sizes above 128 limbs (129-256, 257-512, 513-1024) with too
// few divisions for long division's throughput to win goes to the shifted
// inverse on CTAs: at most 2, 3 and 6 per SM in the band.  The band, not the
// class, is counted: the classes that split a band (384 and 512; 768 and
// 1024) each hold a share of its divisions, and counting them one by one
// sent classes of a 100000-instance batch that split the 513-1024 band more
// finely to the shifted inverse (15.9M -> 13.5M instances/s).  (Up to 128 limbs long division
// stays: beside the batch's other kernels its small lane groups pack where
// a CTA per division does not -- a 20000-instance batch ran 1.74 ms so and
// 1.94 ms with the uniform entry's crossover.)  map[c] is the class that
// size class c runs as.
static uint32_t div_band(uint32_t max_mv) { return max_mv <= 256 ? 256 : max_mv <= 512 ? 512 : 1024; }

static void div_class_map(const bi_desc* descs, const uint32_t* div, uint32_t n, int sms, int* map) {
    uint64_t cnt[DIV_CLASSES] = {};
    uint32_t max_m[DIV_CLASSES] = {};
    for (uint32_t k = 0; k < n; k++) {
        const int c = div_class(mb64(descs[div[k]]));
        cnt[c]++;
        max_m[c] = std::max(max_m[c], m64(descs[div[k]]));
    }
    for (int c = 0; c < DIV_CLASSES; c++) {
        map[c] = c;
        if (c >= DIV_THREAD_CLASSES && c < DIV_CTA_CLASS && max_m[c] <= BATCH_SHINV_MAX_M) {
            const uint32_t max_mv = DIV_WARP_CLASS_MAX_MV[c - DIV_THREAD_CLASSES];   // the class's largest divisor
            if (max_mv > 128) {
                const uint32_t band = div_band(max_mv);
                uint64_t band_cnt = 0;
                for (int b = DIV_THREAD_CLASSES; b < DIV_CTA_CLASS; b++) {
                    const uint32_t bmv = DIV_WARP_CLASS_MAX_MV[b - DIV_THREAD_CLASSES];
                    if (bmv > 128 && div_band(bmv) == band) band_cnt += cnt[b];
                }
                const uint64_t per_sm = band == 256 ? 2 : band == 512 ? 3 : 6;
                if (band_cnt <= per_sm * (uint64_t)sms) map[c] = DIV_CTA_CLASS;
            }
        }
    }
}

// Division order: by class, then most expensive first.
static bool div_before(const bi_desc& x, const bi_desc& y, const int* map) {
    const int cx = map[div_class(mb64(x))], cy = map[div_class(mb64(y))];
    if (cx != cy) return cx < cy;
    return (uint64_t)m64(x) * mb64(x) > (uint64_t)m64(y) * mb64(y);
}

// Per-class offsets, counts and shared memory of a division list sorted by div_before.
static void div_classes(bi_plan* p, const bi_desc* descs, const uint32_t* div, uint32_t n, const int* map) {
    p->div_smem = 0;
    for (int c = 0; c < DIV_CLASSES; c++) {
        p->div_off[c] = 0;
        p->n_divc[c] = 0;
        p->divc_smem[c] = 0;
    }
    for (uint32_t k = 0; k < n; k++) {
        const bi_desc& d = descs[div[k]];
        const int c = map[div_class(mb64(d))];
        if (p->n_divc[c]++ == 0) p->div_off[c] = k;
        if (c == DIV_CTA_CLASS) p->divc_smem[c] = std::max(p->divc_smem[c], div_smem_bytes(div_geom(m64(d), mb64(d), 8)));
        p->div_smem = std::max(p->div_smem, p->divc_smem[c]);
    }
}

enum { COMP_ADDSUB = 1, COMP_MUL = 2, COMP_DIV = 4, COMP_ALL = 7 };

struct Launch3 {
    unsigned grid[PLAN_KERNELS];
    size_t smem[PLAN_KERNELS];
};

static bi_status grid_for(const void* k, int threads, size_t smem, uint64_t work_ctas, int sms, unsigned* grid) {
    int occ = 1;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, smem) != cudaSuccess)
        return set_error(BI_ECUDA, "batch kernel setup: %s", cudaGetErrorString(cudaGetLastError()));
    *grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(work_ctas, (uint64_t)sms * (occ < 1 ? 1 : occ)));
    return BI_OK;
}

// The kernel of division class c (host-side function pointer) and its CTA width.
static const void* div_class_kernel(int c, int* threads) {
    *threads = c < DIV_THREAD_CLASSES ? DIV_THREAD_CTA : c < DIV_CTA_CLASS ? DIV_WARP_CTA
               : c == DIV_BLK2_CLASS ? 64 : c == DIV_BLK4_CLASS ? 128 : DIV_CTA_THREADS;
    switch (c) {
    case DIV_BLK2_CLASS: return (const void*)batch_divblk_kernel<2>;
    case DIV_BLK4_CLASS: return (const void*)batch_divblk_kernel<4>;
    case 0: return (const void*)batch_divthread_kernel<4>;
    case 1: return (const void*)batch_divthread_kernel<8>;
    case 2: return (const void*)batch_divthread_kernel<16>;
    case 3: return (const void*)batch_divgroup_kernel<4, 8>;
    case 4: return (const void*)batch_divgroup_kernel<8, 8>;
    case 5: return (const void*)batch_divgroup_kernel<8, 16>;
    case 6: return (const void*)batch_divwarp_kernel<8>;
    case 7: return (const void*)batch_divgroup_kernel<24, 16>;
    case 8: return (const void*)batch_divwarp_kernel<16>;
    case 9: return (const void*)batch_divwarp3_kernel<24>;
    case 10: return (const void*)batch_divwarp_kernel<32>;
    default: return (const void*)batch_div_kernel<DIV_CTA_THREADS>;
    }
}

// Whether tuning t sends the plan's small full products to the warp kernel.
static bool plan_small_on_warps(const bi_plan* p, const BatchTune& t) {
    return t.mul_small_bits == 32 && p->n_mulw_total > 0;
}

// The warp-multiply kernel of class c (host-side function pointer).
static const void* mulw_class_kernel(int c) {
    switch (c) {
    case 0: return (const void*)batch_mulwarp_kernel<2>;
    case 1: return (const void*)batch_mulwarp_kernel<4>;
    case 2: return (const void*)batch_mulwarp_kernel<8>;
    case 3: return (const void*)batch_mulwarp_kernel<16>;
    default: return (const void*)batch_mulwarp_kernel<32>;
    }
}

// Grid sizes and shared memory of the kernels for tuning t; sets the
// kernels' shared-memory limits (done outside any stream capture).
static bi_status prepare_launch(bi_plan* p, const BatchTune& t, Launch3* L) {
    const int sms = num_sms();
    const bool small_warp = plan_small_on_warps(p, t);
    const uint32_t n_items = small_warp ? p->n_items_large : p->n_items;
    L->grid[0] = (unsigned)std::min<uint64_t>((p->n_addsub + 7) / 8, (uint64_t)sms * 8);
    L->smem[0] = 0;
    L->smem[1] = mul_smem_for(p, t.mul_ipc_div);
    for (int c = 0; c < DIV_CLASSES; c++) {
        L->smem[2 + c] = p->divc_smem[c];
        L->grid[2 + c] = 0;
    }
    for (int c = 0; c < MULW_CLASSES; c++) {
        L->smem[PLAN_MULW0 + c] = 0;
        L->grid[PLAN_MULW0 + c] = 0;
    }
    int occ = 1;
    L->grid[1] = 0;
    if (n_items) {
        if (cudaFuncSetAttribute(batch_mul_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem[1]) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_mul_kernel, BATCH_CTA, L->smem[1]) != cudaSuccess)
            return set_error(BI_ECUDA, "batch mul kernel setup: %s", cudaGetErrorString(cudaGetLastError()));
        L->grid[1] = (unsigned)std::min<uint64_t>(n_items, (uint64_t)sms * (occ < 1 ? 1 : occ));
    }
    for (int c = 0; small_warp && c < MULW_CLASSES; c++) {
        const uint64_t n = p->n_mulw[c];
        if (!n) continue;
        const uint32_t G = 2u << c, ipw = 32 / G, warps = MUL_WARP_CTA / 32;
        const size_t smem = (size_t)warps * ipw * (3 * 2 * G) * sizeof(uint32_t);
        L->smem[PLAN_MULW0 + c] = smem;
        BI_RETURN_IF(grid_for(mulw_class_kernel(c), MUL_WARP_CTA, smem, (n + warps * ipw - 1) / (warps * ipw), sms,
                              &L->grid[PLAN_MULW0 + c]));
    }
    for (int c = 0; c < DIV_CLASSES; c++) {
        const uint64_t n = p->n_divc[c];
        if (!n) continue;
        int threads = 0;
        const void* k = div_class_kernel(c, &threads);
        // instances per CTA: one a thread, one a lane group (8, 16 or 32 lanes), one a CTA
        static constexpr uint32_t group_ipw[DIV_WARP_CLASSES] = {4, 4, 2, 1, 2, 1, 1, 1};
        const uint64_t per = c < DIV_THREAD_CLASSES ? (uint64_t)threads
                             : c < DIV_CTA_CLASS    ? (uint64_t)threads / 32 * group_ipw[c - DIV_THREAD_CLASSES]
                                                    : 1;
        BI_RETURN_IF(grid_for(k, threads, L->smem[2 + c], (n + per - 1) / per, sms, &L->grid[2 + c]));
    }
    return BI_OK;
}

// s[k] is the stream of kernel k (add/sub, multiply, then the division classes).
static bi_status launch_plan_kernels(bi_plan* p, const uint64_t* in, uint64_t* out, uint8_t* flags,
                                     const BatchTune& t, const Launch3& L, const cudaStream_t* s,
                                     int comps = COMP_ALL) {
    cudaStream_t s_add = s[0], s_mul = s[1];
    if (p->n_addsub && (comps & COMP_ADDSUB)) {
        const unsigned grid = L.grid[0];
        if (t.addsub_vec == 2 && t.addsub_rows == 4)
            batch_addsub_kernel<2, 4><<<grid, 256, 0, s_add>>>(p->d_descs, p->d_addsub, p->n_addsub, p->d_counters + 0, in, out, flags);
        else if (t.addsub_vec == 2 && t.addsub_rows == 2)
            batch_addsub_kernel<2, 2><<<grid, 256, 0, s_add>>>(p->d_descs, p->d_addsub, p->n_addsub, p->d_counters + 0, in, out, flags);
        else if (t.addsub_vec == 2)
            batch_addsub_kernel<2, 8><<<grid, 256, 0, s_add>>>(p->d_descs, p->d_addsub, p->n_addsub, p->d_counters + 0, in, out, flags);
        else
            batch_addsub_kernel<1, 4><<<grid, 256, 0, s_add>>>(p->d_descs, p->d_addsub, p->n_addsub, p->d_counters + 0, in, out, flags);
        BI_RETURN_IF(check_launch("batch add/sub kernel"));
    }
    if (comps & COMP_MUL) {
        const bool small_warp = plan_small_on_warps(p, t);
        const MulItem* items = small_warp ? p->d_items_large : p->d_items;
        const uint32_t n_items = small_warp ? p->n_items_large : p->n_items;
        if (n_items) {
            batch_mul_kernel<<<L.grid[1], BATCH_CTA, L.smem[1], s_mul>>>(p->d_descs, p->d_mul, items, n_items,
                                                                         p->d_counters + 1, in, out, t.mul_ipc_div);
            BI_RETURN_IF(check_launch("batch mul kernel"));
        }
        for (int c = 0; small_warp && c < MULW_CLASSES; c++) {
            const uint32_t n = p->n_mulw[c];
            if (!n) continue;
            const uint32_t* list = p->d_mulw + p->mulw_off[c];
            uint32_t* ctr = p->d_counters + PLAN_MULW0 + c;
            const unsigned grid = L.grid[PLAN_MULW0 + c];
            const size_t smem = L.smem[PLAN_MULW0 + c];
            cudaStream_t st = s[PLAN_MULW0 + c];
            switch (c) {
            case 0: batch_mulwarp_kernel<2><<<grid, MUL_WARP_CTA, smem, st>>>(p->d_descs, list, n, ctr, in, out); break;
            case 1: batch_mulwarp_kernel<4><<<grid, MUL_WARP_CTA, smem, st>>>(p->d_descs, list, n, ctr, in, out); break;
            case 2: batch_mulwarp_kernel<8><<<grid, MUL_WARP_CTA, smem, st>>>(p->d_descs, list, n, ctr, in, out); break;
            case 3: batch_mulwarp_kernel<16><<<grid, MUL_WARP_CTA, smem, st>>>(p->d_descs, list, n, ctr, in, out); break;
            default: batch_mulwarp_kernel<32><<<grid, MUL_WARP_CTA, smem, st>>>(p->d_descs, list, n, ctr, in, out);
            }
            BI_RETURN_IF(check_launch("batch warp mul kernel"));
        }
    }
    if (comps & COMP_DIV) {
        // the largest class first: its divisions take longest
        for (int c = DIV_CLASSES - 1; c >= 0; c--) {
            const uint32_t n = p->n_divc[c];
            if (!n) continue;
            const uint32_t* list = p->d_div + p->div_off[c];
            uint32_t* ctr = p->d_counters + 2 + c;
            const unsigned grid = L.grid[2 + c];
            cudaStream_t st = s[2 + c];
            switch (c) {
            case 0: batch_divthread_kernel<4><<<grid, DIV_THREAD_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 1: batch_divthread_kernel<8><<<grid, DIV_THREAD_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 2: batch_divthread_kernel<16><<<grid, DIV_THREAD_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 3: batch_divgroup_kernel<4, 8><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 4: batch_divgroup_kernel<8, 8><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 5: batch_divgroup_kernel<8, 16><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 6: batch_divwarp_kernel<8><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 7: batch_divgroup_kernel<24, 16><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 8: batch_divwarp_kernel<16><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 9: batch_divwarp3_kernel<24><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case 10: batch_divwarp_kernel<32><<<grid, DIV_WARP_CTA, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case DIV_BLK2_CLASS: batch_divblk_kernel<2><<<grid, 64, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            case DIV_BLK4_CLASS: batch_divblk_kernel<4><<<grid, 128, 0, st>>>(p->d_descs, list, n, ctr, in, out, flags); break;
            default:
                batch_div_kernel<DIV_CTA_THREADS><<<grid, DIV_CTA_THREADS, L.smem[2 + c], st>>>(p->d_descs, list, n, ctr,
                                                                                             in, out, flags);
            }
            BI_RETURN_IF(check_launch("batch div kernel"));
        }
    }
    return BI_OK;
}

// Capture counter reset, fork, the persistent kernels and the join into one
// executable graph.
static bi_status capture_plan(bi_plan* p, const uint64_t* in, uint64_t* out, uint8_t* flags) {
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    Launch3 L;
    BI_RETURN_IF(prepare_launch(p, p->tune, &L));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "plan capture: %s", cudaGetErrorString(e));
    cudaMemsetAsync(p->d_counters, 0, PLAN_KERNELS * sizeof(uint32_t), p->cap);
    cudaEventRecord(p->ev_fork, p->cap);
    for (int k = 0; k < PLAN_KERNELS; k++) cudaStreamWaitEvent(p->side[k], p->ev_fork, 0);
    bi_status st = launch_plan_kernels(p, in, out, flags, p->tune, L, p->side);
    for (int k = 0; k < PLAN_KERNELS; k++) {
        cudaEventRecord(p->ev_join[k], p->side[k]);
        cudaStreamWaitEvent(p->cap, p->ev_join[k], 0);
    }
    e = cudaStreamEndCapture(p->cap, &graph);
    if (st != BI_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return set_error(BI_ECUDA, "plan capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&p->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        p->exec = nullptr;
        return set_error(BI_ECUDA, "plan instantiate: %s", cudaGetErrorString(e));
    }
    p->g_in = in;
    p->g_out = out;
    p->g_flags = flags;
    p->g_tune = p->tune;
    return BI_OK;
}

static void plan_free(bi_plan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    cudaFree(p->d_descs);
    cudaFree(p->d_addsub);
    cudaFree(p->d_mul);
    cudaFree(p->d_div);
    cudaFree(p->d_items);
    cudaFree(p->d_items_large);
    cudaFree(p->d_mulw);
    cudaFree(p->d_counters);
    for (int k = 0; k < PLAN_KERNELS; k++) {
        if (p->side[k]) cudaStreamDestroy(p->side[k]);
        if (p->ev_join[k]) cudaEventDestroy(p->ev_join[k]);
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->cap) cudaStreamDestroy(p->cap);
    delete p;
}

// Descriptor i against the arenas: its op and sizes, and every operand,
// result and flag it names inside the input arena (in_limbs limbs), the
// output arena (out_limbs limbs) and the flag arena (nflags bytes; with
// nflags = 0 the batch writes no flags, so flag offsets are not read).
static bi_status check_desc(const bi_desc& d, uint64_t i, uint64_t in_limbs, uint64_t out_limbs, uint64_t nflags) {
    const unsigned long long k = (unsigned long long)i;
    if (d.m == 0) return set_error(BI_EINVAL, "descriptor %llu: m=0", k);
    if (d.width != 0 && d.width != 32 && d.width != 64)
        return set_error(BI_EINVAL, "descriptor %llu: width %u (0, 32 or 64)", k, d.width);
    const bool w32 = desc_w32(d);
    if (d.op == BI_OP_DIV ? (m64(d) > BATCH_DIV_MAX_M || mb64(d) > BATCH_DIV_MAX_MB) : m64(d) > BATCH_MAX_LIMBS)
        return set_error(BI_EUNSUPPORTED, "descriptor %llu: m=%u mb=%u above the batch's limits", k, d.m, d.mb);
    // the arenas in the descriptor's elements
    if (w32) {
        in_limbs *= 2;
        out_limbs *= 2;
    }
    auto inside = [](uint64_t off, uint64_t len, uint64_t size) { return off <= size && len <= size - off; };
    uint64_t la = d.m, lb = d.m, lr = d.m, lr2 = 0;
    bool flag = false;
    switch (d.op) {
    case BI_OP_ADD: break;
    case BI_OP_SUB: flag = true; break;
    case BI_OP_MUL: break;
    case BI_OP_MULFULL: {
        const uint32_t Lp = (m64(d) + 2 * MUL_C - 1) / (2 * MUL_C) * (2 * MUL_C);
        if (Lp > 2048) return set_error(BI_EUNSUPPORTED, "descriptor %llu: mulfull m=%u", k, d.m);
        lr = 2ull * d.m;
        break;
    }
    case BI_OP_DIV:
        if (d.mb == 0 || d.mb > d.m) return set_error(BI_EINVAL, "descriptor %llu: need 1 <= mb <= m", k);
        lb = d.mb;
        lr2 = d.mb;
        flag = true;
        break;
    default:
        return set_error(BI_EINVAL, "descriptor %llu: unknown op %u", k, d.op);
    }
    if (!inside(d.a, la, in_limbs) || !inside(d.b, lb, in_limbs))
        return set_error(BI_EINVAL, "descriptor %llu: operand outside the input arena of %llu limbs", k,
                         (unsigned long long)in_limbs);
    if (!inside(d.r, lr, out_limbs) || (lr2 && !inside(d.r2, lr2, out_limbs)))
        return set_error(BI_EINVAL, "descriptor %llu: result outside the output arena of %llu limbs", k,
                         (unsigned long long)out_limbs);
    if (flag && nflags && d.flag >= nflags)
        return set_error(BI_EINVAL, "descriptor %llu: flag byte %llu outside the flag arena of %llu bytes", k,
                         (unsigned long long)d.flag, (unsigned long long)nflags);
    return BI_OK;
}

}  // namespace bi

extern "C" {

bi_status bi_plan_create(bi_plan** out_plan, const bi_desc* descs, uint64_t count, uint64_t in_limbs,
                         uint64_t out_limbs, uint64_t nflags) {
    if (!out_plan) return set_error(BI_EINVAL, "out_plan is NULL");
    *out_plan = nullptr;
    if (count && !descs) return set_error(BI_EINVAL, "descs is NULL");
    if (count > 0xffffffffull) return set_error(BI_EINVAL, "too many descriptors");
    for (uint64_t i = 0; i < count; i++) BI_RETURN_IF(check_desc(descs[i], i, in_limbs, out_limbs, nflags));
    bi_plan* p = new bi_plan();
    cudaGetDevice(&p->device);
    p->count = count;
    p->nflags = nflags;
    std::vector<uint32_t> addsub, div, mulw[MULW_CLASSES];
    std::vector<std::pair<uint64_t, uint32_t>> mulkeys;   // (bucket key, index)
    for (uint64_t i = 0; i < count; i++) {
        const bi_desc& d = descs[i];
        switch (d.op) {
        case BI_OP_ADD:
        case BI_OP_SUB:
            addsub.push_back((uint32_t)i);
            break;
        case BI_OP_MUL:
        case BI_OP_MULFULL: {
            const uint32_t Lp = (m64(d) + 2 * MUL_C - 1) / (2 * MUL_C) * (2 * MUL_C);
            const uint32_t full = d.op == BI_OP_MULFULL;
            if (full) p->max_mul_Lp_full = std::max(p->max_mul_Lp_full, Lp);
            else p->max_mul_Lp_trunc = std::max(p->max_mul_Lp_trunc, Lp);
            mulkeys.push_back({((uint64_t)full << 40) | ((uint64_t)Lp << 8), (uint32_t)i});
            if (full && m64(d) <= MULW_MAX_M) mulw[mulw_class(m64(d))].push_back((uint32_t)i);
            break;
        }
        default:   // BI_OP_DIV (check_desc refused every other op)
            div.push_back((uint32_t)i);
            break;
        }
    }
    // largest first: long instances start early, short ones fill the tail
    std::stable_sort(addsub.begin(), addsub.end(), [&](uint32_t x, uint32_t y) { return m64(descs[x]) > m64(descs[y]); });
    int dmap[DIV_CLASSES];
    div_class_map(descs, div.data(), (uint32_t)div.size(), num_sms(), dmap);
    std::stable_sort(div.begin(), div.end(), [&](uint32_t x, uint32_t y) { return div_before(descs[x], descs[y], dmap); });
    std::stable_sort(mulkeys.begin(), mulkeys.end(), [](const std::pair<uint64_t, uint32_t>& x,
                                                        const std::pair<uint64_t, uint32_t>& y) {
        return x.first > y.first;
    });
    std::vector<uint32_t> mul;
    std::vector<MulItem> items, items_large;   // all multiplies; those the warp classes do not take
    for (size_t k = 0; k < mulkeys.size();) {
        const uint64_t key = mulkeys[k].first;
        const uint32_t full = (uint32_t)(key >> 40), Lp = (uint32_t)((key >> 8) & 0xffffffffu);
        const MulGeom g = mul_geometry(Lp, full != 0, 256);
        size_t end = k;
        while (end < mulkeys.size() && mulkeys[end].first == key) end++;
        for (size_t s = k; s < end; s += g.ipc) {
            MulItem it;
            it.first = (uint32_t)mul.size();
            it.count = (uint32_t)std::min<size_t>(g.ipc, end - s);
            it.Lp = Lp;
            it.full = full;
            for (size_t j = s; j < s + it.count; j++) mul.push_back(mulkeys[j].second);
            items.push_back(it);
            if (!(full && Lp <= MULW_MAX_M)) items_large.push_back(it);   // Lp <= 32 iff m <= 32
        }
        k = end;
    }
    // the warp classes' lists, largest first within a class, one after another
    std::vector<uint32_t> mulw_all;
    for (int c = 0; c < MULW_CLASSES; c++) {
        std::stable_sort(mulw[c].begin(), mulw[c].end(), [&](uint32_t x, uint32_t y) { return m64(descs[x]) > m64(descs[y]); });
        p->mulw_off[c] = (uint32_t)mulw_all.size();
        p->n_mulw[c] = (uint32_t)mulw[c].size();
        mulw_all.insert(mulw_all.end(), mulw[c].begin(), mulw[c].end());
    }
    p->n_mulw_total = (uint32_t)mulw_all.size();
    p->n_items_large = (uint32_t)items_large.size();
    p->n_addsub = (uint32_t)addsub.size();
    p->n_mul = (uint32_t)mul.size();
    p->n_items = (uint32_t)items.size();
    p->n_div = (uint32_t)div.size();
    div_classes(p, descs, div.data(), p->n_div, dmap);
    if (p->div_smem > 227 * 1024 || mul_smem_for(p, 1) > 227 * 1024) {
        plan_free(p);
        return set_error(BI_EUNSUPPORTED, "batch sizes need too much shared memory");
    }
    cudaError_t e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    for (int k = 0; k < PLAN_KERNELS && e == cudaSuccess; k++) e = cudaStreamCreateWithFlags(&p->side[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
    for (int k = 0; k < PLAN_KERNELS && e == cudaSuccess; k++) e = cudaEventCreateWithFlags(&p->ev_join[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        plan_free(p);
        return set_error(BI_ECUDA, "plan streams: %s", cudaGetErrorString(e));
    }
    std::vector<bi_desc> hd(descs, descs + count);
    bi_status st = dev_upload(&p->d_descs, hd, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_addsub, addsub, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_mul, mul, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_div, div, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_items, items, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_items_large, items_large, p->cap);
    if (st == BI_OK) st = dev_upload(&p->d_mulw, mulw_all, p->cap);
    if (st == BI_OK) {
        std::vector<uint32_t> zeros(PLAN_KERNELS, 0);
        st = dev_upload(&p->d_counters, zeros, p->cap);
    }
    if (st == BI_OK && cudaStreamSynchronize(p->cap) != cudaSuccess) st = set_error(BI_ECUDA, "plan upload failed");
    if (st != BI_OK) {
        plan_free(p);
        return st;
    }
    *out_plan = p;
    return BI_OK;
}

bi_status bi_plan_set_tuning(bi_plan* p, int addsub_rows, int addsub_vec, int mul_ipc_div) {
    if (!p) return set_error(BI_EINVAL, "NULL plan");
    if (!(addsub_rows == 2 || addsub_rows == 4 || addsub_rows == 8) || !(addsub_vec == 1 || addsub_vec == 2) ||
        mul_ipc_div < 1 || mul_ipc_div > 8)
        return set_error(BI_EINVAL, "tuning out of range");
    if (addsub_vec == 1) addsub_rows = 4;
    std::lock_guard<std::mutex> lk(p->mu);
    p->tune.addsub_rows = addsub_rows;
    p->tune.addsub_vec = addsub_vec;
    p->tune.mul_ipc_div = mul_ipc_div;
    return BI_OK;
}

bi_status bi_plan_set_mul_word_bits(bi_plan* p, int bits) {
    if (!p) return set_error(BI_EINVAL, "NULL plan");
    if (bits != 32 && bits != 64) return set_error(BI_EINVAL, "word bits must be 32 or 64");
    std::lock_guard<std::mutex> lk(p->mu);
    p->tune.mul_small_bits = bits;
    return BI_OK;
}

bi_status bi_plan_get_tuning(bi_plan* p, int* tuning) {
    if (!p || !tuning) return set_error(BI_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(p->mu);
    tuning[0] = p->tune.addsub_rows;
    tuning[1] = p->tune.addsub_vec;
    tuning[2] = p->tune.mul_ipc_div;
    tuning[3] = p->tune.mul_small_bits;
    return BI_OK;
}

bi_status bi_plan_execute(bi_plan* p, const uint64_t* in, uint64_t* out, uint8_t* flags, bi_stream stream) {
    if (!p) return set_error(BI_EINVAL, "NULL plan");
    if (p->count == 0) return BI_OK;
    if (!in || !out) return set_error(BI_EINVAL, "NULL arena");
    if (flags && p->nflags == 0) return set_error(BI_EINVAL, "flags given to a plan created with nflags = 0");
    if ((uintptr_t)in % 16 || (uintptr_t)out % 16) return set_error(BI_EINVAL, "arenas must be 16-byte aligned");
    std::lock_guard<std::mutex> lk(p->mu);
    if (!p->exec || p->g_in != in || p->g_out != out || p->g_flags != flags ||
        memcmp(&p->g_tune, &p->tune, sizeof(BatchTune)) != 0) {
        BI_RETURN_IF(capture_plan(p, in, out, flags));
    }
    cudaError_t e = cudaGraphLaunch(p->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "plan launch: %s", cudaGetErrorString(e));
    return BI_OK;
}

// Time the plan's components `comp` with tuning t (ms per run, median of
// reps), their kernels forked onto the plan's streams as the captured graph
// runs them, so that kernels that share the GPU are timed sharing it.
static float time_component(bi_plan* p, const uint64_t* in, uint64_t* out, uint8_t* flags, const BatchTune& t,
                            int comp, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ts;
    Launch3 L;
    if (prepare_launch(p, t, &L) != BI_OK) return 1e30f;
    for (int r = 0; r < reps + 1; r++) {
        cudaMemsetAsync(p->d_counters, 0, PLAN_KERNELS * sizeof(uint32_t), p->cap);
        cudaEventRecord(e0, p->cap);
        cudaEventRecord(p->ev_fork, p->cap);
        for (int k = 0; k < PLAN_KERNELS; k++) cudaStreamWaitEvent(p->side[k], p->ev_fork, 0);
        bi_status st = launch_plan_kernels(p, in, out, flags, t, L, p->side, comp);
        for (int k = 0; k < PLAN_KERNELS; k++) {
            cudaEventRecord(p->ev_join[k], p->side[k]);
            cudaStreamWaitEvent(p->cap, p->ev_join[k], 0);
        }
        cudaEventRecord(e1, p->cap);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (st != BI_OK) ms = 1e30f;
        if (r > 0) ts.push_back(ms);   // the first run warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::sort(ts.begin(), ts.end());
    return ts[ts.size() / 2];
}

// Pick, on this plan's own data, the add/sub rows per step (limbs per lane)
// and limb width per lane, the multiply instances per CTA, and the word
// width of the small full products' arithmetic (32-bit words on the warp
// kernel or 64-bit limbs on the CTA kernel), one after another, each
// candidate timed as a run of the whole plan (its kernels sharing the GPU as
// in an execute); results land in `out` exactly as an execute would write
// them.
bi_status bi_plan_autotune(bi_plan* p, const uint64_t* in, uint64_t* out, uint8_t* flags, int reps,
                           int* chosen) {
    if (!p) return set_error(BI_EINVAL, "NULL plan");
    if (p->count == 0) return BI_OK;
    if (!in || !out) return set_error(BI_EINVAL, "NULL arena");
    if (flags && p->nflags == 0) return set_error(BI_EINVAL, "flags given to a plan created with nflags = 0");
    if (reps < 1) reps = 1;
    std::lock_guard<std::mutex> lk(p->mu);
    BatchTune best = p->tune;
    if (p->n_addsub) {
        const int cand[4][2] = {{2, 2}, {4, 2}, {8, 2}, {4, 1}};
        float bt = 1e30f;
        for (auto& c : cand) {
            BatchTune t = best;
            t.addsub_rows = c[0];
            t.addsub_vec = c[1];
            const float ms = time_component(p, in, out, flags, t, COMP_ALL, reps);
            if (ms < bt) { bt = ms; best.addsub_rows = c[0]; best.addsub_vec = c[1]; }
        }
    }
    if (p->n_items) {
        float bt = 1e30f;
        for (int d = 1; d <= 4; d *= 2) {
            BatchTune t = best;
            t.mul_ipc_div = d;
            if (mul_smem_for(p, d) > 227 * 1024) continue;
            const float ms = time_component(p, in, out, flags, t, COMP_ALL, reps);
            if (ms < bt) { bt = ms; best.mul_ipc_div = d; }
        }
    }
    if (p->n_mulw_total) {   // the small full products' word width: the warp kernel's 32 or the CTA's 64
        float bt = 1e30f;
        for (int bits : {32, 64}) {
            BatchTune t = best;
            t.mul_small_bits = bits;
            const float ms = time_component(p, in, out, flags, t, COMP_ALL, reps);
            if (ms < bt) { bt = ms; best.mul_small_bits = bits; }
        }
    }
    cudaError_t e = cudaStreamSynchronize(p->cap);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "autotune: %s", cudaGetErrorString(e));
    p->tune = best;
    if (chosen) {
        chosen[0] = best.addsub_rows;
        chosen[1] = best.addsub_vec;
        chosen[2] = best.mul_ipc_div;
    }
    return BI_OK;
}

bi_status bi_plan_destroy(bi_plan* p) {
    if (!p) return BI_OK;
    cudaDeviceSynchronize();
    plan_free(p);
    return BI_OK;
}

bi_status bi_plan_stats(const bi_plan* p, uint64_t* stats) {
    if (!p || !stats) return set_error(BI_EINVAL, "NULL argument");
    stats[0] = p->n_addsub;
    stats[1] = p->n_mul;
    stats[2] = p->n_items;
    stats[3] = p->n_div;
    stats[4] = p->mul_smem ? p->mul_smem : mul_smem_for(p, p->tune.mul_ipc_div);
    stats[5] = p->div_smem;
    return BI_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Uneven batch without any device allocation.
//
// bi_plan_create allocates device work lists and counters.  Some callers
// cannot allocate device memory at the point where they need a batch run --
// code running under an allocator that forbids cudaMalloc, or inside a
// framework callback that must not allocate -- so this entry point keeps the
// same scratch (a copy of the descriptors, the three work lists, the
// multiply items and the work counters) in a fixed array in device memory
// that the library owns, and launches the same three persistent kernels on
// the caller's stream.  The array is a file-scope __device__ variable: every
// GPU that loads the library holds NOALLOC_SCRATCH_BYTES of it until the
// process exits, and all calls share it.
// ---------------------------------------------------------------------------
namespace bi {

constexpr uint32_t NOALLOC_MAX_DESCS = 4096;
constexpr size_t NA_DESC_OFF = 0;
constexpr size_t NA_ADD_OFF = NA_DESC_OFF + (size_t)NOALLOC_MAX_DESCS * sizeof(bi_desc);
constexpr size_t NA_MUL_OFF = NA_ADD_OFF + (size_t)NOALLOC_MAX_DESCS * sizeof(uint32_t);
constexpr size_t NA_DIV_OFF = NA_MUL_OFF + (size_t)NOALLOC_MAX_DESCS * sizeof(uint32_t);
constexpr size_t NA_ITEM_OFF = NA_DIV_OFF + (size_t)NOALLOC_MAX_DESCS * sizeof(uint32_t);
constexpr size_t NA_CNT_OFF = NA_ITEM_OFF + (size_t)NOALLOC_MAX_DESCS * sizeof(MulItem);
constexpr size_t NOALLOC_SCRATCH_BYTES = NA_CNT_OFF + 256;
static_assert(PLAN_KERNELS * sizeof(uint32_t) <= 256, "plan counters outgrow their scratch slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Host-side staging of the work lists, reused by every call (no heap use).
static bi_desc na_descs[NOALLOC_MAX_DESCS];
static uint32_t na_add[NOALLOC_MAX_DESCS], na_mul[NOALLOC_MAX_DESCS], na_div[NOALLOC_MAX_DESCS];
static std::pair<uint64_t, uint32_t> na_keys[NOALLOC_MAX_DESCS];
static MulItem na_items[NOALLOC_MAX_DESCS];
static std::mutex na_mu;                 // guards the staging arrays

// Device address of the scratch array on the current device: the host-side
// name of a __device__ variable is not a device address.  Looked up on every
// call (cheap next to the call's stream synchronisation), so a context that
// was torn down and created again (cudaDeviceReset) gets its own address.
static bi_status noalloc_scratch(void** ptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return set_error(BI_ECUDA, "scratch address lookup: %s", cudaGetErrorString(e));
    }
    *ptr = p;
    return BI_OK;
}

}  // namespace bi

extern "C" uint32_t bi_batch_noalloc_max_descs(void) { return NOALLOC_MAX_DESCS; }

extern "C" bi_status bi_batch_run_noalloc(const bi_desc* descs, uint64_t count, const uint64_t* in,
                                          uint64_t in_limbs, uint64_t* out, uint64_t out_limbs, uint8_t* flags,
                                          uint64_t nflags, bi_stream stream) {
    if (count == 0) return BI_OK;
    if (!descs) return set_error(BI_EINVAL, "descs is NULL");
    if (count > NOALLOC_MAX_DESCS)
        return set_error(BI_EINVAL, "bi_batch_run_noalloc takes at most %u descriptors, got %llu (use bi_plan_*)",
                         NOALLOC_MAX_DESCS, (unsigned long long)count);
    if (!in || !out) return set_error(BI_EINVAL, "NULL arena");
    if ((uintptr_t)in % 16 || (uintptr_t)out % 16) return set_error(BI_EINVAL, "arenas must be 16-byte aligned");
    if (flags && nflags == 0) return set_error(BI_EINVAL, "flags given with nflags = 0");
    for (uint64_t i = 0; i < count; i++) BI_RETURN_IF(check_desc(descs[i], i, in_limbs, out_limbs, nflags));
    // the call stages its lists from host memory and waits for its stream,
    // which a stream in capture cannot do: refuse it before anything is enqueued
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return set_error(BI_ECUDA, "bi_batch_run_noalloc: %s", cudaGetErrorString(ce));
    }
    if (cs != cudaStreamCaptureStatusNone)
        return set_error(BI_EUNSUPPORTED, "bi_batch_run_noalloc: the stream is being captured");
    std::lock_guard<std::mutex> lk(na_mu);
    void* scratch = nullptr;
    BI_RETURN_IF(noalloc_scratch(&scratch));
    unsigned char* base = (unsigned char*)scratch;

    // the work lists, exactly as bi_plan_create builds them
    bi_plan p;                            // on the stack; owns nothing
    uint32_t na = 0, nm = 0, nd = 0, nk = 0, ni = 0;
    for (uint64_t i = 0; i < count; i++) {
        const bi_desc& d = descs[i];
        na_descs[i] = d;
        if (d.op == BI_OP_ADD || d.op == BI_OP_SUB) {
            na_add[na++] = (uint32_t)i;
        } else if (d.op == BI_OP_MUL || d.op == BI_OP_MULFULL) {
            const uint32_t Lp = (m64(d) + 2 * MUL_C - 1) / (2 * MUL_C) * (2 * MUL_C);
            const uint32_t full = d.op == BI_OP_MULFULL;
            if (full) p.max_mul_Lp_full = std::max(p.max_mul_Lp_full, Lp);
            else p.max_mul_Lp_trunc = std::max(p.max_mul_Lp_trunc, Lp);
            na_keys[nk++] = {((uint64_t)full << 40) | ((uint64_t)Lp << 8), (uint32_t)i};
        } else {   // BI_OP_DIV (check_desc refused every other op)
            na_div[nd++] = (uint32_t)i;
        }
    }
    std::stable_sort(na_add, na_add + na, [&](uint32_t x, uint32_t y) { return m64(descs[x]) > m64(descs[y]); });
    int dmap[DIV_CLASSES];
    div_class_map(descs, na_div, nd, num_sms(), dmap);
    std::stable_sort(na_div, na_div + nd, [&](uint32_t x, uint32_t y) { return div_before(descs[x], descs[y], dmap); });
    std::stable_sort(na_keys, na_keys + nk, [](const std::pair<uint64_t, uint32_t>& x,
                                               const std::pair<uint64_t, uint32_t>& y) { return x.first > y.first; });
    for (uint32_t k = 0; k < nk;) {
        const uint64_t key = na_keys[k].first;
        const uint32_t full = (uint32_t)(key >> 40), Lp = (uint32_t)((key >> 8) & 0xffffffffu);
        const MulGeom g = mul_geometry(Lp, full != 0, 256);
        uint32_t end = k;
        while (end < nk && na_keys[end].first == key) end++;
        for (uint32_t s = k; s < end; s += g.ipc) {
            MulItem it;
            it.first = nm;
            it.count = std::min<uint32_t>(g.ipc, end - s);
            it.Lp = Lp;
            it.full = full;
            for (uint32_t j = s; j < s + it.count; j++) na_mul[nm++] = na_keys[j].second;
            na_items[ni++] = it;
        }
        k = end;
    }
    p.count = count;
    p.nflags = nflags;
    p.n_addsub = na;
    p.n_mul = nm;
    p.n_items = ni;
    p.n_div = nd;
    div_classes(&p, descs, na_div, nd, dmap);
    if (p.div_smem > 227 * 1024 || mul_smem_for(&p, 1) > 227 * 1024)
        return set_error(BI_EUNSUPPORTED, "batch sizes need too much shared memory");
    p.d_descs = (bi_desc*)(base + NA_DESC_OFF);
    p.d_addsub = (uint32_t*)(base + NA_ADD_OFF);
    p.d_mul = (uint32_t*)(base + NA_MUL_OFF);
    p.d_div = (uint32_t*)(base + NA_DIV_OFF);
    p.d_items = (MulItem*)(base + NA_ITEM_OFF);
    p.d_counters = (uint32_t*)(base + NA_CNT_OFF);

    // stage the lists (the array keeps the previous call's contents: every
    // region read below is rewritten, and the counters are cleared)
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(p.d_descs, na_descs, count * sizeof(bi_desc), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && na) e = cudaMemcpyAsync(p.d_addsub, na_add, na * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nm) e = cudaMemcpyAsync(p.d_mul, na_mul, nm * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nd) e = cudaMemcpyAsync(p.d_div, na_div, nd * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && ni) e = cudaMemcpyAsync(p.d_items, na_items, ni * sizeof(MulItem), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.d_counters, 0, PLAN_KERNELS * sizeof(uint32_t), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(BI_ECUDA, "staging the batch: %s", cudaGetErrorString(e));
    }
    Launch3 L;
    BI_RETURN_IF(prepare_launch(&p, p.tune, &L));
    cudaStream_t ss[PLAN_KERNELS];
    for (int k = 0; k < PLAN_KERNELS; k++) ss[k] = s;
    BI_RETURN_IF(launch_plan_kernels(&p, in, out, flags, p.tune, L, ss));
    // the host staging arrays may be reused once the copies have read them
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "batch run: %s", cudaGetErrorString(e));
    return BI_OK;
}
