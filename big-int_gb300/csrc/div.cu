// div.cu -- batched division (quotient and remainder) by a shifted inverse.
//
// The reference defines division only as a sequential C prototype
// (prototypes/div.c:427-467, div_shinv) and an unvalidated Futhark version
// (futhark/div.fut:150-167): q = floor(u * shinv_h(v) / B^h) + delta with the
// shifted inverse shinv_h(v) ~ B^h / v refined by Newton steps that use
// shorter iterates and prefixes of the divisor (refine3, div.c:333-349), then
// the remainder r = u - v*q and a final correction (div.c:457-463).  This
// kernel computes the same quantities on the GPU, one instance per CTA, all
// operands in shared memory, on 64-bit limbs:
//
//   1. normalise: shift u and v left by s bits so v's top limb has its top
//      bit set (K = limbs of v, H = limbs of the shifted u);
//   2. shifted inverse Y ~ B^(K+P) / v with P = H-K+2 limbs of precision:
//      start from floor((B^2-1)/v_top) (one correct limb) and apply Newton
//      steps y' = y + y(1 - x y) at growing precision p -> p' <= 2p-2, each
//      using only the top p'+1 limbs of v (divisor prefix) and a p+1-limb
//      iterate (shorter iterate); the error term 1 - x y is recovered from
//      the low p'+2 limbs of the product, as div.c's powerdiff recovers
//      B^h - v*w from a truncated product (div.c:246-280);
//   3. q = floor(u * Y / B^(K+P)); r = u - q*v from the low K+1 limbs of q*v;
//      while r < 0: q--, r += v; while r >= v: q++, r -= v (the reference's
//      delta step, div.c:459-463, made two-sided and bounded);
//   4. r is shifted back right by s bits.
// The estimate is exact or one short in every case tested; a bound of
// DIV_MAX_CORRECTIONS steps on each side turns anything else into status 2.
//
// Small and medium divisors take another route to the same unique (q, r):
// schoolbook long division (divsmall.cuh) on one thread per instance up to
// DIV_THREAD_MAX_MV 64-bit limbs and on one warp per instance up to
// DIV_WARP_MAX_MV, where its K (MU - K + 1) limb products and no barriers
// cost less than a CTA running the steps above (div_use_long holds the
// measured crossover, which depends on the batch size too).
#include "divblock.cuh"
#include "divcore.cuh"
#include "divsmall.cuh"

namespace bi {

template <typename T>
__device__ __forceinline__ uint64_t limb64(const T* p, uint32_t count_T, uint32_t i) {
    if constexpr (sizeof(T) == 8) {
        return i < count_T ? p[i] : 0;
    } else {
        uint64_t x = 2 * i < count_T ? p[2 * i] : 0u;
        if (2 * i + 1 < count_T) x |= (uint64_t)p[2 * i + 1] << 32;
        return x;
    }
}

template <typename T>
__device__ __forceinline__ void put_limb64(T* p, uint32_t count_T, uint32_t i, uint64_t x) {
    if constexpr (sizeof(T) == 8) {
        if (i < count_T) p[i] = x;
    } else {
        if (2 * i < count_T) p[2 * i] = (uint32_t)x;
        if (2 * i + 1 < count_T) p[2 * i + 1] = (uint32_t)(x >> 32);
    }
}

template <typename T>
__global__ void __launch_bounds__(512)
div_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
           uint8_t* __restrict__ status, uint64_t n, DivGeom g) {
    extern __shared__ __align__(16) uint64_t smem[];
    for (uint64_t inst = blockIdx.x; inst < n; inst += gridDim.x) {
        const T* ui = u + inst * g.mu;
        const T* vi = v + inst * g.mv;
        T* qi = q + inst * g.mu;
        T* ri = r + inst * g.mv;
        div_cta(
            g, smem, [&](uint32_t i) { return limb64(ui, g.mu, i); }, [&](uint32_t i) { return limb64(vi, g.mv, i); },
            [&](uint32_t i, uint64_t x) { put_limb64(qi, g.mu, i, x); },
            [&](uint32_t i, uint64_t x) { put_limb64(ri, g.mv, i, x); },
            [&](uint8_t code) { if (status) status[inst] = code; });
    }
}

// ---------------------------------------------------------------------------

// One thread per instance: long division for divisors of at most MX limbs
// (divsmall.cuh).
template <typename T, int MX>
__global__ void __launch_bounds__(DIV_THREAD_CTA)
div_thread_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
                  uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    const uint32_t MU = sizeof(T) == 8 ? mu : (mu + 1) / 2, MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    for (uint64_t inst = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; inst < n;
         inst += (uint64_t)gridDim.x * blockDim.x) {
        const T* ui = u + inst * mu;
        const T* vi = v + inst * mv;
        T* qi = q + inst * mu;
        T* ri = r + inst * mv;
        const uint8_t st = div_thread<MX>(
            MU, MV, [&](uint32_t i) { return limb64(ui, mu, i); }, [&](uint32_t i) { return limb64(vi, mv, i); },
            [&](uint32_t i, uint64_t x) { put_limb64(qi, mu, i, x); },
            [&](uint32_t i, uint64_t x) { put_limb64(ri, mv, i, x); });
        if (status) status[inst] = st;
    }
}

// Several instances a warp: long division on G-lane groups (divsmall.cuh).
template <typename T, int VPL, int G>
__global__ void __launch_bounds__(DIV_WARP_CTA)
div_group_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
                 uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv);

template <typename T>
static void launch_div_thread(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv,
                              uint64_t n, cudaStream_t s) {
    const uint32_t MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    if (div_small_on_groups(MV, n, num_sms())) {   // few instances: four 8-lane groups a warp
        const uint64_t warps = (n + 3) / 4, blocks = (warps + DIV_WARP_CTA / 32 - 1) / (DIV_WARP_CTA / 32);
        div_group_kernel<T, 2, 8><<<(unsigned)blocks, DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
        return;
    }
    const uint64_t blocks = (n + DIV_THREAD_CTA - 1) / DIV_THREAD_CTA;
    const unsigned grid = (unsigned)(blocks < (1u << 20) ? blocks : (1u << 20));
    // register windows of 2, 3, 4, 6, 8, 12 or 16 limbs: a divisor is
    // right-aligned in its window, whose rows below it are zeros, so the widths
    // between the powers of two ran 6-20 % faster at 3, 5, 6, 10, 12 limbs
    if (MV <= 2) div_thread_kernel<T, 2><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 3) div_thread_kernel<T, 3><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 4) div_thread_kernel<T, 4><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 6) div_thread_kernel<T, 6><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 8) div_thread_kernel<T, 8><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 12) div_thread_kernel<T, 12><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else div_thread_kernel<T, 16><<<grid, DIV_THREAD_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
}

// One warp per instance: long division for divisors of at most 32 VPL limbs
// (divsmall.cuh).
template <typename T, int VPL>
__device__ __forceinline__ void div_warp_instances(const T* __restrict__ u, const T* __restrict__ v,
                                                   T* __restrict__ q, T* __restrict__ r,
                                                   uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    const uint32_t MU = sizeof(T) == 8 ? mu : (mu + 1) / 2, MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    const uint64_t warps = (uint64_t)gridDim.x * (DIV_WARP_CTA / 32);
    for (uint64_t inst = (uint64_t)blockIdx.x * (DIV_WARP_CTA / 32) + threadIdx.x / 32; inst < n; inst += warps) {
        const T* ui = u + inst * mu;
        const T* vi = v + inst * mv;
        T* qi = q + inst * mu;
        T* ri = r + inst * mv;
        const uint8_t st = div_warp<VPL>(
            MU, MV, [&](uint32_t i) { return limb64(ui, mu, i); }, [&](uint32_t i) { return limb64(vi, mv, i); },
            [&](uint32_t i, uint64_t x) { put_limb64(qi, mu, i, x); },
            [&](uint32_t i, uint64_t x) { put_limb64(ri, mv, i, x); });
        if (status && (threadIdx.x & 31) == 0) status[inst] = st;
    }
}

template <typename T, int VPL>
__global__ void __launch_bounds__(DIV_WARP_CTA)
div_warp_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
                uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    div_warp_instances<T, VPL>(u, v, q, r, status, n, mu, mv);
}

// The same, held to three CTAs (12 warps) an SM: for 24 limbs a lane, where
// ptxas otherwise takes 255 registers (8 warps an SM), 168 registers and a
// few spills ran 4-10 % faster (700- and 768-limb divisors); the 20- and
// 28-limb shapes stay on the default bound (their 3-CTA variants were slower
// or spilled 240 bytes).
template <typename T, int VPL>
__global__ void __launch_bounds__(DIV_WARP_CTA, 3)
div_warp3_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
                 uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    div_warp_instances<T, VPL>(u, v, q, r, status, n, mu, mv);
}

template <typename T, int VPL, int G>
__global__ void __launch_bounds__(DIV_WARP_CTA)
div_group_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
                 uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    constexpr uint32_t ipw = 32 / G;
    const uint32_t MU = sizeof(T) == 8 ? mu : (mu + 1) / 2, MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    const uint64_t warps = (uint64_t)gridDim.x * (DIV_WARP_CTA / 32);
    for (uint64_t w = (uint64_t)blockIdx.x * (DIV_WARP_CTA / 32) + threadIdx.x / 32; w * ipw < n; w += warps) {
        const uint64_t inst = w * ipw + (threadIdx.x & 31) / G;
        const bool valid = inst < n;
        const uint64_t k = valid ? inst : 0;   // an invalid group reads and writes nothing
        const T* ui = u + k * mu;
        const T* vi = v + k * mv;
        T* qi = q + k * mu;
        T* ri = r + k * mv;
        const uint8_t st = div_group<VPL, G>(
            valid, MU, MV, [&](uint32_t i) { return limb64(ui, mu, i); }, [&](uint32_t i) { return limb64(vi, mv, i); },
            [&](uint32_t i, uint64_t x) { put_limb64(qi, mu, i, x); },
            [&](uint32_t i, uint64_t x) { put_limb64(ri, mv, i, x); });
        if (status && valid && (threadIdx.x & (G - 1)) == 0) status[inst] = st;
    }
}

// Long division for divisors of 17..1024 64-bit limbs: the group shape per
// divisor size that ran fastest on GB300 (2m/m divisions, thousands of
// instances): 8-lane groups of 3, 4, 6 and 8 limbs a lane up to 24, 32, 48
// and 64 limbs, 16-lane groups of 6 and 8 up to 96 and 128, a whole warp of 6
// and 8 up to 192 and 256, 16-lane groups of 20, 24, 28 and 32 up to 320,
// 384, 448 and 512, a warp of 20, 24, 28 and 32 up to 640, 768, 896 and 1024
// (the shapes between the powers of two run 1.07-1.4x faster there: fewer
// rows of zeros below the right-aligned divisor, fewer registers); with few instances
// (div_small_on_warps) one warp each up to 128 limbs.
template <typename T>
static void launch_div_warp(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv,
                            uint64_t n, cudaStream_t s) {
    const uint32_t MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    constexpr uint32_t WPC = DIV_WARP_CTA / 32;   // warps per CTA
    auto grid_for = [&](uint32_t ipw) {
        const uint64_t warps = (n + ipw - 1) / ipw;
        const uint64_t blocks = (warps + WPC - 1) / WPC;
        return (unsigned)(blocks < (1u << 20) ? blocks : (1u << 20));
    };
    if (div_small_on_warps(MV, n, num_sms())) {   // few instances: one warp each
        if (MV <= 32) div_warp_kernel<T, 1><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
        else if (MV <= 64) div_warp_kernel<T, 2><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
        else div_warp_kernel<T, 4><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
        return;
    }
    if (MV <= 24) div_group_kernel<T, 3, 8><<<grid_for(4), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 32) div_group_kernel<T, 4, 8><<<grid_for(4), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 48) div_group_kernel<T, 6, 8><<<grid_for(4), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 64) div_group_kernel<T, 8, 8><<<grid_for(4), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 96) div_group_kernel<T, 6, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 128) div_group_kernel<T, 8, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 192) div_warp_kernel<T, 6><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 256) div_warp_kernel<T, 8><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    // 20, 24 and 28 limbs a lane between the powers of two: a divisor is
    // right-aligned in the lanes' 32 VPL (or G VPL) limbs, whose rows below it
    // are zeros
    else if (MV <= 320) div_group_kernel<T, 20, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 384) div_group_kernel<T, 24, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 448) div_group_kernel<T, 28, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 512) div_group_kernel<T, 32, 16><<<grid_for(2), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 640) div_warp_kernel<T, 20><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 768) div_warp3_kernel<T, 24><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else if (MV <= 896) div_warp_kernel<T, 28><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
    else div_warp_kernel<T, 32><<<grid_for(1), DIV_WARP_CTA, 0, s>>>(u, v, q, r, status, n, mu, mv);
}

// One instance on NW warps: long division KB quotient limbs at a time
// (divblock.cuh) for divisors of at most 32 NW VPL limbs.  NW = 1: four
// warps a CTA, one instance each; NW > 1: one instance a CTA of NW warps.
template <typename T, int VPL, int KB, int NW>
__global__ void __launch_bounds__(NW == 1 ? DIV_WARP_CTA : 32 * NW)
div_blk_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
               uint8_t* __restrict__ status, uint64_t n, uint32_t mu, uint32_t mv) {
    __shared__ DivBlkShared<KB, NW> sh;
    const uint32_t MU = sizeof(T) == 8 ? mu : (mu + 1) / 2, MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    const uint64_t per_cta = NW == 1 ? DIV_WARP_CTA / 32 : 1;
    const uint64_t stride = (uint64_t)gridDim.x * per_cta;
    for (uint64_t inst = (uint64_t)blockIdx.x * per_cta + (NW == 1 ? threadIdx.x / 32 : 0); inst < n;
         inst += stride) {
        const T* ui = u + inst * mu;
        const T* vi = v + inst * mv;
        T* qi = q + inst * mu;
        T* ri = r + inst * mv;
        const uint8_t st = div_blk<VPL, KB, NW>(
            MU, MV, [&](uint32_t i) { return limb64(ui, mu, i); }, [&](uint32_t i) { return limb64(vi, mv, i); },
            [&](uint32_t i, uint64_t x) { put_limb64(qi, mu, i, x); },
            [&](uint32_t i, uint64_t x) { put_limb64(ri, mv, i, x); }, &sh);
        if (status && threadIdx.x % (32 * NW) == 0) status[inst] = st;
    }
}

template <typename T, int VPL, int KB, int NW>
static void launch_blk(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                       cudaStream_t s) {
    const uint64_t per_cta = NW == 1 ? DIV_WARP_CTA / 32 : 1;
    const uint64_t blocks = (n + per_cta - 1) / per_cta;
    const unsigned grid = (unsigned)(blocks < (1u << 20) ? blocks : (1u << 20));
    div_blk_kernel<T, VPL, KB, NW><<<grid, NW == 1 ? DIV_WARP_CTA : 32 * NW, 0, s>>>(u, v, q, r, status, n, mu, mv);
}

// Long division of divisors of 1025..DIV_LONG_MAX_MV limbs, KB = 8 quotient
// limbs at a time (divblock.cuh) on two or four warps.
template <typename T>
static void launch_div_blk(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv,
                           uint64_t n, cudaStream_t s) {
    const uint32_t MV = sizeof(T) == 8 ? mv : (mv + 1) / 2;
    if (MV <= 2048) launch_blk<T, 32, 8, 2>(u, v, q, r, status, mu, mv, n, s);
    else launch_blk<T, 32, 8, 4>(u, v, q, r, status, mu, mv, n, s);
}

// dividend limbs (u64 view) per instance: any long division, and the shifted inverse's limit
constexpr uint32_t DIV_MAX_MU64 = 8192, DIV_SHINV_MAX_MU64 = 2048;
constexpr int DIV_AUTO = 0, DIV_SHINV = 1, DIV_LONG = 2;   // method of div_entry

template <typename T>
static bi_status div_entry(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv,
                           uint64_t n, bi_stream s, int method = DIV_AUTO) {
    if (n == 0) return BI_OK;
    if (mu == 0 || mv == 0) return set_error(BI_EINVAL, "mu and mv must be >= 1");
    if (mv > mu) return set_error(BI_EINVAL, "divisor limbs mv=%u exceed dividend limbs mu=%u", mv, mu);
    if (!u || !v || !q || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)u % sizeof(T) || (uintptr_t)v % sizeof(T) || (uintptr_t)q % sizeof(T) ||
        (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    const DivGeom g = div_geom(mu, mv, (int)sizeof(T));
    if (g.MU > DIV_MAX_MU64) return set_error(BI_EUNSUPPORTED, "div: dividend of %u limbs above the supported size", mu);
    if (method == DIV_LONG && g.MV > (uint32_t)DIV_LONG_MAX_MV)
        return set_error(BI_EUNSUPPORTED, "div_long: divisor of %u limbs above %d 64-bit limbs", mv, DIV_LONG_MAX_MV);
    if (method == DIV_SHINV && g.MU > DIV_SHINV_MAX_MU64)
        return set_error(BI_EUNSUPPORTED, "div_shinv: dividend of %u limbs above %u 64-bit limbs", mu,
                         DIV_SHINV_MAX_MU64);
    if (method != DIV_SHINV && g.MV <= (uint32_t)DIV_THREAD_MAX_MV) {
        launch_div_thread(u, v, q, r, status, mu, mv, n, (cudaStream_t)s);
        return check_launch("div thread kernel");
    }
    // the shifted inverse holds its operands in shared memory: dividends above
    // DIV_SHINV_MAX_MU64 limbs always take long division
    if (method != DIV_SHINV && g.MV <= (uint32_t)DIV_LONG_MAX_MV &&
        (method == DIV_LONG || g.MU > DIV_SHINV_MAX_MU64 || div_use_long(g.MV, n, num_sms()))) {
        if (g.MV <= (uint32_t)DIV_WARP_MAX_MV) {
            launch_div_warp(u, v, q, r, status, mu, mv, n, (cudaStream_t)s);
            return check_launch("div warp kernel");
        }
        launch_div_blk(u, v, q, r, status, mu, mv, n, (cudaStream_t)s);
        return check_launch("div block kernel");
    }
    const size_t smem = div_smem_bytes(g);
    if (smem > 227 * 1024) return set_error(BI_EUNSUPPORTED, "div: sizes need too much shared memory");
    const int threads = div_threads(g.MU);
    auto kern = div_kernel<T>;
    cudaError_t e = smem_opt_in((const void*)kern, smem);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "div: %s", cudaGetErrorString(e));
    const uint64_t grid = n < (1ull << 30) ? n : (1ull << 30);
    kern<<<(unsigned)grid, threads, smem, (cudaStream_t)s>>>(u, v, q, r, status, n, g);
    return check_launch("div kernel");
}

}  // namespace bi

using namespace bi;

extern "C" {

uint32_t bi_max_limbs_div_u64(void) { return DIV_MAX_MU64; }
uint32_t bi_max_limbs_div_u32(void) { return 2 * DIV_MAX_MU64; }

bi_status bi_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r, uint8_t* status,
                     uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint64_t>(u, v, q, r, status, mu, mv, n, s);
}
bi_status bi_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r, uint8_t* status,
                     uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint32_t>(u, v, q, r, status, mu, mv, n, s);
}

bi_status bi_div_shinv_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r, uint8_t* status,
                           uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint64_t>(u, v, q, r, status, mu, mv, n, s, DIV_SHINV);
}
bi_status bi_div_shinv_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r, uint8_t* status,
                           uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint32_t>(u, v, q, r, status, mu, mv, n, s, DIV_SHINV);
}
bi_status bi_div_long_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r, uint8_t* status,
                          uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint64_t>(u, v, q, r, status, mu, mv, n, s, DIV_LONG);
}
bi_status bi_div_long_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r, uint8_t* status,
                          uint32_t mu, uint32_t mv, uint64_t n, bi_stream s) {
    return div_entry<uint32_t>(u, v, q, r, status, mu, mv, n, s, DIV_LONG);
}

}  // extern "C"
