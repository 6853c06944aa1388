// prims.cu -- the division prototype's helper primitives as batched ops.
//
// The reference's shifted-inverse division is built from small helpers on
// whole big integers (prototypes/div.c:49-202; their parallel Futhark forms
// are futhark/helper.fut:83-124 and futhark/div.fut:21-69): compare (lt,
// eq), test for zero (ez), the index of the top nonzero digit (findk), a
// shift by whole digits (shift), and multiplication and division by one
// digit (multd, quod).  Here each is a batched device entry over [n][m]
// limbs, u32 or u64:
//   * bi_cmp / bi_findk: one warp per instance, scanning rows of 32 limbs
//     from the most significant end with ballots;
//   * bi_shift: element-wise, one thread per output limb;
//   * bi_muld: one warp per instance; a*d is the sum of the low halves of the
//     limb products and the high halves shifted up one limb, added with the
//     warp-ballot carry lookahead;
//   * bi_quod: one thread per instance, long division from the top limb with
//     the 2-by-1 division by a precomputed reciprocal of Moller and Granlund
//     ("Improved division by invariant integers", IEEE Trans. Computers
//     60(2), 2011, Algorithm 4), on the u64 view of the instance.
#include "common.cuh"
#include "divlimb.cuh"   // recip_limb, div_2by1

namespace bi {

constexpr int PRIM_CTA = 256;   // 8 warps, one instance each

// ---------------------------------------------------------------------------
// compare: out = -1, 0, 1 as a <, ==, > b  (div.c lt/eq, :49-62)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(PRIM_CTA) cmp_kernel(const T* a, const T* b, int8_t* out, uint32_t m, uint64_t n) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (PRIM_CTA / 32);
    for (uint64_t inst = (uint64_t)blockIdx.x * (PRIM_CTA / 32) + (threadIdx.x >> 5); inst < n; inst += warps) {
        const T* x = a + inst * m;
        const T* y = b + inst * m;
        int res = 0;
        for (int64_t base = (int64_t)((m - 1) / 32) * 32; base >= 0; base -= 32) {
            const int64_t i = base + lane;
            const T xv = i < (int64_t)m ? x[i] : 0, yv = i < (int64_t)m ? y[i] : 0;
            const uint32_t diff = __ballot_sync(0xffffffffu, xv != yv);
            if (diff) {
                const int hi = 31 - __clz(diff);
                res = __shfl_sync(0xffffffffu, xv < yv ? -1 : 1, hi);
                break;
            }
        }
        if (lane == 0) out[inst] = (int8_t)res;
    }
}

// ---------------------------------------------------------------------------
// findk: k = index of the top nonzero limb (0 for zero), zero = (a == 0)
// (div.c findk/ez, :64-69, :92-96)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(PRIM_CTA) findk_kernel(const T* a, uint32_t* k, uint8_t* zero, uint32_t m, uint64_t n) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (PRIM_CTA / 32);
    for (uint64_t inst = (uint64_t)blockIdx.x * (PRIM_CTA / 32) + (threadIdx.x >> 5); inst < n; inst += warps) {
        const T* x = a + inst * m;
        int64_t top = -1;
        for (int64_t base = (int64_t)((m - 1) / 32) * 32; base >= 0; base -= 32) {
            const int64_t i = base + lane;
            const uint32_t nz = __ballot_sync(0xffffffffu, i < (int64_t)m && x[i] != 0);
            if (nz) {
                top = base + 31 - __clz(nz);
                break;
            }
        }
        if (lane == 0) {
            if (k) k[inst] = top < 0 ? 0u : (uint32_t)top;
            if (zero) zero[inst] = top < 0 ? 1 : 0;
        }
    }
}

// ---------------------------------------------------------------------------
// shift by whole digits (div.c shift, :104-117): digits >= 0 moves limbs up,
// r = a * B^digits mod B^m; digits < 0 moves them down, r = a / B^-digits.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void shift_kernel(const T* a, T* r, int32_t digits, uint32_t m, uint64_t n) {
    const uint64_t total = n * m;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t inst = idx / m;
        const int64_t i = (int64_t)(idx - inst * m);
        const int64_t src = i - digits;
        r[idx] = (src >= 0 && src < (int64_t)m) ? a[inst * m + src] : (T)0;
    }
}

// ---------------------------------------------------------------------------
// muld: r = a * d mod B^m, d one limb per instance (div.c multd, :197-217)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void limb_mul(uint64_t x, uint64_t d, uint64_t& lo, uint64_t& hi) {
    lo = x * d;
    hi = __umul64hi(x, d);
}
__device__ __forceinline__ void limb_mul(uint32_t x, uint32_t d, uint32_t& lo, uint32_t& hi) {
    const uint64_t p = (uint64_t)x * d;
    lo = (uint32_t)p;
    hi = (uint32_t)(p >> 32);
}

template <typename T>
__global__ void __launch_bounds__(PRIM_CTA) muld_kernel(const T* a, const T* dv, T* r, uint32_t m, uint64_t n) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (PRIM_CTA / 32);
    for (uint64_t inst = (uint64_t)blockIdx.x * (PRIM_CTA / 32) + (threadIdx.x >> 5); inst < n; inst += warps) {
        const T* x = a + inst * m;
        T* out = r + inst * m;
        const T d = dv[inst];
        T hi_prev = 0;       // high half of the limb below this row's lane 0
        uint32_t cin = 0;
        for (uint32_t base = 0; base < m; base += 32) {
            const uint32_t i = base + lane;
            T lo = 0, hi = 0;
            if (i < m) limb_mul(x[i], d, lo, hi);
            // limb i of a*d is lo_i + hi_{i-1} (+ carries)
            T h = __shfl_up_sync(0xffffffffu, hi, 1);
            if (lane == 0) h = hi_prev;
            hi_prev = __shfl_sync(0xffffffffu, hi, 31);
            const T s = lo + h;
            const uint32_t g = s < lo, p = s == (T)~(T)0;
            const uint32_t A = __ballot_sync(0xffffffffu, g | p);
            const uint32_t B = __ballot_sync(0xffffffffu, g);
            const WarpCarry wc = warp_carry_resolve(A, B, cin);
            cin = wc.cout;
            if (i < m) out[i] = s + (T)((wc.carries >> lane) & 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// quod: q = floor(a / d), rem = a mod d, d one limb per instance
// (div.c quod, :165-181); d = 0 gives q = 0 and rem = 0.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ uint64_t limb64_of(const T* x, uint32_t m, uint32_t i) {
    if constexpr (sizeof(T) == 8) {
        return x[i];
    } else {
        const uint64_t lo = 2 * i < m ? x[2 * i] : 0;
        const uint64_t hi = 2 * i + 1 < m ? x[2 * i + 1] : 0;
        return lo | (hi << 32);
    }
}
template <typename T>
__device__ __forceinline__ void put_limb64_of(T* x, uint32_t m, uint32_t i, uint64_t v) {
    if constexpr (sizeof(T) == 8) {
        x[i] = v;
    } else {
        if (2 * i < m) x[2 * i] = (uint32_t)v;
        if (2 * i + 1 < m) x[2 * i + 1] = (uint32_t)(v >> 32);
    }
}

template <typename T>
__global__ void quod_kernel(const T* a, const T* dv, T* q, T* rem, uint32_t m, uint64_t n) {
    const uint32_t L = sizeof(T) == 8 ? m : (m + 1) / 2;   // u64-view limbs
    for (uint64_t inst = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; inst < n;
         inst += (uint64_t)gridDim.x * blockDim.x) {
        const T* x = a + inst * m;
        T* qo = q + inst * m;
        const uint64_t d0 = (uint64_t)dv[inst];
        if (d0 == 0) {
            for (uint32_t i = 0; i < m; i++) qo[i] = 0;
            if (rem) rem[inst] = 0;
            continue;
        }
        const int s = __clzll((long long)d0);
        const uint64_t d = d0 << s;
        const uint64_t v = recip_limb(d);
        // long division of (a << s) by d, top limb first; r < d throughout
        uint64_t r = s ? limb64_of(x, m, L - 1) >> (64 - s) : 0;
        for (int64_t i = (int64_t)L - 1; i >= 0; i--) {
            const uint64_t cur = limb64_of(x, m, (uint32_t)i);
            const uint64_t below = (s && i > 0) ? limb64_of(x, m, (uint32_t)i - 1) >> (64 - s) : 0;
            const uint64_t u0 = (cur << s) | below;
            uint64_t nr;
            const uint64_t qi = div_2by1(r, u0, d, v, nr);
            put_limb64_of(qo, m, (uint32_t)i, qi);
            r = nr;
        }
        if (rem) rem[inst] = (T)(r >> s);
    }
}

// ---------------------------------------------------------------------------

template <typename T>
static bi_status check_args(const void* a, const void* b, const void* r, uint32_t m, uint64_t n) {
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!a) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)a % sizeof(T) || (uintptr_t)b % sizeof(T) || (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    if (n * (uint64_t)m > (1ull << 46)) return set_error(BI_EINVAL, "n*m too large");
    return BI_OK;
}

static unsigned warp_grid(uint64_t n) {
    const uint64_t blocks = (n + PRIM_CTA / 32 - 1) / (PRIM_CTA / 32);
    const uint64_t cap = (uint64_t)num_sms() * 64;
    return (unsigned)(blocks < cap ? blocks : cap);
}

template <typename T>
static bi_status cmp_entry(const T* a, const T* b, int8_t* out, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (!b || !out) return set_error(BI_EINVAL, "NULL buffer");
    BI_RETURN_IF(check_args<T>(a, b, out, m, n));
    cmp_kernel<T><<<warp_grid(n), PRIM_CTA, 0, (cudaStream_t)s>>>(a, b, out, m, n);
    return check_launch("cmp kernel");
}

template <typename T>
static bi_status findk_entry(const T* a, uint32_t* k, uint8_t* zero, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (!k && !zero) return set_error(BI_EINVAL, "findk: k and zero are both NULL");
    if ((uintptr_t)k % 4) return set_error(BI_EINVAL, "findk: k must be 4-byte aligned");
    BI_RETURN_IF(check_args<T>(a, nullptr, a, m, n));
    findk_kernel<T><<<warp_grid(n), PRIM_CTA, 0, (cudaStream_t)s>>>(a, k, zero, m, n);
    return check_launch("findk kernel");
}

template <typename T>
static bi_status shift_entry(const T* a, T* r, int32_t digits, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (!r) return set_error(BI_EINVAL, "NULL buffer");
    BI_RETURN_IF(check_args<T>(a, nullptr, r, m, n));
    if (a == r && digits != 0) return set_error(BI_EINVAL, "shift: r must not alias a");
    const uint64_t total = n * m;
    const uint64_t blocks = (total + 255) / 256;
    const uint64_t cap = (uint64_t)num_sms() * 32;
    shift_kernel<T><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, (cudaStream_t)s>>>(a, r, digits, m, n);
    return check_launch("shift kernel");
}

template <typename T>
static bi_status muld_entry(const T* a, const T* d, T* r, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (!d || !r) return set_error(BI_EINVAL, "NULL buffer");
    BI_RETURN_IF(check_args<T>(a, d, r, m, n));
    muld_kernel<T><<<warp_grid(n), PRIM_CTA, 0, (cudaStream_t)s>>>(a, d, r, m, n);
    return check_launch("muld kernel");
}

template <typename T>
static bi_status quod_entry(const T* a, const T* d, T* q, T* rem, uint32_t m, uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (!d || !q) return set_error(BI_EINVAL, "NULL buffer");
    BI_RETURN_IF(check_args<T>(a, d, q, m, n));
    if ((uintptr_t)rem % sizeof(T)) return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    if (q == a) return set_error(BI_EINVAL, "quod: q must not alias a");
    const uint64_t blocks = (n + 127) / 128;
    const uint64_t cap = (uint64_t)num_sms() * 16;
    quod_kernel<T><<<(unsigned)(blocks < cap ? blocks : cap), 128, 0, (cudaStream_t)s>>>(a, d, q, rem, m, n);
    return check_launch("quod kernel");
}

}  // namespace bi

using namespace bi;

extern "C" {

bi_status bi_cmp_u64(const uint64_t* a, const uint64_t* b, int8_t* out, uint32_t m, uint64_t n, bi_stream s) {
    return cmp_entry<uint64_t>(a, b, out, m, n, s);
}
bi_status bi_cmp_u32(const uint32_t* a, const uint32_t* b, int8_t* out, uint32_t m, uint64_t n, bi_stream s) {
    return cmp_entry<uint32_t>(a, b, out, m, n, s);
}
bi_status bi_findk_u64(const uint64_t* a, uint32_t* k, uint8_t* zero, uint32_t m, uint64_t n, bi_stream s) {
    return findk_entry<uint64_t>(a, k, zero, m, n, s);
}
bi_status bi_findk_u32(const uint32_t* a, uint32_t* k, uint8_t* zero, uint32_t m, uint64_t n, bi_stream s) {
    return findk_entry<uint32_t>(a, k, zero, m, n, s);
}
bi_status bi_shift_u64(const uint64_t* a, uint64_t* r, int32_t digits, uint32_t m, uint64_t n, bi_stream s) {
    return shift_entry<uint64_t>(a, r, digits, m, n, s);
}
bi_status bi_shift_u32(const uint32_t* a, uint32_t* r, int32_t digits, uint32_t m, uint64_t n, bi_stream s) {
    return shift_entry<uint32_t>(a, r, digits, m, n, s);
}
bi_status bi_muld_u64(const uint64_t* a, const uint64_t* d, uint64_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return muld_entry<uint64_t>(a, d, r, m, n, s);
}
bi_status bi_muld_u32(const uint32_t* a, const uint32_t* d, uint32_t* r, uint32_t m, uint64_t n, bi_stream s) {
    return muld_entry<uint32_t>(a, d, r, m, n, s);
}
bi_status bi_quod_u64(const uint64_t* a, const uint64_t* d, uint64_t* q, uint64_t* rem, uint32_t m, uint64_t n,
                      bi_stream s) {
    return quod_entry<uint64_t>(a, d, q, rem, m, n, s);
}
bi_status bi_quod_u32(const uint32_t* a, const uint32_t* d, uint32_t* q, uint32_t* rem, uint32_t m, uint64_t n,
                      bi_stream s) {
    return quod_entry<uint32_t>(a, d, q, rem, m, n, s);
}

}  // extern "C"
