// warpops.cuh -- one add or sign-magnitude subtraction per warp, for any m,
// with no shared memory and no CTA barrier (used by the uneven-batch and the
// serving kernels).
#pragma once

#include "common.cuh"

namespace bi {

// T: the element type, 64-bit limbs (16-byte rows when VEC = 2) or 32-bit words
template <int VEC, typename T>
__device__ __forceinline__ void ld_row(const T* p, int64_t base, uint32_t m, T (&v)[VEC]) {
    if (sizeof(T) == 8 && VEC == 2 && base >= 0 && base + 2 <= (int64_t)m) {
        const ulonglong2 x = __ldcs(reinterpret_cast<const ulonglong2*>(p + base));
        v[0] = (T)x.x;
        if constexpr (VEC == 2) v[1] = (T)x.y;
    } else {
#pragma unroll
        for (int e = 0; e < VEC; e++) v[e] = (base + e >= 0 && base + e < (int64_t)m) ? __ldcs(p + base + e) : 0;
    }
}

template <int VEC, int R, typename T = uint64_t>
__device__ void warp_addsub(const T* a, const T* b, T* r, uint8_t* sign, uint32_t m, bool sub) {
    static_assert(sizeof(T) == 8 || VEC == 1, "32-bit words one a lane per row");
    constexpr T ONES = (T)~(T)0;
    constexpr int ROWL = 32 * VEC;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nrows = (m + ROWL - 1) / ROWL;
    if (sub) {
        // which operand is larger: scan rows from the most significant end
        bool lt = false;
        for (int row = (int)nrows - 1; row >= 0; row--) {
            const int64_t base = (int64_t)row * ROWL + lane * VEC;
            T x[VEC], y[VEC];
            ld_row<VEC>(a, base, m, x);
            ld_row<VEC>(b, base, m, y);
            int top = -1;
            bool lane_lt = false;
#pragma unroll
            for (int e = 0; e < VEC; e++)
                if (x[e] != y[e]) { top = e; lane_lt = x[e] < y[e]; }
            const uint32_t diff = __ballot_sync(0xffffffffu, top >= 0);
            if (diff) {
                const int hi = 31 - __clz(diff);
                lt = __shfl_sync(0xffffffffu, lane_lt, hi);
                break;
            }
        }
        if (lt) {   // |a - b| = b - a
            const T* t = a;
            a = b;
            b = t;
        }
        if (lane == 0 && sign) *sign = lt ? 1 : 0;
    }
    uint32_t cin = 0;
    for (uint32_t row0 = 0; row0 < nrows; row0 += R) {
        T x[R][VEC], y[R][VEC];
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int64_t base = (int64_t)(row0 + rr) * ROWL + lane * VEC;
            ld_row<VEC>(a, base, m, x[rr]);
            ld_row<VEC>(b, base, m, y[rr]);
        }
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            if (row0 + rr >= nrows) break;
            T s[VEC];
            uint32_t G = 0, P = 1, gb = 0, pb = 0;
#pragma unroll
            for (int e = 0; e < VEC; e++) {
                uint32_t g, p;
                if (!sub) { s[e] = x[rr][e] + y[rr][e]; g = s[e] < x[rr][e]; p = s[e] == ONES; }
                else      { s[e] = x[rr][e] - y[rr][e]; g = x[rr][e] < y[rr][e]; p = x[rr][e] == y[rr][e]; }
                gb |= g << e;
                pb |= p << e;
                G = g | (p & G);
                P = p & P;
            }
            const uint32_t A = __ballot_sync(0xffffffffu, G | P);
            const uint32_t B = __ballot_sync(0xffffffffu, G);
            const WarpCarry wc = warp_carry_resolve(A, B, cin);
            uint32_t c = (wc.carries >> lane) & 1u;
            cin = wc.cout;
            const int64_t base = (int64_t)(row0 + rr) * ROWL + lane * VEC;
            T out[VEC];
#pragma unroll
            for (int e = 0; e < VEC; e++) {
                out[e] = sub ? s[e] - c : s[e] + c;
                c = ((gb >> e) & 1u) | (((pb >> e) & 1u) & c);
            }
            if (sizeof(T) == 8 && VEC == 2 && base + 2 <= (int64_t)m) {
                ulonglong2 v;
                v.x = (uint64_t)out[0];
                v.y = (uint64_t)out[VEC - 1];
                __stcs(reinterpret_cast<ulonglong2*>(r + base), v);
            } else {
#pragma unroll
                for (int e = 0; e < VEC; e++)
                    if (base + e < (int64_t)m) __stcs(r + base + e, out[e]);
            }
        }
    }
}

}  // namespace bi
