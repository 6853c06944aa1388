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
#include "blockops.cuh"

namespace bi {

constexpr int DIV_MAX_CORRECTIONS = 8;

struct DivGeom {
    uint32_t mu, mv;        // limbs per dividend / divisor in the caller's type
    uint32_t MU, MV;        // the same in 64-bit limbs
    uint32_t Pmax;          // largest reciprocal precision (limbs)
    uint32_t oUn, oVn, oY, oX;
    uint32_t oVs, oT, oProd, oW;             // phase N (Newton) offsets inside X
    uint32_t oBig, oQ, oQV, oR, oW2;         // phases Q/R offsets inside X
    uint32_t smem_limbs;
};

// floor((2^128 - 1) / d) - 2^64 for d >= 2^63: the low limb of a one-limb
// reciprocal (the quotient is in (2^64, 2^65)).  Restoring long division of
// (~d) * 2^64 + (2^64 - 1) by d; ~d < d so the quotient fits 64 bits.
__device__ __forceinline__ uint64_t recip_limb(uint64_t d) {
    uint64_t rem = ~d, q = 0;
    for (int i = 0; i < 64; i++) {
        const uint64_t top = rem >> 63;
        rem = (rem << 1) | 1ull;
        q <<= 1;
        if (top || rem >= d) {
            rem -= d;
            q |= 1ull;
        }
    }
    return q;
}

template <typename T>
__device__ __forceinline__ void load_limbs64(uint64_t* dst, const T* src, uint32_t count_T, uint32_t L) {
    for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) {
        uint64_t x;
        if constexpr (sizeof(T) == 8) {
            x = i < count_T ? src[i] : 0;
        } else {
            x = 2 * i < count_T ? src[2 * i] : 0u;
            if (2 * i + 1 < count_T) x |= (uint64_t)src[2 * i + 1] << 32;
        }
        dst[i] = x;
    }
}

template <typename T>
__device__ __forceinline__ void store_limbs64(T* dst, uint32_t count_T, const uint64_t* src, uint32_t L) {
    for (uint32_t i = threadIdx.x; i < count_T; i += blockDim.x) {
        if constexpr (sizeof(T) == 8) {
            dst[i] = i < L ? src[i] : 0;
        } else {
            const uint32_t li = i / 2;
            const uint64_t x = li < L ? src[li] : 0;
            dst[i] = (i & 1) ? (uint32_t)(x >> 32) : (uint32_t)x;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(512)
div_kernel(const T* __restrict__ u, const T* __restrict__ v, T* __restrict__ q, T* __restrict__ r,
           uint8_t* __restrict__ status, uint64_t n, DivGeom g) {
    extern __shared__ __align__(16) uint64_t smem[];
    uint64_t* Un = smem + g.oUn;
    uint64_t* Vn = smem + g.oVn;
    uint64_t* Yb = smem + g.oY;
    uint64_t* X = smem + g.oX;
    uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + g.smem_limbs);
    const uint32_t MU = g.MU, MV = g.MV, Pmax = g.Pmax;

    for (uint64_t inst = blockIdx.x; inst < n; inst += gridDim.x) {
        const T* ui = u + inst * g.mu;
        const T* vi = v + inst * g.mv;
        T* qi = q + inst * g.mu;
        T* ri = r + inst * g.mv;

        // ---- raw operands: u into X[0, MU), v into X[MU, MU+MV)
        uint64_t* Uraw = X;
        uint64_t* Vraw = X + MU;
        load_limbs64<T>(Uraw, ui, g.mu, MU);
        load_limbs64<T>(Vraw, vi, g.mv, MV);
        __syncthreads();
        const int K = block_prec(Vraw, (int)MV, scratch);
        if (K == 0) {                                  // division by zero
            store_limbs64<T>(qi, g.mu, Un, 0);
            store_limbs64<T>(ri, g.mv, Un, 0);
            if (status && threadIdx.x == 0) status[inst] = 1;
            __syncthreads();
            continue;
        }
        const int s = __clzll((long long)Vraw[K - 1]);
        block_shl_bits(Vn, Vraw, K, K, s);
        block_shl_bits(Un, Uraw, (int)MU, (int)MU + 1, s);
        __syncthreads();
        const int H = block_prec(Un, (int)MU + 1, scratch);
        if (H < K) {                                   // u < v: q = 0, r = u
            store_limbs64<T>(qi, g.mu, Un, 0);
            store_limbs64<T>(ri, g.mv, Uraw, MU);
            if (status && threadIdx.x == 0) status[inst] = 0;
            __syncthreads();
            continue;
        }
        const int Qlen = H - K + 1;
        const int P = Qlen + 1;

        // ---- shifted inverse: Y_p at Yb + (Pmax - p), p + 1 limbs
        if (threadIdx.x == 0) {
            Yb[Pmax - 1] = recip_limb(Vn[K - 1]);
            Yb[Pmax] = 1;
            Yb[Pmax + 1] = 0;
        }
        int sched[40];
        int ns = 0;
        {
            int x = P;
            sched[ns++] = x;
            while (x > 2 && ns < 40) {
                x = (x + 2) / 2;
                sched[ns++] = x;
            }
        }
        __syncthreads();
        int p = 1;
        uint64_t* Vs = X + g.oVs;
        uint64_t* Tb = X + g.oT;
        uint64_t* Pr = X + g.oProd;
        uint64_t* Wb = X + g.oW;
        for (int si = ns - 1; si >= 0; si--) {
            const int pn = sched[si];
            if (pn <= p) continue;
            const int sl = pn + 1;
            // divisor prefix: the top sl limbs of v (zero-extended below when K < sl)
            for (int i = threadIdx.x; i < sl; i += blockDim.x) {
                const int src = K - sl + i;
                Vs[i] = src >= 0 ? Vn[src] : 0;
            }
            __syncthreads();
            const uint64_t* Yp = Yb + (Pmax - p);
            // T = Vs * Y_p mod B^(sl+1); E = B^(sl+p) - Vs*Y_p, |E| < B^(sl+1)/2
            block_mul(Vs, sl, Yp, p + 1, Tb, sl + 1, Wb, scratch);
            const bool e_neg = (Tb[sl] >> 63) == 0;    // T small: E = -T
            if (!e_neg) block_addsub(Tb, nullptr, 0, Tb, sl + 1, sl + 1, true, scratch);   // |E| = -T
            // D = floor(Y_p * |E| / B^(2p+1))
            block_mul(Yp, p + 1, Tb, sl + 1, Pr, p + sl + 2, Wb, scratch);
            const uint64_t* D = Pr + 2 * p + 1;
            const int Dlen = sl - p + 1;
            // Y_pn = Y_p * B^(pn-p) +/- D
            for (int i = threadIdx.x; i < pn - p; i += blockDim.x) Yb[Pmax - pn + i] = 0;
            __syncthreads();
            uint64_t* Ypn = Yb + (Pmax - pn);
            block_addsub(Ypn, Ypn, pn + 1, D, Dlen, pn + 1, e_neg, scratch);
            p = pn;
        }
        const uint64_t* Y = Yb + (Pmax - P);

        // ---- quotient estimate: floor(Un * Y / B^(P+K))
        uint64_t* Big = X + g.oBig;
        uint64_t* Qb = X + g.oQ;
        uint64_t* QV = X + g.oQV;
        uint64_t* Rb = X + g.oR;
        uint64_t* W2 = X + g.oW2;
        block_mul(Un, H, Y, P + 1, Big, H + P + 1, W2, scratch);
        for (int i = threadIdx.x; i < Qlen + 1; i += blockDim.x) Qb[i] = i < Qlen ? Big[P + K + i] : 0;
        __syncthreads();

        // ---- remainder r = u - q*v from the low K+1 limbs, then corrections
        block_mul(Qb, Qlen + 1, Vn, K, QV, K + 1, W2, scratch);
        block_addsub(Rb, Un, K + 1, QV, K + 1, K + 1, true, scratch);
        int fixes = 0;
        bool ok = true;
        while ((Rb[K] >> 63) != 0) {                  // r < 0
            if (++fixes > DIV_MAX_CORRECTIONS) { ok = false; break; }
            block_addsub(Rb, Rb, K + 1, Vn, K, K + 1, false, scratch);
            // q -= 1
            uint64_t* onebuf = QV;                     // QV is free now
            if (threadIdx.x == 0) onebuf[0] = 1;
            __syncthreads();
            block_addsub(Qb, Qb, Qlen + 1, onebuf, 1, Qlen + 1, true, scratch);
        }
        fixes = 0;
        while (ok && block_cmp(Rb, K + 1, Vn, K, K + 1, scratch) >= 0) {   // r >= v
            if (++fixes > DIV_MAX_CORRECTIONS) { ok = false; break; }
            block_addsub(Rb, Rb, K + 1, Vn, K, K + 1, true, scratch);
            uint64_t* onebuf = QV;
            if (threadIdx.x == 0) onebuf[0] = 1;
            __syncthreads();
            block_addsub(Qb, Qb, Qlen + 1, onebuf, 1, Qlen + 1, false, scratch);
        }

        // ---- outputs: q, and r shifted back by s bits
        uint64_t* Rout = QV;
        block_shr_bits(Rout, Rb, K, K, s);
        __syncthreads();
        store_limbs64<T>(qi, g.mu, Qb, (uint32_t)(Qlen + 1 < (int)MU ? Qlen + 1 : MU));
        store_limbs64<T>(ri, g.mv, Rout, (uint32_t)K);
        if (status && threadIdx.x == 0) status[inst] = ok ? 0 : 2;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------

constexpr uint32_t DIV_MAX_MU64 = 2048;   // dividend limbs (u64 view) per instance

static DivGeom div_geom(uint32_t mu, uint32_t mv, int wbytes) {
    DivGeom g;
    g.mu = mu;
    g.mv = mv;
    g.MU = wbytes == 8 ? mu : (mu + 1) / 2;
    g.MV = wbytes == 8 ? mv : (mv + 1) / 2;
    g.Pmax = g.MU + 2;
    const uint32_t MU = g.MU, MV = g.MV, Pm = g.Pmax;
    g.oUn = 0;
    g.oVn = g.oUn + MU + 2;
    g.oY = g.oVn + MV + 2;
    g.oX = g.oY + Pm + 4;
    // phase N
    g.oVs = 0;
    g.oT = g.oVs + Pm + 4;
    g.oProd = g.oT + Pm + 4;
    const uint32_t prodlen = 2 * Pm + 8;
    g.oW = g.oProd + prodlen;
    const uint32_t endN = g.oW + (prodlen + 7) / 8 * 10 + 10;
    // phases Q and R
    const uint32_t biglen = MU + Pm + 4;
    g.oBig = 0;
    g.oQ = g.oBig + biglen;
    g.oQV = g.oQ + Pm + 4;
    g.oR = g.oQV + (MV + 4 > Pm + 4 ? MV + 4 : Pm + 4);
    g.oW2 = g.oR + MV + 4;
    const uint32_t endQ = g.oW2 + (biglen + 7) / 8 * 10 + 10;
    // the raw operands are staged in X too
    uint32_t endX = endN > endQ ? endN : endQ;
    if (endX < MU + MV) endX = MU + MV;
    g.smem_limbs = g.oX + endX;
    return g;
}

template <typename T>
static bi_status div_entry(const T* u, const T* v, T* q, T* r, uint8_t* status, uint32_t mu, uint32_t mv,
                           uint64_t n, bi_stream s) {
    if (n == 0) return BI_OK;
    if (mu == 0 || mv == 0) return set_error(BI_EINVAL, "mu and mv must be >= 1");
    if (mv > mu) return set_error(BI_EINVAL, "divisor limbs mv=%u exceed dividend limbs mu=%u", mv, mu);
    if (!u || !v || !q || !r) return set_error(BI_EINVAL, "NULL buffer");
    if ((uintptr_t)u % sizeof(T) || (uintptr_t)v % sizeof(T) || (uintptr_t)q % sizeof(T) ||
        (uintptr_t)r % sizeof(T))
        return set_error(BI_EINVAL, "buffers must be aligned to the limb size");
    const DivGeom g = div_geom(mu, mv, (int)sizeof(T));
    if (g.MU > DIV_MAX_MU64) return set_error(BI_EUNSUPPORTED, "div: dividend of %u limbs above the supported size", mu);
    const size_t smem = (size_t)g.smem_limbs * 8 + BLOCKOPS_SCRATCH_WORDS * 4;
    if (smem > 227 * 1024) return set_error(BI_EUNSUPPORTED, "div: sizes need too much shared memory");
    const int threads = g.MU >= 1024 ? 512 : g.MU >= 256 ? 256 : g.MU >= 64 ? 128 : g.MU >= 16 ? 64 : 32;
    auto kern = div_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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

}  // extern "C"
