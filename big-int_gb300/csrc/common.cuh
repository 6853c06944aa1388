// common.cuh -- shared device and host helpers of the GB300 big-integer library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bigint_gb300.h"

namespace bi {

// ---------------------------------------------------------------------------
// Limb traits.  The reference's U32bits/U64bits (cuda/ker-helpers.cu.h:28-44)
// carry a 2-word type for products; here products are formed with explicit
// mul.hi/mad instructions, so only the word type and its all-ones value are
// needed.
// ---------------------------------------------------------------------------
template <typename T> struct Limb;
template <> struct Limb<uint32_t> {
    static constexpr uint32_t HIGHEST = 0xFFFFFFFFu;
    static constexpr int BITS = 32;
};
template <> struct Limb<uint64_t> {
    static constexpr uint64_t HIGHEST = 0xFFFFFFFFFFFFFFFFull;
    static constexpr int BITS = 64;
};

// ---------------------------------------------------------------------------
// Division by a runtime constant (Granlund-Montgomery, round-up variant).
// Exact for every 32-bit numerator and divisor >= 1.
// ---------------------------------------------------------------------------
struct FastDiv {
    uint32_t d;
    uint32_t magic;
    uint32_t shift;

    __host__ __device__ FastDiv() : d(1), magic(0), shift(0) {}
    __host__ __device__ explicit FastDiv(uint32_t divisor) : d(divisor) {
        uint32_t l = 0;
        while (l < 32 && (1ull << l) < divisor) l++;
        shift = l;
        // magic = floor(2^32 * (2^l - d) / d) + 1
        magic = (uint32_t)((((1ull << l) - divisor) << 32) / divisor + 1);
    }
    __device__ __forceinline__ uint32_t div(uint32_t x) const {
        uint64_t t = __umulhi(x, magic);
        return (uint32_t)((t + x) >> shift);
    }
};

// ---------------------------------------------------------------------------
// Carry lookahead across the 32 lanes of a warp.
//
// The reference propagates a 2-bit carry class (bit0 = generates a carry,
// bit1 = propagates one) with an associative operator and a shared-memory
// block scan (CarryProp/SegCarryProp, cuda/ker-add.cu.h:10-41; scanIncBlock,
// cuda/ker-helpers.cu.h:66-95).  Here the classes of the 32 lanes are packed
// into two 32-bit ballots and resolved by one integer addition: with
// A = generate|propagate and B = generate, the carry out of bit t of A + B is
// exactly g_t | (p_t & c_t).  The carry into each lane is therefore bit t of
// (A + B + cin) ^ A ^ B, and bit 32 of the 64-bit sum is the carry out of
// lane 31.  A lane whose successor starts a new instance has its classes
// cleared so no carry crosses the instance boundary (the segment flag of
// SegCarryProp).
// ---------------------------------------------------------------------------
struct WarpCarry {
    uint32_t carries;   // bit t: carry into lane t
    uint32_t cout;      // carry out of lane 31
};

__device__ __forceinline__ WarpCarry warp_carry_resolve(uint32_t A, uint32_t B, uint32_t cin) {
    uint64_t s = (uint64_t)A + (uint64_t)B + (uint64_t)cin;
    WarpCarry w;
    w.carries = (uint32_t)s ^ A ^ B;
    w.cout = (uint32_t)(s >> 32);
    return w;
}

// Carry into each thread of a CTA for a segmented carry chain that runs over
// the threads in index order.  Thread t supplies the (generate, propagate)
// pair of its stage and `seg` = 1 if it begins a new segment (no carry
// enters it).  Returns the carry into the thread's stage.  Every thread of
// the CTA must call it (blockDim.x a multiple of 32, at most 32 warps);
// `scratch` holds 3 * 32 words of shared memory.  Contains __syncthreads.
__device__ __forceinline__ uint32_t block_carry_in(uint32_t g, uint32_t p, bool seg, uint32_t* scratch) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const uint32_t S = __ballot_sync(0xffffffffu, seg);
    const uint32_t kill = S >> 1;
    const uint32_t A = __ballot_sync(0xffffffffu, g | p) & ~kill;
    const uint32_t B = __ballot_sync(0xffffffffu, g) & ~kill;
    if (lane == 0) {
        const uint32_t g0 = warp_carry_resolve(A, B, 0).cout;
        const uint32_t g1 = warp_carry_resolve(A, B, 1).cout;
        scratch[warp] = g0;
        scratch[32 + warp] = g1 & ~g0;
        scratch[64 + warp] = S & 1u;
    }
    __syncthreads();
    const bool before = lane < warp;
    const bool killed = before && scratch[64 + (lane + 1 < nwarps ? lane + 1 : 0)];
    const bool live = before && !killed;
    const uint32_t wg = live ? scratch[lane] : 0u, wp = live ? scratch[32 + lane] : 0u;
    const uint32_t A2 = __ballot_sync(0xffffffffu, wg | wp);
    const uint32_t B2 = __ballot_sync(0xffffffffu, wg);
    uint32_t cin = (warp_carry_resolve(A2, B2, 0).carries >> warp) & 1u;
    if (S & 1u) cin = 0;
    __syncthreads();   // scratch may be reused by the caller
    return (warp_carry_resolve(A, B, cin).carries >> lane) & 1u;
}

}  // namespace bi

// ---------------------------------------------------------------------------
// Host-side status plumbing (defined in capi.cu).
// ---------------------------------------------------------------------------
#define BI_RETURN_IF(x)                \
    do {                               \
        bi_status _s = (x);            \
        if (_s != BI_OK) return _s;    \
    } while (0)

namespace bi {
bi_status set_error(bi_status st, const char* fmt, ...);
bi_status check_launch(const char* what);
int num_sms();
cudaError_t smem_opt_in(const void* func, size_t smem);
// add/sub on pinned host buffers read over the CPU-GPU link (addsub.cu)
bi_status add_link_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, bi_stream s);
bi_status add_link_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n, bi_stream s);
bi_status sub_link_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m, uint64_t n,
                       bi_stream s);
bi_status sub_link_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* sign, uint32_t m, uint64_t n,
                       bi_stream s);
}  // namespace bi
