// multhread.cuh -- products (full or truncated) of at most 24 64-bit limbs,
// one thread per instance.
//
// A thread holds both operands in registers (M 64-bit limbs each, M a
// compile-time size) and forms the product (2M limbs, or the low M) column by column
// (product scanning, Comba's method): column c adds a_i * b_{c-i} for every
// i into a three-limb accumulator -- one mul.lo/mul.hi pair and an
// add/addc/addc chain a term -- emits the low limb and shifts the
// accumulator down.  The triangle is exact (M^2 terms, none padded), no
// thread waits on another, and the one accumulator keeps ptxas from
// hoisting the whole triangle's products into registers (independent
// per-column accumulators did, at 250 registers a thread, and ran slower).
#pragma once
#include <cstdint>

namespace bi {

constexpr uint32_t MUL_THREAD_MAX_L = 24;        // largest operand of a full product, in 64-bit limbs
constexpr uint32_t MUL_THREAD_TRUNC_MAX_L = 32;  // of a truncated one (about half the terms)

// Instances (threads) per CTA: 128, or 64 above 16 limbs, where 128 rows of
// staged operands would pass the 48 KB of static shared memory.
template <int M>
__host__ __device__ constexpr uint32_t mul_thread_cta() { return M <= 16 ? 128u : 64u; }

// (c2:c1:c0) += x * y, the carry count c2 in 32 bits (a column's count stays
// below 2M), which saves an ALU instruction a term against a 64-bit c2 and
// measured 4-9 % faster at 12 to 24 limbs
__device__ __forceinline__ void mac3(uint64_t& c0, uint64_t& c1, uint32_t& c2, uint64_t x, uint64_t y) {
    asm("{\n\t.reg .u64 t;\n\t"
        "mul.lo.u64 t, %3, %4;\n\tadd.cc.u64 %0, %0, t;\n\t"
        "mul.hi.u64 t, %3, %4;\n\taddc.cc.u64 %1, %1, t;\n\t"
        "addc.u32 %2, %2, 0;\n\t}"
        : "+l"(c0), "+l"(c1), "+r"(c2)
        : "l"(x), "l"(y));
}

// The product of x and y (M limbs each): the full 2M limbs (FULL), or the
// low M (the product mod B^M: only the columns below M are formed, about
// half the terms); put(c, limb) receives the limbs in order.  A column holds
// at most M terms below 2^128, so with the carry from the column below the
// accumulator stays below 2^160.
template <int M, bool FULL, typename Put>
__device__ __forceinline__ void mul_thread_product(const uint64_t (&x)[M], const uint64_t (&y)[M], Put put) {
    constexpr int COLS = FULL ? 2 * M - 1 : M;
    uint64_t c0 = 0, c1 = 0;
    uint32_t c2 = 0;
#pragma unroll
    for (int c = 0; c < COLS; ++c) {
#pragma unroll
        for (int i = (c - M + 1 > 0 ? c - M + 1 : 0); i <= (c < M - 1 ? c : M - 1); ++i)
            mac3(c0, c1, c2, x[i], y[c - i]);
        put(c, c0);
        c0 = c1;
        c1 = c2;
        c2 = 0;
    }
    if constexpr (FULL) put(2 * M - 1, c0);
}

}  // namespace bi
