// chain.cuh -- 8-limb carry chains on the hardware carry flag.
//
// add.cc/addc.cc (sub.cc/subc.cc) pass the carry (borrow) from one limb to
// the next in the condition code, which does not survive from one asm
// statement to the next, so each 8-limb step is one asm block.  The carry-in
// c (0 or 1) enters through a 32-bit add of c + 0xFFFFFFFF (carry iff c = 1)
// or 0 - c (borrow iff c = 1); the carry-out is read back with addc/subc of
// zeros.
#pragma once

#include <stdint.h>

namespace bi {

#define BI_CH_OPS(OPC, TY)                                                                               \
    OPC "." TY " %0, %0, %9;\n\t" OPC "." TY " %1, %1, %10;\n\t" OPC "." TY " %2, %2, %11;\n\t" OPC "." TY \
        " %3, %3, %12;\n\t" OPC "." TY " %4, %4, %13;\n\t" OPC "." TY " %5, %5, %14;\n\t" OPC "." TY        \
        " %6, %6, %15;\n\t" OPC "." TY " %7, %7, %16;\n\t"

#define BI_CH_OUTS(C) \
    "+" C(x[0]), "+" C(x[1]), "+" C(x[2]), "+" C(x[3]), "+" C(x[4]), "+" C(x[5]), "+" C(x[6]), "+" C(x[7])
#define BI_CH_INS(C) C(y[0]), C(y[1]), C(y[2]), C(y[3]), C(y[4]), C(y[5]), C(y[6]), C(y[7])

// x = x + y + c over 8 limbs; returns the carry out (0 or 1).
#define BI_DEF_ADD8(NAME, T, TY, C)                                                          \
    __device__ __forceinline__ uint32_t NAME(T (&x)[8], const T (&y)[8], uint32_t c) {       \
        uint32_t co;                                                                         \
        asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %17, 0xFFFFFFFF;\n\t" BI_CH_OPS("addc.cc", TY) \
            "addc.u32 %8, 0, 0;\n\t}"                                                        \
            : BI_CH_OUTS(C), "=r"(co)                                                        \
            : BI_CH_INS(C), "r"(c));                                                         \
        return co;                                                                           \
    }

// x = x - y - c over 8 limbs; returns the borrow out (0 or 1).
#define BI_DEF_SUB8(NAME, T, TY, C)                                                          \
    __device__ __forceinline__ uint32_t NAME(T (&x)[8], const T (&y)[8], uint32_t c) {       \
        uint32_t bo;                                                                         \
        asm("{\n\t.reg .u32 t;\n\tsub.cc.u32 t, 0, %17;\n\t" BI_CH_OPS("subc.cc", TY)         \
            "subc.u32 %8, 0, 0;\n\t}"                                                        \
            : BI_CH_OUTS(C), "=r"(bo)                                                        \
            : BI_CH_INS(C), "r"(c));                                                         \
        return bo & 1u;                                                                      \
    }

BI_DEF_ADD8(chain_add8, uint64_t, "u64", "l")
BI_DEF_SUB8(chain_sub8, uint64_t, "u64", "l")
BI_DEF_ADD8(chain_add8, uint32_t, "u32", "r")
BI_DEF_SUB8(chain_sub8, uint32_t, "u32", "r")

#undef BI_DEF_ADD8
#undef BI_DEF_SUB8
#undef BI_CH_OPS
#undef BI_CH_OUTS
#undef BI_CH_INS

// x = x - y - c over N = 1, 2 or 4 limbs of 64 bits; returns the borrow out.
__device__ __forceinline__ uint32_t chain_sub_n(uint64_t (&x)[1], const uint64_t (&y)[1], uint32_t c) {
    uint32_t bo;
    asm("{\n\t.reg .u32 t;\n\tsub.cc.u32 t, 0, %3;\n\tsubc.cc.u64 %0, %0, %2;\n\tsubc.u32 %1, 0, 0;\n\t}"
        : "+l"(x[0]), "=r"(bo)
        : "l"(y[0]), "r"(c));
    return bo & 1u;
}
__device__ __forceinline__ uint32_t chain_sub_n(uint64_t (&x)[2], const uint64_t (&y)[2], uint32_t c) {
    uint32_t bo;
    asm("{\n\t.reg .u32 t;\n\tsub.cc.u32 t, 0, %5;\n\tsubc.cc.u64 %0, %0, %3;\n\tsubc.cc.u64 %1, %1, %4;\n\t"
        "subc.u32 %2, 0, 0;\n\t}"
        : "+l"(x[0]), "+l"(x[1]), "=r"(bo)
        : "l"(y[0]), "l"(y[1]), "r"(c));
    return bo & 1u;
}
__device__ __forceinline__ uint32_t chain_sub_n(uint64_t (&x)[4], const uint64_t (&y)[4], uint32_t c) {
    uint32_t bo;
    asm("{\n\t.reg .u32 t;\n\tsub.cc.u32 t, 0, %9;\n\tsubc.cc.u64 %0, %0, %5;\n\tsubc.cc.u64 %1, %1, %6;\n\t"
        "subc.cc.u64 %2, %2, %7;\n\tsubc.cc.u64 %3, %3, %8;\n\tsubc.u32 %4, 0, 0;\n\t}"
        : "+l"(x[0]), "+l"(x[1]), "+l"(x[2]), "+l"(x[3]), "=r"(bo)
        : "l"(y[0]), "l"(y[1]), "l"(y[2]), "l"(y[3]), "r"(c));
    return bo & 1u;
}
// Any N that is 1, 2, 4 or a multiple of 8: blocks of 8 pass the borrow on.
template <int N>
__device__ __forceinline__ uint32_t chain_sub(uint64_t (&x)[N], const uint64_t (&y)[N], uint32_t c) {
    if constexpr (N == 1 || N == 2 || N == 4) {
        return chain_sub_n(x, y, c);
    } else {
        static_assert(N % 8 == 0, "chain_sub: N must be 1, 2, 4 or a multiple of 8");
#pragma unroll
        for (int b = 0; b < N / 8; b++)
            c = chain_sub8(*reinterpret_cast<uint64_t(*)[8]>(&x[8 * b]),
                           *reinterpret_cast<const uint64_t(*)[8]>(&y[8 * b]), c);
        return c;
    }
}

__device__ __forceinline__ uint32_t chain_add_n(uint64_t (&x)[1], const uint64_t (&y)[1], uint32_t c) {
    uint32_t co;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %3, 0xFFFFFFFF;\n\taddc.cc.u64 %0, %0, %2;\n\taddc.u32 %1, 0, 0;\n\t}"
        : "+l"(x[0]), "=r"(co)
        : "l"(y[0]), "r"(c));
    return co;
}
__device__ __forceinline__ uint32_t chain_add_n(uint64_t (&x)[2], const uint64_t (&y)[2], uint32_t c) {
    uint32_t co;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %5, 0xFFFFFFFF;\n\taddc.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\t"
        "addc.u32 %2, 0, 0;\n\t}"
        : "+l"(x[0]), "+l"(x[1]), "=r"(co)
        : "l"(y[0]), "l"(y[1]), "r"(c));
    return co;
}
__device__ __forceinline__ uint32_t chain_add_n(uint64_t (&x)[4], const uint64_t (&y)[4], uint32_t c) {
    uint32_t co;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %9, 0xFFFFFFFF;\n\taddc.cc.u64 %0, %0, %5;\n\taddc.cc.u64 %1, %1, %6;\n\t"
        "addc.cc.u64 %2, %2, %7;\n\taddc.cc.u64 %3, %3, %8;\n\taddc.u32 %4, 0, 0;\n\t}"
        : "+l"(x[0]), "+l"(x[1]), "+l"(x[2]), "+l"(x[3]), "=r"(co)
        : "l"(y[0]), "l"(y[1]), "l"(y[2]), "l"(y[3]), "r"(c));
    return co;
}
template <int N>
__device__ __forceinline__ uint32_t chain_add(uint64_t (&x)[N], const uint64_t (&y)[N], uint32_t c) {
    if constexpr (N == 1 || N == 2 || N == 4) {
        return chain_add_n(x, y, c);
    } else {
        static_assert(N % 8 == 0, "chain_add: N must be 1, 2, 4 or a multiple of 8");
#pragma unroll
        for (int b = 0; b < N / 8; b++)
            c = chain_add8(*reinterpret_cast<uint64_t(*)[8]>(&x[8 * b]),
                           *reinterpret_cast<const uint64_t(*)[8]>(&y[8 * b]), c);
        return c;
    }
}

// x[0..N-1] -= (gen(OFF), gen(OFF + 1), ...) + c, for any N >= 1: blocks of 8
// limbs, then one of 4, 2 and 1 for the rest, each an asm chain, the borrow
// handed from block to block.  Returns the borrow out.
template <int N, int OFF = 0, typename Gen>
__device__ __forceinline__ uint32_t chain_sub_gen(uint64_t* x, Gen gen, uint32_t c) {
    static_assert(N >= 1, "chain_sub_gen: N >= 1");
    constexpr int Bk = N >= 8 ? 8 : N >= 4 ? 4 : N >= 2 ? 2 : 1;
    uint64_t y[Bk];
#pragma unroll
    for (int j = 0; j < Bk; j++) y[j] = gen(OFF + j);
    c = chain_sub<Bk>(*reinterpret_cast<uint64_t(*)[Bk]>(x), y, c);
    if constexpr (N > Bk) c = chain_sub_gen<N - Bk, OFF + Bk>(x + Bk, gen, c);
    return c;
}

// x[0..N-1] += (gen(OFF), gen(OFF + 1), ...) + c, for any N >= 1; returns the carry out.
template <int N, int OFF = 0, typename Gen>
__device__ __forceinline__ uint32_t chain_add_gen(uint64_t* x, Gen gen, uint32_t c) {
    static_assert(N >= 1, "chain_add_gen: N >= 1");
    constexpr int Bk = N >= 8 ? 8 : N >= 4 ? 4 : N >= 2 ? 2 : 1;
    uint64_t y[Bk];
#pragma unroll
    for (int j = 0; j < Bk; j++) y[j] = gen(OFF + j);
    c = chain_add<Bk>(*reinterpret_cast<uint64_t(*)[Bk]>(x), y, c);
    if constexpr (N > Bk) c = chain_add_gen<N - Bk, OFF + Bk>(x + Bk, gen, c);
    return c;
}

// x = x - (gen(0), gen(1), ...) - c over N limbs, the subtrahend produced
// eight limbs at a time just before its chain block, so that no more than
// eight of its limbs are live at once (any N: a length that is not 1, 2, 4
// or a multiple of 8 ends in blocks of 4, 2 and 1, as chain_sub_gen does).
template <int N, typename Gen>
__device__ __forceinline__ uint32_t chain_sub_from(uint64_t (&x)[N], Gen gen, uint32_t c) {
    constexpr int Bk = N < 8 ? N : 8;
    if constexpr (N % Bk != 0 || (N < 8 && N != 1 && N != 2 && N != 4)) {
        return chain_sub_gen<N>(&x[0], gen, c);
    } else {
#pragma unroll
        for (int b = 0; b < N / Bk; b++) {
            uint64_t y[Bk];
#pragma unroll
            for (int j = 0; j < Bk; j++) y[j] = gen(b * Bk + j);
            c = chain_sub<Bk>(*reinterpret_cast<uint64_t(*)[Bk]>(&x[b * Bk]), y, c);
        }
        return c;
    }
}

// The carry out alone (x and y unchanged): the same chain on copies.
template <typename T>
__device__ __forceinline__ uint32_t chain_add8_cout(const T (&x)[8], const T (&y)[8], uint32_t c) {
    T t[8];
#pragma unroll
    for (int e = 0; e < 8; e++) t[e] = x[e];
    return chain_add8(t, y, c);
}
template <typename T>
__device__ __forceinline__ uint32_t chain_sub8_bout(const T (&x)[8], const T (&y)[8], uint32_t c) {
    T t[8];
#pragma unroll
    for (int e = 0; e < 8; e++) t[e] = x[e];
    return chain_sub8(t, y, c);
}

}  // namespace bi
