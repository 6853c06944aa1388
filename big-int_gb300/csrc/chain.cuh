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
