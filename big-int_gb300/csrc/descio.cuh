// descio.cuh -- the elements of a bi_desc instance: 64-bit limbs or 32-bit
// words, read and written as 64-bit limbs by the batch and serving kernels.
#pragma once

#include "common.cuh"

namespace bi {

// A descriptor's elements: 64-bit limbs (width 0 or 64) or 32-bit words
// (width 32: m, mb and the offsets count words of the arenas).  The kernels
// work on 64-bit limbs either way: a word instance is read as the limbs of
// its zero-extended value and written back word by word.
__host__ __device__ inline bool desc_w32(const bi_desc& d) { return d.width == 32; }
__host__ __device__ inline uint32_t m64(const bi_desc& d) { return desc_w32(d) ? (d.m + 1) / 2 : d.m; }
__host__ __device__ inline uint32_t mb64(const bi_desc& d) { return desc_w32(d) ? (d.mb + 1) / 2 : d.mb; }
// 64-bit limb i of the n-element operand at element offset off of an arena
__device__ __forceinline__ uint64_t ld64(const uint64_t* arena, uint64_t off, uint32_t n, bool w32, uint32_t i) {
    if (!w32) return i < n ? arena[off + i] : 0;
    const uint32_t* p = reinterpret_cast<const uint32_t*>(arena) + off;
    uint64_t x = 2 * i < n ? p[2 * i] : 0u;
    if (2 * i + 1 < n) x |= (uint64_t)p[2 * i + 1] << 32;
    return x;
}
// limb i of an n-element result: the elements of it that lie below n
__device__ __forceinline__ void st64(uint64_t* arena, uint64_t off, uint32_t n, bool w32, uint32_t i, uint64_t v) {
    if (!w32) {
        if (i < n) arena[off + i] = v;
        return;
    }
    uint32_t* p = reinterpret_cast<uint32_t*>(arena) + off;
    if (2 * i < n) p[2 * i] = (uint32_t)v;
    if (2 * i + 1 < n) p[2 * i + 1] = (uint32_t)(v >> 32);
}

}  // namespace bi
