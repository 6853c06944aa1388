// util.cu -- device-side synthetic input generation.
//
// Fills a buffer with the splitmix64 stream used by the benchmark and test
// workloads: element i (0-based, after `offset`) is mix(seed + (offset+i+1) *
// 0x9E3779B97F4A7C15).  Generating inputs on the device keeps multi-GiB
// workloads cheap to set up; the host generator in workloads.py produces the
// same values.
#include "common.cuh"

namespace bi {

__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t idx) {
    uint64_t z = seed + idx * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void fill_splitmix64_kernel(uint64_t* dst, uint64_t count, uint64_t seed, uint64_t offset) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
        dst[i] = splitmix64_at(seed, offset + i + 1);
}

}  // namespace bi

using namespace bi;

extern "C" bi_status bi_fill_splitmix64(uint64_t* dst, uint64_t count, uint64_t seed, uint64_t offset,
                                        bi_stream s) {
    if (count == 0) return BI_OK;
    if (!dst || (uintptr_t)dst % 8) return set_error(BI_EINVAL, "dst must be a non-NULL 8-byte aligned pointer");
    const uint64_t blocks = (count + 255) / 256;
    const unsigned grid = (unsigned)(blocks < (uint64_t)num_sms() * 16 ? blocks : (uint64_t)num_sms() * 16);
    fill_splitmix64_kernel<<<grid, 256, 0, (cudaStream_t)s>>>(dst, count, seed, offset);
    return check_launch("fill kernel");
}
