// probe.cu -- integer-pipe throughput probe (the multiply roofline's denominator).
//
// Big-integer multiplication runs on the integer multiply-add pipe, for which
// no vendor peak is quoted, so the peak is measured: each probe kernel keeps
// eight independent accumulator chains per thread busy with one instruction
// form and reports how many 32x32-bit word products per second the whole GPU
// sustains in that form.
//   0  mad.lo.u32                       (1 instruction  = 1/2 word product)
//   1  mad.hi.u32                       (1 instruction  = 1/2 word product)
//   2  mad.wide.u32 with 64-bit addend  (1 instruction  = 1 word product)
//   3  row of mad.lo.cc / madc.hi.cc carry chains, 8 products + 2 addc
//   4  64x64 products via mul.lo.u64 + mul.hi.u64 (= 4 word products)
//   5  column accumulation: one new row multiplicand, 8 mad.wide.u32 into
//      eight 64-bit column sums (1 instruction = 1 word product)
#include "common.cuh"

namespace bi {

template <int MODE>
__global__ void __launch_bounds__(256) intpipe_kernel(uint32_t* sink, uint32_t iters, uint32_t seed) {
    uint32_t a = threadIdx.x * 2654435761u + seed;
    uint32_t b[8];
#pragma unroll
    for (int k = 0; k < 8; k++) b[k] = blockIdx.x * 97u + k * 31u + 1u;
    uint32_t acc = 0;
    if (MODE == 0 || MODE == 1) {
        uint32_t x[8];
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = a ^ k;
        // x[k] is both a multiplicand and the addend, so nothing is loop-invariant
        for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                if (MODE == 0) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[k]) : "r"(b[k]), "r"(a));
                else           asm volatile("mad.hi.u32 %0, %0, %1, %0;" : "+r"(x[k]) : "r"(b[k]));
            }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) acc ^= x[k];
    } else if (MODE == 2) {
        uint64_t y[8];
#pragma unroll
        for (int k = 0; k < 8; k++) y[k] = a + k;
        // the low half of each accumulator is the next multiplicand
        for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t lo = (uint32_t)y[k];
                asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(y[k]) : "r"(lo), "r"(b[k]));
            }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) acc ^= (uint32_t)y[k] ^ (uint32_t)(y[k] >> 32);
    } else if (MODE == 3) {
        uint32_t r[10];
#pragma unroll
        for (int k = 0; k < 10; k++) r[k] = a + k;
        for (uint32_t i = 0; i < iters; i++) {
            asm volatile(
                "mad.lo.cc.u32  %0, %10, %11, %0;\n\t"
                "madc.lo.cc.u32 %1, %10, %12, %1;\n\t"
                "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
                "madc.lo.cc.u32 %3, %10, %14, %3;\n\t"
                "madc.lo.cc.u32 %4, %10, %15, %4;\n\t"
                "madc.lo.cc.u32 %5, %10, %16, %5;\n\t"
                "madc.lo.cc.u32 %6, %10, %17, %6;\n\t"
                "madc.lo.cc.u32 %7, %10, %18, %7;\n\t"
                "addc.u32       %8, %8, 0;\n\t"
                "mad.hi.cc.u32  %1, %10, %11, %1;\n\t"
                "madc.hi.cc.u32 %2, %10, %12, %2;\n\t"
                "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
                "madc.hi.cc.u32 %4, %10, %14, %4;\n\t"
                "madc.hi.cc.u32 %5, %10, %15, %5;\n\t"
                "madc.hi.cc.u32 %6, %10, %16, %6;\n\t"
                "madc.hi.cc.u32 %7, %10, %17, %7;\n\t"
                "madc.hi.cc.u32 %8, %10, %18, %8;\n\t"
                "addc.u32       %9, %9, 0;"
                : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                  "+r"(r[7]), "+r"(r[8]), "+r"(r[9])
                : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]),
                  "r"(b[7]));
            a += r[0];
        }
#pragma unroll
        for (int k = 0; k < 10; k++) acc ^= r[k];
    } else if (MODE == 5) {
        uint64_t y[8];
#pragma unroll
        for (int k = 0; k < 8; k++) y[k] = a + k;
        uint32_t ai = a;
        for (uint32_t i = 0; i < iters; i++) {
            ai += 0x9E3779B9u;   // a new row multiplicand each iteration (IADD, not the multiply pipe)
#pragma unroll
            for (int k = 0; k < 8; k++)
                asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(y[k]) : "r"(ai), "r"(b[k]));
        }
#pragma unroll
        for (int k = 0; k < 8; k++) acc ^= (uint32_t)y[k] ^ (uint32_t)(y[k] >> 32);
    } else {
        uint64_t lo[4], hi[4];
        uint64_t A = ((uint64_t)a << 32) | (a * 3u);
#pragma unroll
        for (int k = 0; k < 4; k++) { lo[k] = A + k; hi[k] = 0; }
        for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint64_t B = ((uint64_t)b[k] << 32) | b[k + 4];
                uint64_t l, h;
                asm volatile("mul.lo.u64 %0, %1, %2;" : "=l"(l) : "l"(lo[k]), "l"(B));
                asm volatile("mul.hi.u64 %0, %1, %2;" : "=l"(h) : "l"(lo[k]), "l"(B));
                lo[k] = l ^ i;
                hi[k] += h;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) acc ^= (uint32_t)lo[k] ^ (uint32_t)hi[k];
    }
    if (acc == 0x12345678u) sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

template <int MODE>
static bi_status time_mode(uint32_t* sink, int blocks, uint32_t iters, cudaStream_t st, float* ms) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    intpipe_kernel<MODE><<<blocks, 256, 0, st>>>(sink, 16, 1);   // warm-up
    cudaEventRecord(e0, st);
    intpipe_kernel<MODE><<<blocks, 256, 0, st>>>(sink, iters, 1);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return set_error(BI_ECUDA, "intpipe probe: %s", cudaGetErrorString(e));
    return check_launch("intpipe probe");
}

}  // namespace bi

using namespace bi;

// rates[k], k = 0..5: word products per second for probe form k (see the top of this file).
extern "C" bi_status bi_probe_intpipe(double* rates, bi_stream s) {
    if (!rates) return set_error(BI_EINVAL, "rates must point to 6 doubles");
    cudaStream_t st = (cudaStream_t)s;
    const int blocks = num_sms() * 8;
    uint32_t* sink = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&sink, (size_t)blocks * 256 * 4, st);
    if (e != cudaSuccess) return set_error(BI_ENOMEM, "probe sink: %s", cudaGetErrorString(e));
    const uint32_t iters = 4096;
    const double threads = (double)blocks * 256;
    float ms = 0;
    bi_status r = BI_OK;
    // word products per thread per iteration of each form
    const double wp[6] = {8 * 0.5, 8 * 0.5, 8.0, 8.0, 4 * 4.0, 8.0};
    for (int mode = 0; mode < 6 && r == BI_OK; mode++) {
        switch (mode) {
        case 0: r = time_mode<0>(sink, blocks, iters, st, &ms); break;
        case 1: r = time_mode<1>(sink, blocks, iters, st, &ms); break;
        case 2: r = time_mode<2>(sink, blocks, iters, st, &ms); break;
        case 3: r = time_mode<3>(sink, blocks, iters, st, &ms); break;
        case 4: r = time_mode<4>(sink, blocks, iters, st, &ms); break;
        default: r = time_mode<5>(sink, blocks, iters, st, &ms); break;
        }
        rates[mode] = (r == BI_OK && ms > 0) ? threads * iters * wp[mode] / (ms * 1e-3) : 0.0;
    }
    cudaFreeAsync(sink, st);
    cudaStreamSynchronize(st);
    return r;
}
