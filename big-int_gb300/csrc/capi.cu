// capi.cu -- status plumbing and the host-pointer entry points of the C ABI.
//
// The host twins mirror the reference's host wrappers gpuAdd/gpuMultiply
// (cuda/main.cu:108-222, 280-419): allocate device buffers, copy the inputs
// in, launch, copy the result out and free.  Unlike the reference they
// report every failure as a status code instead of printing and carrying on.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.cuh"

namespace bi {

static thread_local char g_err[512];

bi_status set_error(bi_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return st;
}

bi_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(BI_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return BI_OK;
}

int num_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return sms;
}

// RAII device buffer used only by the host-pointer entry points.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    bi_status alloc(size_t nbytes) {
        bytes = nbytes;
        if (nbytes == 0) return BI_OK;
        cudaError_t e = cudaMalloc(&p, nbytes);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return set_error(e == cudaErrorMemoryAllocation ? BI_ENOMEM : BI_ECUDA,
                             "cudaMalloc(%zu): %s", nbytes, cudaGetErrorString(e));
        }
        return BI_OK;
    }
};

static bi_status cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return BI_OK;
    cudaGetLastError();
    return set_error(BI_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define BI_TRY(x)                      \
    do {                               \
        bi_status _s = (x);            \
        if (_s != BI_OK) return _s;    \
    } while (0)

template <typename T, typename Launch>
static bi_status host_binary(const T* ha, const T* hb, T* hr, uint8_t* hsign, uint32_t m, uint64_t n,
                             size_t out_limbs_per_inst, Launch launch) {
    if (n == 0) return BI_OK;
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!ha || !hb || !hr) return set_error(BI_EINVAL, "NULL host buffer");
    const size_t in_bytes = (size_t)n * m * sizeof(T);
    const size_t out_bytes = (size_t)n * out_limbs_per_inst * sizeof(T);
    DevBuf da, db, dr, ds;
    BI_TRY(da.alloc(in_bytes));
    BI_TRY(db.alloc(in_bytes));
    BI_TRY(dr.alloc(out_bytes));
    if (hsign) BI_TRY(ds.alloc(n));
    BI_TRY(cuda_ok(cudaMemcpy(da.p, ha, in_bytes, cudaMemcpyHostToDevice), "copy a"));
    BI_TRY(cuda_ok(cudaMemcpy(db.p, hb, in_bytes, cudaMemcpyHostToDevice), "copy b"));
    BI_TRY(launch((const T*)da.p, (const T*)db.p, (T*)dr.p, (uint8_t*)ds.p));
    BI_TRY(cuda_ok(cudaMemcpy(hr, dr.p, out_bytes, cudaMemcpyDeviceToHost), "copy r"));
    if (hsign) BI_TRY(cuda_ok(cudaMemcpy(hsign, ds.p, n, cudaMemcpyDeviceToHost), "copy sign"));
    return BI_OK;
}

template <typename T>
static bi_status host_div(const T* hu, const T* hv, T* hq, T* hr, uint8_t* hstatus, uint32_t mu, uint32_t mv,
                          uint64_t n) {
    if (n == 0) return BI_OK;
    if (mu == 0 || mv == 0 || mv > mu) return set_error(BI_EINVAL, "need 1 <= mv <= mu");
    if (!hu || !hv || !hq || !hr) return set_error(BI_EINVAL, "NULL host buffer");
    DevBuf du, dv, dq, dr, ds;
    BI_TRY(du.alloc((size_t)n * mu * sizeof(T)));
    BI_TRY(dv.alloc((size_t)n * mv * sizeof(T)));
    BI_TRY(dq.alloc((size_t)n * mu * sizeof(T)));
    BI_TRY(dr.alloc((size_t)n * mv * sizeof(T)));
    BI_TRY(ds.alloc(n));
    BI_TRY(cuda_ok(cudaMemcpy(du.p, hu, du.bytes, cudaMemcpyHostToDevice), "copy u"));
    BI_TRY(cuda_ok(cudaMemcpy(dv.p, hv, dv.bytes, cudaMemcpyHostToDevice), "copy v"));
    bi_status st;
    if constexpr (sizeof(T) == 8)
        st = bi_div_u64((const T*)du.p, (const T*)dv.p, (T*)dq.p, (T*)dr.p, (uint8_t*)ds.p, mu, mv, n, nullptr);
    else
        st = bi_div_u32((const T*)du.p, (const T*)dv.p, (T*)dq.p, (T*)dr.p, (uint8_t*)ds.p, mu, mv, n, nullptr);
    BI_TRY(st);
    BI_TRY(cuda_ok(cudaMemcpy(hq, dq.p, dq.bytes, cudaMemcpyDeviceToHost), "copy q"));
    BI_TRY(cuda_ok(cudaMemcpy(hr, dr.p, dr.bytes, cudaMemcpyDeviceToHost), "copy r"));
    uint8_t* stat = hstatus;
    uint8_t* own = nullptr;
    if (!stat) {
        own = (uint8_t*)malloc(n);
        if (!own) return set_error(BI_ENOMEM, "host status buffer");
        stat = own;
    }
    bi_status rs = cuda_ok(cudaMemcpy(stat, ds.p, n, cudaMemcpyDeviceToHost), "copy status");
    if (rs == BI_OK) {
        for (uint64_t i = 0; i < n; i++) {
            if (stat[i] == 1) { rs = set_error(BI_EDIV0, "instance %llu has a zero divisor", (unsigned long long)i); break; }
            if (stat[i] == 2) { rs = set_error(BI_ECUDA, "instance %llu exceeded the correction bound", (unsigned long long)i); break; }
        }
    }
    free(own);
    return rs;
}

}  // namespace bi

using namespace bi;

extern "C" {

bi_status bi_host_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r, uint8_t* status,
                          uint32_t mu, uint32_t mv, uint64_t n) {
    return host_div<uint64_t>(u, v, q, r, status, mu, mv, n);
}
bi_status bi_host_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r, uint8_t* status,
                          uint32_t mu, uint32_t mv, uint64_t n) {
    return host_div<uint32_t>(u, v, q, r, status, mu, mv, n);
}

const char* bi_status_string(bi_status s) {
    switch (s) {
    case BI_OK: return "BI_OK";
    case BI_EINVAL: return "BI_EINVAL";
    case BI_EDIV0: return "BI_EDIV0";
    case BI_ENOMEM: return "BI_ENOMEM";
    case BI_ETIMEDOUT: return "BI_ETIMEDOUT";
    case BI_ECUDA: return "BI_ECUDA";
    case BI_EUNSUPPORTED: return "BI_EUNSUPPORTED";
    default: return "BI_UNKNOWN";
    }
}

const char* bi_last_error(void) { return g_err; }

int bi_version(void) { return 100; }

bi_status bi_host_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*) {
            return bi_add_u64(da, db, dr, m, n, nullptr);
        });
}
bi_status bi_host_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*) {
            return bi_add_u32(da, db, dr, m, n, nullptr);
        });
}
bi_status bi_host_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m,
                          uint64_t n) {
    return host_binary<uint64_t>(a, b, r, sign, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t* ds) {
            return bi_sub_u64(da, db, dr, ds, m, n, nullptr);
        });
}
bi_status bi_host_sub_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* sign, uint32_t m,
                          uint64_t n) {
    return host_binary<uint32_t>(a, b, r, sign, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t* ds) {
            return bi_sub_u32(da, db, dr, ds, m, n, nullptr);
        });
}

bi_status bi_host_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*) {
            return bi_mul_u64(da, db, dr, m, n, nullptr);
        });
}
bi_status bi_host_mul_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*) {
            return bi_mul_u32(da, db, dr, m, n, nullptr);
        });
}
bi_status bi_host_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, 2 * (size_t)m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*) {
            return bi_mulfull_u64(da, db, dr, m, n, nullptr);
        });
}
bi_status bi_host_mulfull_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, 2 * (size_t)m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*) {
            return bi_mulfull_u32(da, db, dr, m, n, nullptr);
        });
}

}  // extern "C"
