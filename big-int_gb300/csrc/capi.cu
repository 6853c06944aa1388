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

#include <atomic>
#include <mutex>
#include <vector>

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

// SM count of the current device, queried once per device.
int num_sms() {
    static std::atomic<int> cache[64];
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (dev >= 0 && dev < 64 && (sms = cache[dev].load(std::memory_order_relaxed)) != 0) return sms;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    if (dev >= 0 && dev < 64) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

// Raise a kernel's dynamic shared-memory limit to `smem` on the current
// device; remembered per (kernel, device), so a launch path calls the driver
// only the first time it needs a larger size.
cudaError_t smem_opt_in(const void* func, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    struct Entry {
        const void* func;
        int dev;
        size_t smem;
    };
    static std::mutex mu;
    static std::vector<Entry> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    for (Entry& x : done)
        if (x.func == func && x.dev == dev) {
            if (x.smem >= smem) return cudaSuccess;
            e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) x.smem = smem;
            return e;
        }
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) done.push_back({func, dev, smem});
    return e;
}

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

// Host-pointer entry points run the batch as a pipeline: the instances are
// cut into chunks of about PIPE_CHUNK_BYTES of the first operand; chunk c
// goes to stream c % PIPE_STREAMS, which copies its inputs in, runs the
// kernel and copies its outputs out, so the copies of one chunk overlap the
// kernels and copies of the others.  Device chunk buffers come from the
// stream-ordered allocator and are returned when the call ends.
constexpr size_t PIPE_CHUNK_BYTES = 32ull << 20;
constexpr int PIPE_STREAMS = 3;

struct HostIO {
    const void* in[2];        // host inputs (per-instance sizes in bytes below)
    size_t in_bytes[2];
    void* out[3];             // host outputs (two limb arrays and one byte array)
    size_t out_bytes[3];
};

template <typename Launch>
static bi_status host_pipelined(const HostIO& io, uint64_t n, Launch launch) {
    if (n == 0) return BI_OK;
    const size_t per = io.in_bytes[0] ? io.in_bytes[0] : 1;
    uint64_t chunk = PIPE_CHUNK_BYTES / per;
    if (chunk < 1) chunk = 1;
    if (chunk > n) chunk = n;
    const uint64_t nchunks = (n + chunk - 1) / chunk;
    const int ns = nchunks < (uint64_t)PIPE_STREAMS ? (int)nchunks : PIPE_STREAMS;

    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = 4ull << 30;   // keep chunk buffers cached between calls of this process
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaStream_t st[PIPE_STREAMS] = {};
    void* dbuf[PIPE_STREAMS][5] = {};
    bi_status rs = BI_OK;
    for (int k = 0; k < ns && rs == BI_OK; k++) {
        cudaError_t e = cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking);
        if (e != cudaSuccess) { st[k] = nullptr; rs = cuda_ok(e, "stream create"); break; }
        for (int j = 0; j < 2 && rs == BI_OK; j++)
            if (io.in_bytes[j]) rs = cuda_ok(cudaMallocAsync(&dbuf[k][j], io.in_bytes[j] * chunk, st[k]), "chunk alloc");
        for (int j = 0; j < 3 && rs == BI_OK; j++)
            if (io.out_bytes[j]) rs = cuda_ok(cudaMallocAsync(&dbuf[k][2 + j], io.out_bytes[j] * chunk, st[k]), "chunk alloc");
    }
    for (uint64_t c = 0; c < nchunks && rs == BI_OK; c++) {
        const int k = (int)(c % ns);
        const uint64_t i0 = c * chunk;
        const uint64_t cnt = n - i0 < chunk ? n - i0 : chunk;
        for (int j = 0; j < 2 && rs == BI_OK; j++)
            if (io.in_bytes[j])
                rs = cuda_ok(cudaMemcpyAsync(dbuf[k][j], (const char*)io.in[j] + i0 * io.in_bytes[j],
                                             cnt * io.in_bytes[j], cudaMemcpyHostToDevice, st[k]), "copy in");
        if (rs == BI_OK) rs = launch(dbuf[k][0], dbuf[k][1], dbuf[k][2], dbuf[k][3], (uint8_t*)dbuf[k][4], cnt, st[k]);
        for (int j = 0; j < 3 && rs == BI_OK; j++)
            if (io.out_bytes[j] && io.out[j])
                rs = cuda_ok(cudaMemcpyAsync((char*)io.out[j] + i0 * io.out_bytes[j], dbuf[k][2 + j],
                                             cnt * io.out_bytes[j], cudaMemcpyDeviceToHost, st[k]), "copy out");
    }
    for (int k = 0; k < ns; k++) {
        if (!st[k]) continue;
        for (int j = 0; j < 5; j++)
            if (dbuf[k][j]) cudaFreeAsync(dbuf[k][j], st[k]);
        cudaError_t e = cudaStreamSynchronize(st[k]);
        if (rs == BI_OK && e != cudaSuccess) rs = cuda_ok(e, "pipeline");
        cudaStreamDestroy(st[k]);
    }
    return rs;
}

// Device-accessible alias of a pinned (page-locked, registered) host
// buffer, or nullptr for pageable memory.
static void* pinned_alias(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
    return at.devicePointer;
}

// When every host buffer is pinned, the kernel reads and writes them in
// place over the CPU-GPU link (one pass, no staging copies): the link is the
// bound, and a bandwidth-bound kernel keeps it fuller than chunked copies.
template <typename Launch>
static bool run_in_place(const HostIO& io, uint64_t n, Launch launch, bi_status* rs) {
    void* d[5] = {};
    for (int j = 0; j < 2; j++)
        if (io.in_bytes[j] && !(d[j] = pinned_alias(io.in[j]))) return false;
    for (int j = 0; j < 3; j++)
        if (io.out_bytes[j] && io.out[j] && !(d[2 + j] = pinned_alias(io.out[j]))) return false;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    *rs = launch(d[0], d[1], d[2], d[3], (uint8_t*)d[4], n, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (*rs == BI_OK && e != cudaSuccess) *rs = cuda_ok(e, "in-place host launch");
    cudaStreamDestroy(st);
    return true;
}

// `link` runs the in-place pass on pinned buffers, `launch` the staged
// chunks in device memory.
template <typename T, typename Launch, typename Link>
static bi_status host_binary(const T* ha, const T* hb, T* hr, uint8_t* hsign, uint32_t m, uint64_t n,
                             size_t out_limbs_per_inst, Launch launch, Link link) {
    if (n == 0) return BI_OK;
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!ha || !hb || !hr) return set_error(BI_EINVAL, "NULL host buffer");
    HostIO io = {};
    io.in[0] = ha; io.in_bytes[0] = (size_t)m * sizeof(T);
    io.in[1] = hb; io.in_bytes[1] = (size_t)m * sizeof(T);
    io.out[0] = hr; io.out_bytes[0] = out_limbs_per_inst * sizeof(T);
    io.out[2] = hsign; io.out_bytes[2] = hsign ? 1 : 0;
    auto fn = [&](void* da, void* db, void* dr, void*, uint8_t* ds, uint64_t cnt, cudaStream_t s) {
        return launch((const T*)da, (const T*)db, (T*)dr, ds, cnt, s);
    };
    auto fn_link = [&](void* da, void* db, void* dr, void*, uint8_t* ds, uint64_t cnt, cudaStream_t s) {
        return link((const T*)da, (const T*)db, (T*)dr, ds, cnt, s);
    };
    bi_status rs;
    if (run_in_place(io, n, fn_link, &rs)) return rs;
    return host_pipelined(io, n, fn);
}

template <typename T, typename Launch>
static bi_status host_binary(const T* ha, const T* hb, T* hr, uint8_t* hsign, uint32_t m, uint64_t n,
                             size_t out_limbs_per_inst, Launch launch) {
    return host_binary<T>(ha, hb, hr, hsign, m, n, out_limbs_per_inst, launch, launch);
}

template <typename T>
static bi_status host_div(const T* hu, const T* hv, T* hq, T* hr, uint8_t* hstatus, uint32_t mu, uint32_t mv,
                          uint64_t n) {
    if (n == 0) return BI_OK;
    if (mu == 0 || mv == 0 || mv > mu) return set_error(BI_EINVAL, "need 1 <= mv <= mu");
    if (!hu || !hv || !hq || !hr) return set_error(BI_EINVAL, "NULL host buffer");
    uint8_t* stat = hstatus;
    uint8_t* own = nullptr;
    if (!stat) {
        own = (uint8_t*)malloc(n);
        if (!own) return set_error(BI_ENOMEM, "host status buffer");
        stat = own;
    }
    HostIO io = {};
    io.in[0] = hu; io.in_bytes[0] = (size_t)mu * sizeof(T);
    io.in[1] = hv; io.in_bytes[1] = (size_t)mv * sizeof(T);
    io.out[0] = hq; io.out_bytes[0] = (size_t)mu * sizeof(T);
    io.out[1] = hr; io.out_bytes[1] = (size_t)mv * sizeof(T);
    io.out[2] = stat; io.out_bytes[2] = 1;
    auto fn = [&](void* du, void* dv, void* dq, void* dr, uint8_t* ds, uint64_t cnt, cudaStream_t s) {
        if constexpr (sizeof(T) == 8)
            return bi_div_u64((const T*)du, (const T*)dv, (T*)dq, (T*)dr, ds, mu, mv, cnt, s);
        else
            return bi_div_u32((const T*)du, (const T*)dv, (T*)dq, (T*)dr, ds, mu, mv, cnt, s);
    };
    bi_status rs;
    if (!run_in_place(io, n, fn, &rs)) rs = host_pipelined(io, n, fn);
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

namespace bi {

template <typename T>
static bi_status test_div(const T* u, const T* v, T* w, uint32_t m,
                          bi_status (*host_div)(const T*, const T*, T*, T*, uint8_t*, uint32_t, uint32_t, uint64_t)) {
    if (m == 0) return set_error(BI_EINVAL, "m must be >= 1");
    if (!u || !v || !w) return set_error(BI_EINVAL, "NULL host buffer");
    T* rem = (T*)malloc((size_t)m * sizeof(T));
    if (!rem) return set_error(BI_ENOMEM, "test_div: remainder buffer");
    const bi_status st = host_div(u, v, w, rem, nullptr, m, m, 1);
    free(rem);
    return st;
}
static uint64_t read_word(const unsigned char* p, size_t size) {
    switch (size) {
        case 1: return *p;
        case 2: { uint16_t x; memcpy(&x, p, 2); return x; }
        case 4: { uint32_t x; memcpy(&x, p, 4); return x; }
        default: { uint64_t x; memcpy(&x, p, 8); return x; }
    }
}
static void write_word(unsigned char* p, size_t size, uint64_t v) {
    switch (size) {
        case 1: *p = (unsigned char)v; break;
        case 2: { const uint16_t x = (uint16_t)v; memcpy(p, &x, 2); break; }
        case 4: { const uint32_t x = (uint32_t)v; memcpy(p, &x, 4); break; }
        default: memcpy(p, &v, 8);
    }
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
    case BI_EBUSY: return "BI_EBUSY";
    default: return "BI_UNKNOWN";
    }
}

const char* bi_last_error(void) { return g_err; }

// ---- the Futhark library's 1-D entries: one instance through the host twins
bi_status bi_test_add_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m) {
    return bi_host_add_u64(u, v, w, m, 1);
}
bi_status bi_test_add_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m) {
    return bi_host_add_u32(u, v, w, m, 1);
}
bi_status bi_test_sub_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m) {
    uint8_t sign;
    return bi_host_sub_u64(u, v, w, &sign, m, 1);
}
bi_status bi_test_sub_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m) {
    uint8_t sign;
    return bi_host_sub_u32(u, v, w, &sign, m, 1);
}
bi_status bi_test_mul_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m) {
    return bi_host_mul_u64(u, v, w, m, 1);
}
bi_status bi_test_mul_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m) {
    return bi_host_mul_u32(u, v, w, m, 1);
}
bi_status bi_test_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m) {
    return test_div<uint64_t>(u, v, w, m, bi_host_div_u64);
}
bi_status bi_test_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m) {
    return test_div<uint32_t>(u, v, w, m, bi_host_div_u32);
}

// ---- GMP word arrays (order -1, native byte order) <-> 64-bit limbs
bi_status bi_limbs_from_words(const void* words, size_t count, size_t size, uint64_t* limbs, uint32_t m) {
    if (!(size == 1 || size == 2 || size == 4 || size == 8)) return set_error(BI_EINVAL, "word size must be 1, 2, 4 or 8");
    if (!limbs || (count && !words)) return set_error(BI_EINVAL, "NULL buffer");
    const size_t per = 8 / size;   // words per limb
    const unsigned char* w = (const unsigned char*)words;
    for (uint32_t j = 0; j < m; j++) limbs[j] = 0;
    for (size_t k = 0; k < count; k++) {
        const uint64_t x = read_word(w + k * size, size);
        const size_t j = k / per;
        if (j >= m) {
            if (x != 0) return set_error(BI_EINVAL, "value needs more than m=%u limbs", m);
            continue;
        }
        limbs[j] |= x << (8 * size * (k % per));
    }
    return BI_OK;
}

bi_status bi_limbs_to_words(const uint64_t* limbs, uint32_t m, size_t size, void* words, size_t* count) {
    if (!(size == 1 || size == 2 || size == 4 || size == 8)) return set_error(BI_EINVAL, "word size must be 1, 2, 4 or 8");
    if (!limbs || !words || !count) return set_error(BI_EINVAL, "NULL buffer");
    const size_t per = 8 / size;
    const uint64_t mask = size == 8 ? ~0ull : ((1ull << (8 * size)) - 1);
    unsigned char* w = (unsigned char*)words;
    size_t used = 0;
    for (size_t k = 0; k < (size_t)m * per; k++) {
        const uint64_t x = (limbs[k / per] >> (8 * size * (k % per))) & mask;
        write_word(w + k * size, size, x);
        if (x) used = k + 1;
    }
    *count = used;
    return BI_OK;
}

int bi_version(void) { return 100; }

bi_status bi_host_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_add_u64(da, db, dr, m, cnt, cs);
        },
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return add_link_u64(da, db, dr, m, cnt, cs);
        });
}
bi_status bi_host_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_add_u32(da, db, dr, m, cnt, cs);
        },
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return add_link_u32(da, db, dr, m, cnt, cs);
        });
}
bi_status bi_host_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m,
                          uint64_t n) {
    return host_binary<uint64_t>(a, b, r, sign, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t* ds, uint64_t cnt, cudaStream_t cs) {
            return bi_sub_u64(da, db, dr, ds, m, cnt, cs);
        },
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t* ds, uint64_t cnt, cudaStream_t cs) {
            return sub_link_u64(da, db, dr, ds, m, cnt, cs);
        });
}
bi_status bi_host_sub_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* sign, uint32_t m,
                          uint64_t n) {
    return host_binary<uint32_t>(a, b, r, sign, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t* ds, uint64_t cnt, cudaStream_t cs) {
            return bi_sub_u32(da, db, dr, ds, m, cnt, cs);
        },
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t* ds, uint64_t cnt, cudaStream_t cs) {
            return sub_link_u32(da, db, dr, ds, m, cnt, cs);
        });
}

bi_status bi_host_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_mul_u64(da, db, dr, m, cnt, cs);
        });
}
bi_status bi_host_mul_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_mul_u32(da, db, dr, m, cnt, cs);
        });
}
bi_status bi_host_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint64_t>(a, b, r, nullptr, m, n, 2 * (size_t)m,
        [&](const uint64_t* da, const uint64_t* db, uint64_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_mulfull_u64(da, db, dr, m, cnt, cs);
        });
}
bi_status bi_host_mulfull_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t m, uint64_t n) {
    return host_binary<uint32_t>(a, b, r, nullptr, m, n, 2 * (size_t)m,
        [&](const uint32_t* da, const uint32_t* db, uint32_t* dr, uint8_t*, uint64_t cnt, cudaStream_t cs) {
            return bi_mulfull_u32(da, db, dr, m, cnt, cs);
        });
}

}  // extern "C"
