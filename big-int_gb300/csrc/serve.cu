// serve.cu -- the serving loop: a device-resident request loop with
// continuous batching.  No counterpart in the reference, whose benchmarks run
// fixed batches from a host loop (cuda/main.cu:476-515).
//
// Requests are bi_desc records over one device operand arena.  The host side
// (a bi_server) admits a request when a ring slot and room for its results in
// the output arena (the HBM budget) are free, writes it into a ring of 64-byte
// slots in pinned host memory mapped into the GPU, and publishes the new tail.
// On the device a persistent kernel keeps every CTA polling that tail: a CTA
// claims the next request with a compare-and-swap on a device counter, checks
// that the slot holds that request's number, runs it with the cores the batch
// kernels use (warp add/sub, CTA multiply, CTA division) and appends a record
// to a completion queue in mapped host memory.  A request that arrives while
// others run is claimed by whichever CTA frees up first, so requests of every
// size and operation overlap on the device with no batch boundary, and the
// host never launches a kernel per request.
//
// Every device wait is bounded by the global timer.  The loop ends as a whole:
// when no CTA has claimed a request for idle_us (or the host's stop flag is
// set), the first CTA to notice marks the launch closing and every CTA leaves
// after its current request, so a launch never lingers with a few CTAs.  The
// last CTA to leave records the launch's epoch in mapped memory, and the host
// relaunches the kernel when it holds unclaimed requests and the loop has
// ended.  The wait for a claimed slot's contents gives up after a second and
// completes the request with status 0xFF.
//
// The driver functions at the end replay a timed arrival stream open-loop,
// through the server and through one library launch per request, and report
// latency percentiles from arrival to the host seeing the completion.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "descio.cuh"
#include "divcore.cuh"
#include "divsmall.cuh"
#include "mulcore.cuh"
#include "warpops.cuh"

namespace bi {

constexpr int SERVE_CTA = 256;
constexpr uint32_t SERVE_MAX_LIMBS = 2048;       // largest operand (64-bit limbs)
constexpr uint64_t SERVE_WAIT_NS = 1000000000;   // give up on a slot after 1 s
constexpr uint64_t SERVE_LOST = 0xFF;            // status of a request whose slot never filled
// divisors up to this many limbs divide on warp 0 (long division), larger ones
// on the whole CTA (shifted inverse).  One division alone: 160/80 limbs 39 us
// on a warp and 41 on a CTA, 192/96 47 and 41, 256/128 60 and 49.  On the
// serving workload 64 gave p90 40-45 us against 36-38 at 128 (a CTA-wide
// division slows the SM's other serving CTA), and 96 against 128 takes the
// p99 of the 65..256-limb divisions from 61-65 to 55-62 us with the overall
// p50 / p90 / p99 unchanged within 0.6 us (10k, 100k and 1M requests/s)
constexpr uint32_t SERVE_DIV_WARP_MAX_MV = 96;
// divisors up to this many limbs divide on thread 0: one division alone takes
// 3.9 us on a thread and 4.3 on a warp at 8/4 limbs, 5.9 and 5.3 at 16/8,
// 13.7 and 7.9 at 32/16 (GB300)
constexpr uint32_t SERVE_DIV_THREAD_MAX_MV = 8;

struct alignas(64) ServeSlot {   // one request in the ring (mapped host memory)
    bi_desc d;                   // written first
    uint64_t seq;                // request number held, written last (release)
};
static_assert(sizeof(ServeSlot) == 64, "slot is one 64-byte line");

struct alignas(32) ServeDone {   // one completion-queue entry (mapped host memory)
    uint64_t tag;                // queue position + 1, written last (release)
    uint64_t seq;                // request number
    uint64_t flag;               // sub: sign; div: status; SERVE_LOST
    uint64_t pad;
};

struct ServeCtl {                      // mapped host memory
    alignas(128) uint64_t tail;        // requests published (host)
    alignas(128) uint64_t stop;        // nonzero: idle CTAs leave at once (host)
    alignas(128) uint64_t exited;      // epoch of the last launch whose CTAs all left (device)
};

struct ServeDev {                      // device memory
    unsigned long long head;           // requests claimed
    unsigned long long cq_pos;         // completion-queue positions handed out
    unsigned long long tail_seen;      // the host tail as last read by some CTA
    unsigned long long poll_ns;        // when some CTA last read the host tail
    unsigned long long last_work;      // when some CTA last claimed a request (or started)
    unsigned long long closing;        // epoch of a launch whose CTAs are to leave
    unsigned int left;                 // CTAs of the running launch that have left
    unsigned int stop_seen;            // the host stop flag as last read
};

// Idle CTAs read the host-written tail and stop flag at most once per
// SERVE_POLL_NS between them (one CTA wins a compare-and-swap on poll_ns and
// refreshes tail_seen and stop_seen); the others read the copies in device
// memory, so the line the host writes on every publish is not read by every
// CTA.
constexpr uint64_t SERVE_POLL_NS = 256;

struct ServeArgs {
    const ServeSlot* slots;
    ServeDone* cq;
    ServeCtl* ctl;
    ServeDev* dev;
    const uint64_t* in;
    uint64_t* out;
    uint64_t mask;       // ring slots - 1
    uint64_t epoch;
    uint64_t idle_ns;
};

__device__ __forceinline__ uint64_t ld_acquire_sys(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed_sys(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_sys(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys(uint64_t* p, uint64_t v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

enum : int { CLAIM_OK = 0, CLAIM_EXIT = 1, CLAIM_LOST = 2 };

// Thread 0 of a CTA: claim the next published request.  Returns CLAIM_EXIT
// once the launch is closing -- no CTA claimed a request for idle_ns, or
// stop is set and nothing is waiting -- and CLAIM_LOST if the claimed slot
// did not show the request within SERVE_WAIT_NS.
__device__ int serve_claim(const ServeArgs& A, uint64_t& seq, bi_desc& d) {
    volatile unsigned long long* head = &A.dev->head;
    volatile unsigned long long* seen = &A.dev->tail_seen;
    volatile unsigned long long* polled = &A.dev->poll_ns;
    volatile unsigned long long* last_work = &A.dev->last_work;
    volatile unsigned long long* closing = &A.dev->closing;
    uint32_t nap = 32;
    uint64_t h;
    for (;;) {
        if (*closing == A.epoch) return CLAIM_EXIT;
        h = *head;
        uint64_t t = *seen;
        if (h >= t) {
            const uint64_t now = global_ns(), last = *polled;
            if (now - last >= SERVE_POLL_NS && atomicCAS(&A.dev->poll_ns, last, now) == last) {
                const uint64_t ht = ld_acquire_sys(&A.ctl->tail);
                if (ht > t) {
                    atomicMax(&A.dev->tail_seen, ht);
                    t = ht;
                }
                if (ld_relaxed_sys(&A.ctl->stop)) atomicExch(&A.dev->stop_seen, 1u);
            }
        }
        if (h < t) {
            if (atomicCAS(&A.dev->head, h, h + 1) == h) {
                atomicMax(&A.dev->last_work, global_ns());
                break;
            }
            nap = 32;
            continue;
        }
        if (*(volatile unsigned int*)&A.dev->stop_seen || global_ns() - *last_work > A.idle_ns) {
            // close only if the host has published nothing beyond what was claimed
            const uint64_t ht = ld_acquire_sys(&A.ctl->tail);
            if (ht > h) {
                atomicMax(&A.dev->tail_seen, ht);
                continue;
            }
            atomicExch(&A.dev->closing, A.epoch);   // every CTA of this launch leaves
            return CLAIM_EXIT;
        }
        __nanosleep(nap);
        if (nap < 1024) nap *= 2;
    }
    seq = h;
    const ServeSlot* s = A.slots + (h & A.mask);
    const uint64_t t0 = global_ns();
    while (ld_acquire_sys(&s->seq) != h) {
        if (global_ns() - t0 > SERVE_WAIT_NS) return CLAIM_LOST;
        __nanosleep(64);
    }
    const uint64_t* w = reinterpret_cast<const uint64_t*>(&s->d);
    uint64_t* o = reinterpret_cast<uint64_t*>(&d);
#pragma unroll
    for (int i = 0; i < 7; i++) o[i] = ld_relaxed_sys(w + i);
    return CLAIM_OK;
}

// Thread 0: append the completion record (after the CTA's result stores).
__device__ void serve_complete(const ServeArgs& A, uint64_t seq, uint64_t flag) {
    __threadfence_system();
    const uint64_t pos = atomicAdd(&A.dev->cq_pos, 1ull);
    ServeDone* e = A.cq + (pos & A.mask);
    st_relaxed_sys(&e->seq, seq);
    st_relaxed_sys(&e->flag, flag);
    st_release_sys(&e->tag, pos + 1);
}

__global__ void __launch_bounds__(SERVE_CTA, 2) serve_kernel(const ServeArgs A) {
    extern __shared__ __align__(16) uint64_t smem[];
    __shared__ bi_desc s_d;
    __shared__ uint64_t s_seq;
    __shared__ int s_cmd;
    __shared__ uint32_t s_flag;
    __shared__ uint8_t s_sign;
    if (threadIdx.x == 0) atomicMax(&A.dev->last_work, global_ns());   // a launch starts busy
    for (;;) {
        if (threadIdx.x == 0) {
            s_flag = 0;
            s_cmd = serve_claim(A, s_seq, s_d);
        }
        __syncthreads();
        const int cmd = s_cmd;
        if (cmd == CLAIM_EXIT) break;
        if (cmd == CLAIM_OK) {
            const bi_desc d = s_d;
            const bool w32 = desc_w32(d);
            const uint32_t M = m64(d), MB = mb64(d);   // sizes in 64-bit limbs
            if (d.op == BI_OP_ADD || d.op == BI_OP_SUB) {
                if (threadIdx.x < 32) {
                    const bool sub = d.op == BI_OP_SUB;
                    if (w32 && ((d.a | d.b | d.r | d.m) & 1ull) != 0) {   // words that do not pair into limbs
                        const uint32_t* in32 = reinterpret_cast<const uint32_t*>(A.in);
                        warp_addsub<1, 4, uint32_t>(in32 + d.a, in32 + d.b, reinterpret_cast<uint32_t*>(A.out) + d.r,
                                                    &s_sign, d.m, sub);
                    } else {
                        const uint64_t a = w32 ? d.a / 2 : d.a, b = w32 ? d.b / 2 : d.b, r = w32 ? d.r / 2 : d.r;
                        // 16-byte accesses need even limb offsets (the arenas are 16-byte aligned)
                        if (((a | b | r) & 1ull) == 0)
                            warp_addsub<2, 4>(A.in + a, A.in + b, A.out + r, &s_sign, M, sub);
                        else
                            warp_addsub<1, 4>(A.in + a, A.in + b, A.out + r, &s_sign, M, sub);
                    }
                    if (threadIdx.x == 0 && sub) s_flag = s_sign;
                }
            } else if (d.op == BI_OP_MUL || d.op == BI_OP_MULFULL) {
                const bool full = d.op == BI_OP_MULFULL;
                const MulGeom g = mul_geometry_single_sliced(M, full, SERVE_CTA);
                uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + (size_t)g.ipc * g.IS);
                const FastDiv lpdiv(g.Lp);
                const uint32_t outn = full ? 2 * d.m : d.m;   // result elements
                auto load = [&](uint32_t, uint32_t x, uint64_t& va, uint64_t& vb) {
                    va = ld64(A.in, d.a, d.m, w32, x);
                    vb = ld64(A.in, d.b, d.m, w32, x);
                };
                auto store = [&](uint32_t, uint32_t x, uint64_t v) { st64(A.out, d.r, outn, w32, x, v); };
                mul_cta<MUL_C>(g, smem, scratch, lpdiv, load, store);
            } else {   // BI_OP_DIV (the host admits nothing else)
                auto ld_u = [&](uint32_t i) { return ld64(A.in, d.a, d.m, w32, i); };
                auto ld_v = [&](uint32_t i) { return ld64(A.in, d.b, d.mb, w32, i); };
                auto st_q = [&](uint32_t i, uint64_t x) { st64(A.out, d.r, d.m, w32, i, x); };
                auto st_r = [&](uint32_t i, uint64_t x) { st64(A.out, d.r2, d.mb, w32, i, x); };
                // long division on one thread or one warp where it finishes
                // sooner than the CTA's shifted inverse (divsmall.cuh)
                if (MB <= SERVE_DIV_THREAD_MAX_MV) {
                    if (threadIdx.x == 0) {
                        const uint8_t st = MB <= 4 ? div_thread<4>(M, MB, ld_u, ld_v, st_q, st_r)
                                                   : div_thread<8>(M, MB, ld_u, ld_v, st_q, st_r);
                        s_flag = st;
                    }
                } else if (MB <= SERVE_DIV_WARP_MAX_MV) {
                    if (threadIdx.x < 32) {
                        const uint8_t st = MB <= 32 ? div_warp<1>(M, MB, ld_u, ld_v, st_q, st_r)
                                                    : MB <= 64 ? div_warp<2>(M, MB, ld_u, ld_v, st_q, st_r)
                                                               : div_warp<4>(M, MB, ld_u, ld_v, st_q, st_r);
                        if (threadIdx.x == 0) s_flag = st;
                    }
                } else {
                    const DivGeom g = div_geom(M, MB, 8);
                    div_cta(g, smem, ld_u, ld_v, st_q, st_r, [&](uint8_t code) { s_flag = code; });
                }
            }
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) serve_complete(A, s_seq, cmd == CLAIM_OK ? s_flag : SERVE_LOST);
    }
    if (threadIdx.x == 0) {
        __threadfence_system();
        if (atomicAdd(&A.dev->left, 1u) == gridDim.x - 1) {
            A.dev->left = 0;
            __threadfence();
            st_release_sys(&A.ctl->exited, A.epoch);
        }
    }
}

static uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Output-arena limbs a request's results take: whole 64-bit limbs, an even
// number of them so that every result starts 16-byte aligned.
static uint64_t result_limbs(const bi_desc& d) {
    uint64_t e;   // result elements
    switch (d.op) {
        case BI_OP_MULFULL: e = 2ull * d.m; break;
        case BI_OP_DIV: e = (uint64_t)d.m + d.mb; break;
        default: e = d.m;
    }
    const uint64_t limbs = desc_w32(d) ? (e + 1) / 2 : e;
    return (limbs + 1) & ~1ull;
}

static size_t request_smem(const bi_desc& d) {
    if (d.op == BI_OP_MUL || d.op == BI_OP_MULFULL) return mul_smem_bytes(mul_geometry(m64(d), d.op == BI_OP_MULFULL, 1));
    if (d.op == BI_OP_DIV) return div_smem_bytes(div_geom(m64(d), mb64(d), 8));
    return 0;
}

struct ServeReq {            // host bookkeeping of one ring slot
    uint64_t seq = 0;
    uint64_t r = 0, r2 = 0;  // result offsets in the output arena
    uint64_t end = 0;        // arena allocation counter after this request
    uint32_t op = 0;
    uint32_t flag = 0;
    uint8_t state = 0;       // 0 free, 1 in flight, 2 completed, 3 released
};

static void percentiles(const uint64_t* lat, uint64_t n, bi_serve_report* rep) {
    if (n == 0) return;
    std::vector<uint64_t> v(lat, lat + n);
    auto q = [&](double f) {
        const uint64_t k = std::min<uint64_t>(n - 1, (uint64_t)(f * (double)n));
        std::nth_element(v.begin(), v.begin() + k, v.end());
        return (double)v[k] * 1e-3;
    };
    rep->p50_us = q(0.50);
    rep->p90_us = q(0.90);
    rep->p99_us = q(0.99);
    rep->p999_us = q(0.999);
    double sum = 0;
    uint64_t mx = 0;
    for (uint64_t i = 0; i < n; i++) {
        sum += (double)lat[i];
        mx = std::max(mx, lat[i]);
    }
    rep->mean_us = sum / (double)n * 1e-3;
    rep->max_us = (double)mx * 1e-3;
}

}  // namespace bi

using namespace bi;

struct bi_server {
    int device = 0;
    cudaStream_t stream = nullptr;
    ServeSlot* slots = nullptr;    // mapped host memory (host and device address alike under UVA)
    ServeDone* cq = nullptr;
    ServeCtl* ctl = nullptr;
    ServeSlot* slots_d = nullptr;
    ServeDone* cq_d = nullptr;
    ServeCtl* ctl_d = nullptr;
    ServeDev* dev = nullptr;
    const uint64_t* in = nullptr;
    uint64_t in_limbs = 0;
    uint64_t* out = nullptr;
    uint64_t out_limbs = 0;        // arena capacity (even)
    bool own_out = false;
    uint32_t S = 0;                // ring slots (power of two)
    uint32_t max_limbs = 0;
    uint32_t grid = 0;
    size_t smem = 0;
    uint64_t idle_ns = 0;
    // host bookkeeping (one client thread)
    uint64_t published = 0;        // requests written to the ring = next ticket
    uint64_t cursor = 0;           // completion-queue entries consumed
    uint64_t released = 0;         // requests whose slot and arena space are free again
    uint64_t alloc_head = 0;       // arena allocation counter (limbs, monotone)
    uint64_t alloc_tail = 0;       // arena reclaim counter
    uint64_t epoch = 0;
    bool running = false;
    uint64_t launches = 0, busy = 0, lost = 0;
    std::vector<ServeReq> req;
};

namespace bi {

static bi_status server_launch(bi_server* s) {
    s->epoch++;
    ServeArgs a;
    a.slots = s->slots_d;
    a.cq = s->cq_d;
    a.ctl = s->ctl_d;
    a.dev = s->dev;
    a.in = s->in;
    a.out = s->out;
    a.mask = s->S - 1;
    a.epoch = s->epoch;
    a.idle_ns = s->idle_ns;
    serve_kernel<<<s->grid, SERVE_CTA, s->smem, s->stream>>>(a);
    BI_RETURN_IF(check_launch("serve kernel"));
    s->running = true;
    s->launches++;
    return BI_OK;
}

// Completion records written but not yet consumed.
static uint64_t cq_ready(const bi_server* s) {
    uint64_t k = 0;
    while (k < s->S) {
        const ServeDone* e = s->cq + ((s->cursor + k) & (s->S - 1));
        if (__atomic_load_n(&e->tag, __ATOMIC_ACQUIRE) != s->cursor + k + 1) break;
        k++;
    }
    return k;
}

// Relaunch the loop if it has ended while requests remain unclaimed.
static bi_status server_kick(bi_server* s) {
    if (s->running && __atomic_load_n(&s->ctl->exited, __ATOMIC_ACQUIRE) == s->epoch) s->running = false;
    if (!s->running && s->cursor + cq_ready(s) < s->published) return server_launch(s);
    return BI_OK;
}

static void server_publish(bi_server* s) { __atomic_store_n(&s->ctl->tail, s->published, __ATOMIC_RELEASE); }

// The checks every request must pass before it is admitted.
static bi_status server_validate(const bi_server* s, const bi_desc& req) {
    bi_desc d = req;
    if (d.op > BI_OP_DIV) return set_error(BI_EINVAL, "serve: unknown op %u", d.op);
    if (d.op != BI_OP_DIV) d.mb = d.m;
    if (d.width != 0 && d.width != 32 && d.width != 64) return set_error(BI_EINVAL, "serve: width %u (0, 32 or 64)", d.width);
    if (d.m == 0 || m64(d) > s->max_limbs)
        return set_error(BI_EINVAL, "serve: m=%u outside the server's max_limbs (%u 64-bit limbs)", d.m, s->max_limbs);
    if (d.mb == 0 || d.mb > d.m) return set_error(BI_EINVAL, "serve: divisor limbs mb=%u outside 1..m", d.mb);
    const uint64_t in_elems = desc_w32(d) ? 2 * s->in_limbs : s->in_limbs;
    if (d.a > in_elems || d.m > in_elems - d.a || d.b > in_elems || d.mb > in_elems - d.b)
        return set_error(BI_EINVAL, "serve: operand outside the operand arena");
    if (request_smem(d) > s->smem) return set_error(BI_EUNSUPPORTED, "serve: request needs more shared memory than the loop holds");
    if (result_limbs(d) > s->out_limbs) return set_error(BI_EINVAL, "serve: result larger than the output arena");
    return BI_OK;
}

// Admit one validated request into the ring without publishing it.
// BI_EBUSY: no slot or no arena room until earlier requests are released.
static bi_status server_admit(bi_server* s, const bi_desc* req, uint64_t* ticket) {
    bi_desc d = *req;
    if (d.op != BI_OP_DIV) d.mb = d.m;
    if (s->published - s->released >= s->S) {
        s->busy++;
        return BI_EBUSY;
    }
    const uint64_t need = result_limbs(d);
    const uint64_t pos = s->alloc_head % s->out_limbs;
    const uint64_t skip = pos + need > s->out_limbs ? s->out_limbs - pos : 0;
    if (s->alloc_head + skip + need - s->alloc_tail > s->out_limbs) {
        s->busy++;
        return BI_EBUSY;
    }
    const uint64_t off = (s->alloc_head + skip) % s->out_limbs;
    s->alloc_head += skip + need;
    d.r = desc_w32(d) ? 2 * off : off;   // in the request's elements
    d.r2 = d.r + d.m;
    d.flag = 0;
    const uint64_t seq = s->published;
    ServeReq& q = s->req[seq & (s->S - 1)];
    q.seq = seq;
    q.r = d.r;
    q.r2 = d.op == BI_OP_DIV ? d.r2 : 0;
    q.end = s->alloc_head;
    q.op = d.op;
    q.flag = 0;
    q.state = 1;
    ServeSlot* slot = s->slots + (seq & (s->S - 1));
    std::memcpy(&slot->d, &d, sizeof(bi_desc));
    __atomic_store_n(&slot->seq, seq, __ATOMIC_RELEASE);
    s->published++;
    if (ticket) *ticket = seq;
    return BI_OK;
}

static uint32_t server_drain(bi_server* s, bi_completion* out, uint32_t max) {
    uint32_t k = 0;
    while (k < max) {
        const ServeDone* e = s->cq + (s->cursor & (s->S - 1));
        if (__atomic_load_n(&e->tag, __ATOMIC_ACQUIRE) != s->cursor + 1) break;
        const uint64_t seq = e->seq, flag = e->flag;
        s->cursor++;
        ServeReq& q = s->req[seq & (s->S - 1)];
        q.state = 2;
        q.flag = (uint32_t)flag;
        if (flag == SERVE_LOST) s->lost++;
        if (out) {
            out[k].ticket = seq;
            out[k].r = q.r;
            out[k].r2 = q.r2;
            out[k].status = (uint32_t)flag;
            out[k].op = q.op;
        }
        k++;
    }
    return k;
}

static bi_status server_release(bi_server* s, uint64_t ticket) {
    if (ticket < s->released || ticket >= s->published) return set_error(BI_EINVAL, "serve: ticket not in flight");
    ServeReq& q = s->req[ticket & (s->S - 1)];
    if (q.seq != ticket || q.state != 2) return set_error(BI_EINVAL, "serve: request %llu has not completed", (unsigned long long)ticket);
    q.state = 3;
    while (s->released < s->published) {
        ServeReq& f = s->req[s->released & (s->S - 1)];
        if (f.state != 3) break;
        s->alloc_tail = f.end;
        f.state = 0;
        s->released++;
    }
    return BI_OK;
}

static void server_free(bi_server* s) {
    if (s->stream) {
        if (s->ctl) __atomic_store_n(&s->ctl->stop, 1ull, __ATOMIC_RELEASE);
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    if (s->slots) cudaFreeHost(s->slots);
    if (s->cq) cudaFreeHost(s->cq);
    if (s->ctl) cudaFreeHost(s->ctl);
    if (s->dev) cudaFree(s->dev);
    if (s->own_out && s->out) cudaFree(s->out);
    delete s;
}

}  // namespace bi

extern "C" {

bi_status bi_server_create(bi_server** server, const uint64_t* in, uint64_t in_limbs, uint64_t* out,
                           uint64_t out_limbs, uint32_t ring_slots, uint32_t max_limbs, uint32_t ctas,
                           uint32_t idle_us) {
    if (!server) return set_error(BI_EINVAL, "serve: NULL server pointer");
    *server = nullptr;
    if (!in || in_limbs == 0) return set_error(BI_EINVAL, "serve: empty operand arena");
    if ((uintptr_t)in % 16 || (out && (uintptr_t)out % 16))
        return set_error(BI_EINVAL, "serve: arenas must be 16-byte aligned");
    if (ring_slots == 0) ring_slots = 65536;
    if (ring_slots & (ring_slots - 1)) return set_error(BI_EINVAL, "serve: ring_slots must be a power of two");
    if (max_limbs == 0) max_limbs = 512;
    if (max_limbs > SERVE_MAX_LIMBS) return set_error(BI_EUNSUPPORTED, "serve: max_limbs above %u", SERVE_MAX_LIMBS);
    if (idle_us == 0) idle_us = 2000;
    bi_server* s = new bi_server();
    s->S = ring_slots;
    s->max_limbs = max_limbs;
    s->in = in;
    s->in_limbs = in_limbs;
    s->idle_ns = (uint64_t)idle_us * 1000;
    s->smem = std::max(mul_smem_bytes(mul_geometry(max_limbs, true, 1)),
                       div_smem_bytes(div_geom(max_limbs, max_limbs, 8)));
    auto fail = [&](bi_status st) {
        server_free(s);
        return st;
    };
    if (cudaGetDevice(&s->device) != cudaSuccess) return fail(set_error(BI_ECUDA, "serve: no device"));
    if (s->smem > 227 * 1024) return fail(set_error(BI_EUNSUPPORTED, "serve: max_limbs needs too much shared memory"));
    if (cudaFuncSetAttribute(serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem) != cudaSuccess)
        return fail(set_error(BI_ECUDA, "serve: shared-memory opt-in failed"));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, serve_kernel, SERVE_CTA, s->smem) != cudaSuccess ||
        per_sm < 1)
        return fail(set_error(BI_ECUDA, "serve: kernel does not fit an SM"));
    s->grid = ctas ? ctas : (uint32_t)(per_sm * num_sms());
    if (out) {
        s->out = out;
        s->out_limbs = out_limbs & ~1ull;
    } else {
        if (out_limbs == 0) {   // default budget: an eighth of the free HBM, at most 2 GiB
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail(set_error(BI_ECUDA, "serve: cudaMemGetInfo"));
            out_limbs = std::min<uint64_t>(free_b / 8 / 8, 1ull << 28);
        }
        s->out_limbs = out_limbs & ~1ull;
        if (cudaMalloc(&s->out, s->out_limbs * 8) != cudaSuccess)
            return fail(set_error(BI_ENOMEM, "serve: output arena of %llu limbs", (unsigned long long)s->out_limbs));
        s->own_out = true;
    }
    if (s->out_limbs < 2) return fail(set_error(BI_EINVAL, "serve: output arena too small"));
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_error(BI_ECUDA, "serve: stream"));
    if (cudaHostAlloc((void**)&s->slots, sizeof(ServeSlot) * s->S, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc((void**)&s->cq, sizeof(ServeDone) * s->S, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostAlloc((void**)&s->ctl, sizeof(ServeCtl), cudaHostAllocMapped) != cudaSuccess)
        return fail(set_error(BI_ENOMEM, "serve: pinned ring"));
    std::memset((void*)s->slots, 0, sizeof(ServeSlot) * s->S);
    std::memset((void*)s->cq, 0, sizeof(ServeDone) * s->S);
    std::memset((void*)s->ctl, 0, sizeof(ServeCtl));
    // no request has number ~0: an empty slot never matches a claim
    for (uint32_t i = 0; i < s->S; i++) s->slots[i].seq = ~0ull;
    if (cudaHostGetDevicePointer((void**)&s->slots_d, s->slots, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->cq_d, s->cq, 0) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->ctl_d, s->ctl, 0) != cudaSuccess)
        return fail(set_error(BI_ECUDA, "serve: mapped pointers"));
    if (cudaMalloc(&s->dev, sizeof(ServeDev)) != cudaSuccess) return fail(set_error(BI_ENOMEM, "serve: control block"));
    if (cudaMemsetAsync(s->dev, 0, sizeof(ServeDev), s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return fail(set_error(BI_ECUDA, "serve: control block init"));
    s->req.resize(s->S);
    *server = s;
    return BI_OK;
}

bi_status bi_server_submit(bi_server* s, const bi_desc* req, uint64_t* ticket) {
    if (!s || !req) return set_error(BI_EINVAL, "serve: NULL argument");
    BI_RETURN_IF(server_validate(s, *req));
    const bi_status st = server_admit(s, req, ticket);
    if (st != BI_OK) return st;
    server_publish(s);
    return server_kick(s);
}

bi_status bi_server_poll(bi_server* s, bi_completion* out, uint32_t max, uint32_t* count) {
    if (!s) return set_error(BI_EINVAL, "serve: NULL server");
    const uint32_t k = server_drain(s, out, max);
    if (count) *count = k;
    return server_kick(s);
}

bi_status bi_server_release(bi_server* s, uint64_t ticket) {
    if (!s) return set_error(BI_EINVAL, "serve: NULL server");
    return server_release(s, ticket);
}

bi_status bi_server_inject_dropped(bi_server* s, uint64_t* ticket) {
    if (!s) return set_error(BI_EINVAL, "serve: NULL server");
    if (s->published - s->released >= s->S) return BI_EBUSY;
    // a slot published with its contents never written: the claiming CTA's
    // bounded wait for the slot's sequence number runs out
    const uint64_t seq = s->published;
    ServeReq& q = s->req[seq & (s->S - 1)];
    q.seq = seq;
    q.r = q.r2 = 0;
    q.end = s->alloc_head;       // no arena space
    q.op = 0xffffffffu;
    q.flag = 0;
    q.state = 1;
    s->published++;
    if (ticket) *ticket = seq;
    server_publish(s);
    return server_kick(s);
}

bi_status bi_server_info(const bi_server* s, uint64_t* info) {
    if (!s || !info) return set_error(BI_EINVAL, "serve: NULL argument");
    info[0] = (uint64_t)(uintptr_t)s->out;
    info[1] = s->out_limbs;
    info[2] = s->grid;
    info[3] = s->smem;
    info[4] = s->launches;
    info[5] = s->busy;
    info[6] = s->lost;
    info[7] = s->S;
    info[8] = s->published;
    info[9] = s->cursor;
    return BI_OK;
}

bi_status bi_server_destroy(bi_server* s) {
    if (!s) return BI_OK;
    server_free(s);
    return BI_OK;
}

bi_status bi_server_replay(bi_server* s, const bi_desc* reqs, const uint64_t* arrival_ns, uint64_t n,
                           uint64_t* latency_ns, bi_completion* done, bi_serve_report* rep) {
    if (!s || (n && (!reqs || !arrival_ns || !latency_ns))) return set_error(BI_EINVAL, "serve: NULL argument");
    for (uint64_t i = 0; i < n; i++) {
        if (i && arrival_ns[i] < arrival_ns[i - 1]) return set_error(BI_EINVAL, "serve: arrival times must not decrease");
        BI_RETURN_IF(server_validate(s, reqs[i]));
    }
    const uint64_t seq0 = s->published, launches0 = s->launches, busy0 = s->busy;
    if (s->published != s->released) return set_error(BI_EINVAL, "serve: replay needs an idle server");
    std::vector<bi_completion> buf(4096);
    uint64_t arrived = 0, admitted = 0, completed = 0;
    const uint64_t t0 = now_ns();
    uint64_t last_progress = t0, t_last = t0;
    while (completed < n) {
        const uint64_t now = now_ns();
        while (arrived < n && arrival_ns[arrived] <= now - t0) arrived++;
        bool progress = false;
        while (admitted < arrived) {
            const bi_status st = server_admit(s, &reqs[admitted], nullptr);
            if (st == BI_EBUSY) break;
            if (st != BI_OK) return st;
            admitted++;
            progress = true;
        }
        if (progress) server_publish(s);
        const uint32_t k = server_drain(s, buf.data(), (uint32_t)buf.size());
        BI_RETURN_IF(server_kick(s));
        if (k) {
            const uint64_t seen = now_ns();
            t_last = seen;
            for (uint32_t j = 0; j < k; j++) {
                const uint64_t idx = buf[j].ticket - seq0;
                latency_ns[idx] = seen - t0 - arrival_ns[idx];
                if (done) done[idx] = buf[j];
                BI_RETURN_IF(server_release(s, buf[j].ticket));
            }
            completed += k;
            progress = true;
        }
        if (progress) last_progress = now;
        else if (now - last_progress > 30ull * 1000000000ull)
            return set_error(BI_ETIMEDOUT, "serve: no progress for 30 s (%llu of %llu done)",
                             (unsigned long long)completed, (unsigned long long)n);
    }
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->requests = (double)n;
        rep->launches = (double)(s->launches - launches0);
        rep->busy = (double)(s->busy - busy0);
        rep->duration_s = (double)(t_last - t0) * 1e-9;
        rep->offered_rps = n && arrival_ns[n - 1] ? (double)n / ((double)arrival_ns[n - 1] * 1e-9) : 0;
        rep->achieved_rps = rep->duration_s > 0 ? (double)n / rep->duration_s : 0;
        percentiles(latency_ns, n, rep);
    }
    return BI_OK;
}

bi_status bi_serve_replay_plain(const uint64_t* in, uint64_t* out, uint64_t out_limbs, const bi_desc* reqs,
                                const uint64_t* arrival_ns, uint64_t n, uint32_t streams, uint64_t* latency_ns,
                                bi_completion* done, bi_serve_report* rep) {
    if (n && (!in || !out || !reqs || !arrival_ns || !latency_ns)) return set_error(BI_EINVAL, "serve: NULL argument");
    if (streams == 0) streams = 1;
    out_limbs &= ~1ull;
    for (uint64_t i = 0; i < n; i++) {
        if (reqs[i].op > BI_OP_DIV || reqs[i].m == 0) return set_error(BI_EINVAL, "serve: bad request %llu", (unsigned long long)i);
        if (reqs[i].width != 0 && reqs[i].width != 32 && reqs[i].width != 64)
            return set_error(BI_EINVAL, "serve: bad request %llu", (unsigned long long)i);
        if (result_limbs(reqs[i]) > out_limbs) return set_error(BI_EINVAL, "serve: output arena too small");
        if (i && arrival_ns[i] < arrival_ns[i - 1]) return set_error(BI_EINVAL, "serve: arrival times must not decrease");
    }
    constexpr uint32_t EV_PER_STREAM = 1024;
    struct Lane {
        cudaStream_t st = nullptr;
        std::vector<cudaEvent_t> ev;
        std::vector<uint64_t> idx;   // request of each event slot
        uint64_t head = 0, tail = 0; // in-flight events [head, tail)
    };
    std::vector<Lane> lanes(streams);
    uint8_t* flags = nullptr;
    std::vector<uint64_t> r_off(n), r2_off(n);
    bi_status result = BI_OK;
    auto cleanup = [&]() {
        for (Lane& l : lanes) {
            if (l.st) cudaStreamSynchronize(l.st);
            for (cudaEvent_t e : l.ev) cudaEventDestroy(e);
            if (l.st) cudaStreamDestroy(l.st);
        }
        if (flags) cudaFree(flags);
    };
    for (Lane& l : lanes) {
        if (cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking) != cudaSuccess) {
            cleanup();
            return set_error(BI_ECUDA, "serve: stream");
        }
        l.ev.resize(EV_PER_STREAM);
        l.idx.resize(EV_PER_STREAM);
        for (cudaEvent_t& e : l.ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                cleanup();
                return set_error(BI_ECUDA, "serve: event");
            }
    }
    if (n && cudaMalloc(&flags, n) != cudaSuccess) {
        cleanup();
        return set_error(BI_ENOMEM, "serve: flags");
    }
    uint64_t arrived = 0, launched = 0, completed = 0, alloc = 0;
    const uint64_t t0 = now_ns();
    uint64_t t_last = t0;
    while (completed < n && result == BI_OK) {
        const uint64_t now = now_ns();
        while (arrived < n && arrival_ns[arrived] <= now - t0) arrived++;
        while (launched < arrived) {
            Lane& l = lanes[launched % streams];
            if (l.tail - l.head >= EV_PER_STREAM) break;
            const bi_desc& d = reqs[launched];
            const uint64_t need = result_limbs(d);
            if (alloc % out_limbs + need > out_limbs) alloc += out_limbs - alloc % out_limbs;
            const uint64_t off = alloc % out_limbs;
            alloc += need;
            const bool w32 = desc_w32(d);
            const uint64_t ro = w32 ? 2 * off : off;   // in the request's elements
            r_off[launched] = ro;
            r2_off[launched] = d.op == BI_OP_DIV ? ro + d.m : 0;
            const bi_stream st = (bi_stream)l.st;
            if (w32) {
                const uint32_t* i32 = reinterpret_cast<const uint32_t*>(in);
                uint32_t* o32 = reinterpret_cast<uint32_t*>(out) + ro;
                switch (d.op) {
                    case BI_OP_ADD: result = bi_add_u32(i32 + d.a, i32 + d.b, o32, d.m, 1, st); break;
                    case BI_OP_SUB: result = bi_sub_u32(i32 + d.a, i32 + d.b, o32, flags + launched, d.m, 1, st); break;
                    case BI_OP_MUL: result = bi_mul_u32(i32 + d.a, i32 + d.b, o32, d.m, 1, st); break;
                    case BI_OP_MULFULL: result = bi_mulfull_u32(i32 + d.a, i32 + d.b, o32, d.m, 1, st); break;
                    default:
                        result = bi_div_u32(i32 + d.a, i32 + d.b, o32, o32 + d.m, flags + launched, d.m, d.mb, 1, st);
                }
            } else {
                switch (d.op) {
                    case BI_OP_ADD: result = bi_add_u64(in + d.a, in + d.b, out + off, d.m, 1, st); break;
                    case BI_OP_SUB: result = bi_sub_u64(in + d.a, in + d.b, out + off, flags + launched, d.m, 1, st); break;
                    case BI_OP_MUL: result = bi_mul_u64(in + d.a, in + d.b, out + off, d.m, 1, st); break;
                    case BI_OP_MULFULL: result = bi_mulfull_u64(in + d.a, in + d.b, out + off, d.m, 1, st); break;
                    default:
                        result = bi_div_u64(in + d.a, in + d.b, out + off, out + off + d.m, flags + launched, d.m, d.mb, 1, st);
                }
            }
            if (result != BI_OK) break;
            const uint64_t e = l.tail % EV_PER_STREAM;
            if (cudaEventRecord(l.ev[e], l.st) != cudaSuccess) {
                result = set_error(BI_ECUDA, "serve: event record");
                break;
            }
            l.idx[e] = launched;
            l.tail++;
            launched++;
        }
        for (Lane& l : lanes) {
            while (l.head < l.tail) {
                const uint64_t e = l.head % EV_PER_STREAM;
                const cudaError_t q = cudaEventQuery(l.ev[e]);
                if (q == cudaErrorNotReady) break;
                if (q != cudaSuccess) {
                    result = set_error(BI_ECUDA, "serve: %s", cudaGetErrorString(q));
                    break;
                }
                const uint64_t seen = now_ns(), i = l.idx[e];
                latency_ns[i] = seen - t0 - arrival_ns[i];
                t_last = seen;
                l.head++;
                completed++;
            }
        }
    }
    if (result == BI_OK && done) {
        std::vector<uint8_t> hf(n);
        if (n && cudaMemcpy(hf.data(), flags, n, cudaMemcpyDeviceToHost) != cudaSuccess)
            result = set_error(BI_ECUDA, "serve: flags copy");
        for (uint64_t i = 0; i < n && result == BI_OK; i++) {
            done[i].ticket = i;
            done[i].r = r_off[i];
            done[i].r2 = r2_off[i];
            done[i].op = reqs[i].op;
            done[i].status = (reqs[i].op == BI_OP_SUB || reqs[i].op == BI_OP_DIV) ? hf[i] : 0;
        }
    }
    cleanup();
    if (result != BI_OK) return result;
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->requests = (double)n;
        rep->launches = (double)n;
        rep->duration_s = (double)(t_last - t0) * 1e-9;
        rep->offered_rps = n && arrival_ns[n - 1] ? (double)n / ((double)arrival_ns[n - 1] * 1e-9) : 0;
        rep->achieved_rps = rep->duration_s > 0 ? (double)n / rep->duration_s : 0;
        percentiles(latency_ns, n, rep);
    }
    return BI_OK;
}

}  // extern "C"
