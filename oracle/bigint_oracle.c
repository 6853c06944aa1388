/*
 * bigint_oracle.c -- CPU oracle for the batched big-integer library.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU and in plain C,
 * the arithmetic that tossenxD/big-int defines for its hot path, so that the
 * CUDA kernels can be checked against it bit for bit.  Only the test suite,
 * the smoke check and the benchmark's CPU-baseline leg may load it; the
 * library itself never calls into it.
 *
 * Representation (as in the reference, cuda/ker-helpers.cu.h:28-44 and
 * prototypes/div.c:24-26): a batch is a flat row-major array [n][m] of
 * little-endian limbs; instance i starts at limb i*m.  Everything here works
 * on 32-bit digits.  A u64 limb array on a little-endian host *is* a u32
 * digit array of twice the length, so the u64 entry points reinterpret their
 * buffers and call the u32 routines with 2m digits; every operation below
 * (mod-B^m add, sign-magnitude sub, truncated and full product, quotient and
 * remainder) is invariant under that regrouping.
 *
 * Per-function citations give the reference file:line each one follows.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef uint32_t dg;          /* one 32-bit digit */

/* ------------------------------------------------------------------------ */
/* Single-instance kernels on u32 digits                                     */
/* ------------------------------------------------------------------------ */

/* r = (a + b) mod B^m; the carry out of the top digit is dropped.
 * Semantics of baddKer{1,2,3} (cuda/ker-add.cu.h:50-67, 121-149, 212-243):
 * the carry-lookahead scan there computes exactly the ripple sum below. */
static void add_one(const dg* a, const dg* b, dg* r, uint32_t m) {
    uint64_t c = 0;
    for (uint32_t i = 0; i < m; i++) {
        uint64_t s = (uint64_t)a[i] + b[i] + c;
        r[i] = (dg)s;
        c = s >> 32;
    }
}

/* Sign-magnitude subtraction: r = |a - b|, sign = (a < b).
 * futhark/sub.fut:14-26 (bsub): pick the larger operand with `lt`
 * (futhark/helper.fut:109-112), subtract with borrow propagation. */
static int less_than(const dg* a, const dg* b, uint32_t m) {
    for (uint32_t i = m; i-- > 0;) {
        if (a[i] != b[i]) return a[i] < b[i];
    }
    return 0;
}

static uint8_t sub_one(const dg* a, const dg* b, dg* r, uint32_t m) {
    uint8_t sign = (uint8_t)less_than(a, b, m);
    const dg* g = sign ? b : a;
    const dg* l = sign ? a : b;
    uint64_t br = 0;
    for (uint32_t i = 0; i < m; i++) {
        uint64_t d = (uint64_t)g[i] - l[i] - br;
        r[i] = (dg)d;
        br = (d >> 63) & 1;   /* borrow iff the 64-bit difference wrapped */
    }
    return sign;
}

/* Schoolbook product of a (ma digits) and b (mb digits), written to w with
 * mw digits (the product is reduced mod B^mw; digits above ma+mb are zero).
 * Column semantics follow cuda/ker-mul.cu.h:147-184 (column k collects
 * a_i*b_{k-i}) and thesis/sections/multiplication.tex; the order of the
 * partial products does not change the exact result. */
static void mul_into(const dg* a, uint32_t ma, const dg* b, uint32_t mb,
                     dg* w, uint32_t mw) {
    memset(w, 0, (size_t)mw * sizeof(dg));
    /* trim leading zero digits: exact, and keeps the oracle fast */
    while (ma > 0 && a[ma - 1] == 0) ma--;
    while (mb > 0 && b[mb - 1] == 0) mb--;
    for (uint32_t i = 0; i < ma && i < mw; i++) {
        uint64_t c = 0;
        uint64_t ai = a[i];
        if (ai == 0) continue;
        uint32_t j = 0;
        for (; j < mb && i + j < mw; j++) {
            uint64_t t = ai * b[j] + w[i + j] + c;
            w[i + j] = (dg)t;
            c = t >> 32;
        }
        for (uint32_t k = i + j; c != 0 && k < mw; k++) {
            uint64_t t = (uint64_t)w[k] + c;
            w[k] = (dg)t;
            c = t >> 32;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Division: restatement of prototypes/div.c (shifted inverse, refine3).     */
/* The reference delegates add/sub/mult to GMP; here they are schoolbook    */
/* routines with the same results.  All buffers have precision p digits.    */
/* ------------------------------------------------------------------------ */

/* index of the most significant nonzero digit, 0 for zero (div.c:92-96) */
static int top_digit(const dg* u, int p) {
    for (int i = p - 1; i > 0; i--) if (u[i] != 0) return i;
    return 0;
}

static int is_zero(const dg* u, int p) {
    for (int i = 0; i < p; i++) if (u[i]) return 0;
    return 1;
}

/* Word products of the division's multiplications, counted as GMP's
 * mpz_mul does them on the operands' significant digits (the reference's
 * mult, div.c:184-199, and mpz_mul_ui): the work figure of the division's
 * roofline, per thread, read by orc_div_ref_word_products_u32. */
static __thread uint64_t g_div_wp;

static void count_wp(const dg* u, int pu, const dg* v, int pv) {
    if (is_zero(u, pu) || is_zero(v, pv)) return;
    g_div_wp += (uint64_t)(top_digit(u, pu) + 1) * (uint64_t)(top_digit(v, pv) + 1);
}

static int equal(const dg* u, const dg* v, int p) {
    return memcmp(u, v, (size_t)p * sizeof(dg)) == 0;
}

/* v = u * B^n for n >= 0, floor(u / B^-n) for n < 0, mod B^p; in place ok
 * (div.c:105-117) */
static void dshift(int n, const dg* u, dg* v, int p) {
    if (n >= 0) {
        for (int i = p - 1; i >= 0; i--) v[i] = (i - n >= 0) ? u[i - n] : 0;
    } else {
        for (int i = 0; i < p; i++) v[i] = (i - n < p) ? u[i - n] : 0;
    }
}

/* u = B^n (div.c:121-126) */
static void set_pow(dg* u, int n, int p) {
    memset(u, 0, (size_t)p * sizeof(dg));
    if (n >= 0 && n < p) u[n] = 1;
}

static void set_digit(dg* u, dg d, int p) {
    memset(u, 0, (size_t)p * sizeof(dg));
    u[0] = d;
}

/* w = u + v mod B^p (div.c:129-144 via GMP) */
static void dadd(const dg* u, const dg* v, dg* w, int p) { add_one(u, v, w, (uint32_t)p); }

/* w = |u - v| (div.c:147-162: GMP mpz_sub then export of the magnitude) */
static void dsub_abs(const dg* u, const dg* v, dg* w, int p) { (void)sub_one(u, v, w, (uint32_t)p); }

/* w = u * v restricted to the low p digits of each operand, result mod B^p.
 * div.c:184-199 imports p digits of each operand and exports the whole
 * product; every call site in the reference keeps the product inside p
 * digits, so the reduction never drops a nonzero digit there. */
static void dmul(const dg* u, const dg* v, dg* w, int p, dg* tmp) {
    count_wp(u, p, v, p);
    mul_into(u, (uint32_t)p, v, (uint32_t)p, tmp, (uint32_t)p);
    memcpy(w, tmp, (size_t)p * sizeof(dg));
}

/* w = u * d, single digit, mod B^p (div.c:202-218) */
static void dmul_digit(const dg* u, dg d, dg* w, int p) {
    if (d && !is_zero(u, p)) g_div_wp += (uint64_t)(top_digit(u, p) + 1);
    uint64_t c = 0;
    for (int i = 0; i < p; i++) {
        uint64_t t = (uint64_t)u[i] * d + c;
        w[i] = (dg)t;
        c = t >> 32;
    }
}

/* w = floor(u / d), single digit long division (div.c:165-181) */
static void ddiv_digit(const dg* u, dg d, dg* w, int p) {
    uint64_t r = 0;
    for (int i = p - 1; i >= 0; i--) {
        r = (r << 32) | u[i];
        w[i] = (dg)(r / d);
        r = r % d;
    }
}

typedef struct {
    int p;
    dg *t0, *t1, *t2, *t3, *mt;   /* scratch, each p digits (mt: 2p) */
} dctx;

/* powerdiff: P = |B^h - v*w| with the sign returned (1 = negative)
 * (div.c:246-280).  The L < h branch follows the reference literally,
 * including its use of the full product of the L-digit truncations
 * (multmod, div.c:221-242). */
static int powerdiff(dctx* c, const dg* v, const dg* w, int h, int l, dg* P) {
    int p = c->p;
    int L = (top_digit(v, p) + 1) + (top_digit(w, p) + 1) - l + 1;
    int neg = 0;
    if (is_zero(v, p) || is_zero(w, p)) {
        set_pow(P, h, p);
    } else if (L >= h) {
        dmul(v, w, P, p, c->mt);
        dg* bh = c->t3;
        set_pow(bh, h, p);
        if (less_than(P, bh, (uint32_t)p)) {
            dsub_abs(bh, P, P, p);
        } else {
            dsub_abs(P, bh, P, p);
            neg = 1;
        }
    } else {
        /* multmod: full product of the low L digits of v and w */
        memset(P, 0, (size_t)p * sizeof(dg));
        count_wp(v, L, w, L);
        mul_into(v, (uint32_t)L, w, (uint32_t)L, c->mt, (uint32_t)p);
        memcpy(P, c->mt, (size_t)p * sizeof(dg));
        if (!is_zero(P, p)) {
            if (P[L - 1] == 0) {
                neg = 1;
            } else {
                dg* bl = c->t3;
                set_pow(bl, L, p);
                if (less_than(P, bl, (uint32_t)p)) {
                    dsub_abs(bl, P, P, p);
                } else {
                    dsub_abs(P, bl, P, p);
                    neg = 1;
                }
            }
        }
    }
    return neg;
}

/* one Newton step: w = w*B^n +/- floor(w * |B^(h-n) - v*w| * B^(2n-h))
 * (div.c:283-304) */
static void newton_step(dctx* c, int h, const dg* v, dg* w, int n, int l, int g) {
    int p = c->p;
    dg* P = c->t1;
    dg* w0 = c->t2;
    dshift(n, w, w0, p);
    int neg = powerdiff(c, v, w, h - n, l - g, P);
    dmul(w, P, w, p, c->mt);
    dshift(2 * n - h, w, w, p);
    if (neg) dsub_abs(w, w0, w, p);
    else     dadd(w, w0, w, p);
}

/* refine3: shorter iterates and divisor prefixes, g = p/4 guard digits
 * (div.c:333-349) */
static void refine3(dctx* c, const dg* v, int h, int k, dg* w, int l) {
    int p = c->p;
    int g = p / 4;
    dshift(g, w, w, p);
    dg* v0 = c->t0;
    while (h - k > l) {
        int n = (h - k + 1 - l < l) ? (h - k + 1 - l) : l;
        int s = k - 2 * l + 1 - g;
        if (s < 0) s = 0;
        dshift(-s, v, v0, p);
        newton_step(c, k + l + n - s + g, v0, w, n, l, g);
        dshift(-1, w, w, p);
        l += n - 1;
    }
    dshift(-g, w, w, p);
}

/* w = floor(B^h / v), whole shifted inverse (div.c:352-423) */
static void shinv(dctx* c, const dg* v, int h, int k, dg* w) {
    int p = c->p;
    dg* tmp = c->t1;
    /* special cases so that B < v <= B^h / 2 holds afterwards */
    if (top_digit(v, p) == 0) {                 /* v < B */
        set_pow(tmp, h, p);
        ddiv_digit(tmp, v[0], w, p);
        return;
    }
    set_pow(tmp, h, p);
    if (less_than(tmp, v, (uint32_t)p)) {       /* B^h < v */
        set_digit(w, 0, p);
        return;
    }
    dg* v2 = c->t2;
    dmul_digit(v, 2, v2, p);
    if (less_than(tmp, v2, (uint32_t)p)) {      /* B^h < 2v */
        set_digit(w, 1, p);
        return;
    }
    set_pow(tmp, k, p);
    if (equal(v, tmp, p)) {                     /* v = B^k */
        set_pow(w, h - k, p);
        return;
    }
    /* initial approximation from the three leading digits:
     * r = (B^4 - V)/V + 1 evaluated in 128-bit arithmetic (div.c:406-417) */
    unsigned __int128 V = ((unsigned __int128)v[k] << 64)
                        | ((unsigned __int128)v[k - 1] << 32)
                        | (unsigned __int128)v[k - 2];
    unsigned __int128 r = ((unsigned __int128)0 - V) / V + 1;
    memset(w, 0, (size_t)p * sizeof(dg));
    w[0] = (dg)r;
    w[1] = (dg)(r >> 32);
    w[2] = (dg)(r >> 64);
    w[3] = (dg)(r >> 96);
    int l = 2;
    if (h - k <= l) dshift(h - k - l, w, w, p);
    else            refine3(c, v, h, k, w, l);
}

/* Quotient and remainder of u by v, both m digits, following div_shinv
 * (div.c:427-467): q = floor(u * shinv_h(v) / B^h) + delta.  Internal
 * precision is 4m digits as in the reference.  v must be nonzero.
 *
 * `faithful` = 1 applies the reference's single delta step (delta in {0,1},
 * div.c:459-463) exactly as written.  That step is not always enough: for
 * some inputs the estimate is two short and div.c returns a remainder >= v
 * (e.g. u = 0xdc4461359674c9cfd718dc1b567834b5, v = 0xdd2982a538271953 with
 * m = 4 digits; about 0.05-0.4 % of random inputs whose divisor has half the
 * dividend's digits).  `faithful` = 0 repeats the step while r >= v, which
 * yields the exact quotient and remainder -- the results the reference
 * itself validates against (mpz_div, div.c:470-486, 525-532). */
static void div_one(const dg* u, const dg* v, dg* q, dg* r, uint32_t m, int faithful) {
    int p = 4 * (int)m;
    dg* buf = (dg*)calloc((size_t)p * 9, sizeof(dg));
    dg *a = buf, *b = buf + p, *cc = buf + 2 * p;
    dctx c;
    c.p = p;
    c.t0 = buf + 3 * p; c.t1 = buf + 4 * p; c.t2 = buf + 5 * p; c.t3 = buf + 6 * p;
    c.mt = buf + 7 * p;                          /* 2p digits */
    int h = top_digit(u, (int)m) + 1;
    int k = top_digit(v, (int)m);
    memcpy(a, u, m * sizeof(dg));
    memcpy(b, v, m * sizeof(dg));
    if (k == 1) {                               /* div.c:443-448 */
        h++; k++;
        dshift(1, a, a, (int)m + 1);
        dshift(1, b, b, (int)m + 1);
    }
    shinv(&c, b, h, k, cc);
    dmul(a, cc, b, p, c.mt);
    dshift(-h, b, b, p);
    memcpy(q, b, m * sizeof(dg));
    /* remainder and the delta correction (div.c:457-463) */
    dg* vq = a;
    count_wp(v, (int)m, q, (int)m);
    mul_into(v, m, q, m, vq, (uint32_t)p);
    (void)sub_one(u, vq, r, m);
    while (!less_than(r, v, m)) {
        set_digit(a, 1, (int)m);
        add_one(q, a, q, m);
        (void)sub_one(r, v, r, m);
        if (faithful) break;
    }
    free(buf);
}

/* ------------------------------------------------------------------------ */
/* Batched entry points (u32 digits), optionally multi-threaded              */
/* ------------------------------------------------------------------------ */

enum { OP_ADD, OP_SUB, OP_MUL, OP_MULFULL, OP_DIV, OP_DIV_REF };

typedef struct {
    int op;
    const dg *a, *b;
    dg *r, *r2;
    uint8_t* sign;
    uint32_t m, mb;
    uint64_t lo, hi;
    int status;
} job_t;

static void run_range(job_t* j) {
    uint32_t m = j->m;
    for (uint64_t i = j->lo; i < j->hi; i++) {
        switch (j->op) {
        case OP_ADD:
            add_one(j->a + i * m, j->b + i * m, j->r + i * m, m);
            break;
        case OP_SUB:
            j->sign[i] = sub_one(j->a + i * m, j->b + i * m, j->r + i * m, m);
            break;
        case OP_MUL:
            mul_into(j->a + i * m, m, j->b + i * m, m, j->r + i * m, m);
            break;
        case OP_MULFULL:
            mul_into(j->a + i * m, m, j->b + i * m, m, j->r + 2 * i * m, 2 * m);
            break;
        case OP_DIV:
        case OP_DIV_REF: {
            /* dividend m digits, divisor mb <= m digits: pad the divisor to
             * m digits as the reference requires equal sizes (div.c:427) */
            uint32_t mb = j->mb;
            const dg* vi = j->b + i * mb;
            int zero = 1;
            for (uint32_t t = 0; t < mb; t++) if (vi[t]) { zero = 0; break; }
            dg* q = j->r + i * m;
            dg* rr = j->r2 + i * mb;
            if (zero) {
                memset(q, 0, m * sizeof(dg));
                memset(rr, 0, mb * sizeof(dg));
                if (j->sign) j->sign[i] = 1;
                j->status = 2;
                break;
            }
            dg* vpad = (dg*)calloc(m, sizeof(dg));
            dg* rpad = (dg*)calloc(m, sizeof(dg));
            memcpy(vpad, vi, mb * sizeof(dg));
            div_one(j->a + i * m, vpad, q, rpad, m, j->op == OP_DIV_REF);
            memcpy(rr, rpad, mb * sizeof(dg));
            if (j->sign) j->sign[i] = 0;
            free(vpad);
            free(rpad);
            break;
        }
        }
    }
}

static void* thread_main(void* arg) { run_range((job_t*)arg); return NULL; }

static int run_batch(job_t proto, uint64_t n, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((uint64_t)nthreads > n) nthreads = n ? (int)n : 1;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = proto;
        jobs[t].lo = n * (uint64_t)t / (uint64_t)nthreads;
        jobs[t].hi = n * (uint64_t)(t + 1) / (uint64_t)nthreads;
        jobs[t].status = 0;
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, thread_main, &jobs[t]);
    run_range(&jobs[0]);
    int status = jobs[0].status;
    for (int t = 1; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        if (jobs[t].status) status = jobs[t].status;
    }
    free(jobs);
    free(th);
    return status;
}

/* ---- exported u32 API ---- */

int orc_add_u32(const dg* a, const dg* b, dg* r, uint32_t m, uint64_t n, int nt) {
    job_t j = {OP_ADD, a, b, r, NULL, NULL, m, 0, 0, 0, 0};
    return run_batch(j, n, nt);
}
int orc_sub_u32(const dg* a, const dg* b, dg* r, uint8_t* sign, uint32_t m, uint64_t n, int nt) {
    job_t j = {OP_SUB, a, b, r, NULL, sign, m, 0, 0, 0, 0};
    return run_batch(j, n, nt);
}
int orc_mul_u32(const dg* a, const dg* b, dg* r, uint32_t m, uint64_t n, int nt) {
    job_t j = {OP_MUL, a, b, r, NULL, NULL, m, 0, 0, 0, 0};
    return run_batch(j, n, nt);
}
int orc_mulfull_u32(const dg* a, const dg* b, dg* r, uint32_t m, uint64_t n, int nt) {
    job_t j = {OP_MULFULL, a, b, r, NULL, NULL, m, 0, 0, 0, 0};
    return run_batch(j, n, nt);
}
/* u: [n][mu], v: [n][mv] (mv <= mu), q: [n][mu], r: [n][mv];
 * status[i] = 1 where v_i == 0 (then q_i = r_i = 0).  Returns 2 if any
 * divisor was zero, else 0. */
int orc_div_u32(const dg* u, const dg* v, dg* q, dg* r, uint8_t* status,
                uint32_t mu, uint32_t mv, uint64_t n, int nt) {
    if (mv > mu) return 1;
    job_t j = {OP_DIV, u, v, q, r, status, mu, mv, 0, 0, 0};
    return run_batch(j, n, nt);
}

/* The reference's division exactly as written (single delta step); for
 * pinning the oracle against prototypes/div.c and documenting its defect. */
int orc_div_ref_u32(const dg* u, const dg* v, dg* q, dg* r, uint8_t* status,
                    uint32_t mu, uint32_t mv, uint64_t n, int nt) {
    if (mv > mu) return 1;
    job_t j = {OP_DIV_REF, u, v, q, r, status, mu, mv, 0, 0, 0};
    return run_batch(j, n, nt);
}

/* ---- exported u64 API: the same arrays viewed as u32 digits ---- */

int orc_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, int nt) {
    return orc_add_u32((const dg*)a, (const dg*)b, (dg*)r, 2 * m, n, nt);
}
int orc_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* sign, uint32_t m, uint64_t n, int nt) {
    return orc_sub_u32((const dg*)a, (const dg*)b, (dg*)r, sign, 2 * m, n, nt);
}
int orc_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, int nt) {
    return orc_mul_u32((const dg*)a, (const dg*)b, (dg*)r, 2 * m, n, nt);
}
int orc_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t m, uint64_t n, int nt) {
    return orc_mulfull_u32((const dg*)a, (const dg*)b, (dg*)r, 2 * m, n, nt);
}
int orc_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r, uint8_t* status,
                uint32_t mu, uint32_t mv, uint64_t n, int nt) {
    return orc_div_u32((const dg*)u, (const dg*)v, (dg*)q, (dg*)r, status, 2 * mu, 2 * mv, n, nt);
}

/* 1 on a little-endian host (the u64 <-> u32 view above needs it) */
/* Word products (32x32-bit) of the multiplications the reference's division
 * performs for one instance -- u and v of m u32 digits, v nonzero, the
 * reference's single delta step -- counted on significant digits as GMP
 * multiplies them.  0 for a zero divisor. */
uint64_t orc_div_ref_word_products_u32(const dg* u, const dg* v, uint32_t m) {
    if (is_zero(v, (int)m)) return 0;
    dg* q = (dg*)calloc(m, sizeof(dg));
    dg* r = (dg*)calloc(m, sizeof(dg));
    g_div_wp = 0;
    div_one(u, v, q, r, m, 1);
    const uint64_t wp = g_div_wp;
    free(q);
    free(r);
    return wp;
}

int orc_little_endian(void) {
    const uint64_t x = 1;
    return *(const uint8_t*)&x == 1;
}
