/*
 * bigint_gb300.h -- C ABI of the GB300 batched big-integer library.
 *
 * Batches are flat row-major arrays [n][m] of little-endian limbs (u32 or
 * u64): instance i occupies limbs [i*m, (i+1)*m), least significant limb
 * first.  This is the layout of the reference's kernels and host wrappers
 * (tossenxD/big-int cuda/ker-helpers.cu.h:117-187, cuda/main.cu:118-128).
 *
 * Conventions (replacing the reference's print-and-continue gpuAssert and
 * exit()-ing CUDA_CHECK, cuda/helpers.h:21-27,192-203):
 *   - every call returns a bi_status; BI_OK is 0; no call ever exits;
 *   - device entry points take device pointers and a CUDA stream (a
 *     cudaStream_t passed as bi_stream; NULL means the legacy default
 *     stream); they are asynchronous with respect to the host and
 *     stream-ordered, and they allocate no memory;
 *   - host entry points (bi_host_*) take host pointers and return when the
 *     results are back in host memory -- the shape of the reference's
 *     gpuAdd/gpuMultiply wrappers.  If every host buffer of the call is
 *     pinned (cudaHostAlloc / cudaHostRegister), the kernel reads and writes
 *     them in place over the CPU-GPU link; otherwise the batch is cut into
 *     chunks whose copies in, kernels and copies out overlap on three
 *     streams;
 *   - n == 0 is a no-op; m == 0 or a NULL buffer with n > 0 is BI_EINVAL;
 *   - any n is accepted: unlike the reference launch (grid = n/ipb, which
 *     drops the remainder, cuda/main.cu:135,307) every instance is computed;
 *   - device buffers need the natural alignment of their limb type; 16-byte
 *     aligned buffers take the vectorised path;
 *   - calls are thread-safe; concurrent calls on different streams overlap.
 */
#ifndef BIGINT_GB300_H
#define BIGINT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int bi_status;
#define BI_OK            0
#define BI_EINVAL        1  /* bad size, NULL pointer, misaligned buffer */
#define BI_EDIV0         2  /* a divisor was zero (host division entry) */
#define BI_ENOMEM        3  /* device allocation failed (host entries) */
#define BI_ETIMEDOUT     4  /* a bounded device wait gave up */
#define BI_ECUDA         5  /* a CUDA runtime call or launch failed */
#define BI_EUNSUPPORTED  6  /* size beyond what this build supports */
#define BI_EBUSY         7  /* serving loop full: retry after a poll/release */

typedef void* bi_stream;

/* Human-readable name of a status code. */
const char* bi_status_string(bi_status status);

/* Detail text of the last failing call on the calling thread ("" if none). */
const char* bi_last_error(void);

/* Library version as 10000*major + 100*minor + patch. */
int bi_version(void);

/* Largest m (in limbs) the one-instance-per-tile add/sub kernels accept. */
uint32_t bi_max_limbs_addsub_u64(void);
uint32_t bi_max_limbs_addsub_u32(void);

/* ---------------------------------------------------------------------- */
/* Addition: r_i = (a_i + b_i) mod B^m, carry-out dropped.                 */
/* Replaces baddKer1/2/3 (cuda/ker-add.cu.h:69-86, 152-172, 246-266) as    */
/* launched by gpuAdd (cuda/main.cu:108-222).  r may alias a or b.         */
/* ---------------------------------------------------------------------- */
bi_status bi_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                     uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                     uint32_t m, uint64_t n, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* Signed (sign-magnitude) subtraction: r_i = |a_i - b_i|,                 */
/* sign[i] = 1 if a_i < b_i else 0.  Replaces bsub (futhark/sub.fut:14-26),*/
/* exported there as test_sub (futhark/test/gmp-validation-lib.fut:16-17), */
/* which the reference validates against mpz_abs(a - b)                    */
/* (futhark/test/gmp-validation.c:38-41).  sign may be NULL.               */
/* ---------------------------------------------------------------------- */
bi_status bi_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                     uint8_t* sign, uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_sub_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                     uint8_t* sign, uint32_t m, uint64_t n, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* Classical (quadratic) multiplication.                                   */
/* bi_mul_*:     r_i = (a_i * b_i) mod B^m, r is [n][m] -- the truncated   */
/*               product of convMul1..5 (cuda/ker-mul.cu.h:202-221,        */
/*               310-329, 420-439, 532-551, 647-666) as launched by        */
/*               gpuMultiply (cuda/main.cu:280-419).                       */
/* bi_mulfull_*: r_i = a_i * b_i, r is [n][2m] -- the full product, which  */
/*               the reference obtains only by zero-padding to 2m limbs.   */
/* r must not overlap a or b.  m <= bi_max_limbs_mul_* ().                 */
/* ---------------------------------------------------------------------- */
uint32_t bi_max_limbs_mul_u64(void);
uint32_t bi_max_limbs_mul_u32(void);
bi_status bi_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                     uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_mul_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                     uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                         uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_mulfull_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                         uint32_t m, uint64_t n, bi_stream stream);

/* Tiling of the CTA multiply (64-bit limb arithmetic): instances per CTA */
/* and row slices per window pair. Full products of at most 24 64-bit     */
/* limbs and truncated ones of at most 32 run by default on the thread    */
/* kernel (one thread an instance, 64-bit limbs), full products of 25 to  */
/* 32 limbs on the warp kernel (32-bit words). bi_mul_autotune_* times    */
/* every tiling that fits on the caller's a, b -- and the warp kernel for */
/* full products of at most 32 64-bit limbs, the thread kernel where it   */
/* takes the size -- (median of `reps` runs each), records the fastest    */
/* for this device, limb width, product kind (full != 0: bi_mulfull_*)    */
/* and m, which later calls then use, and leaves r as that call writes    */
/* it; synchronous on `stream`.  chosen (may be NULL) gets {instances per */
/* CTA, slices}, or {0, 0} when the warp kernel was fastest, {0, 1} for   */
/* the thread kernel.  The reference fixes its tiling per size at compile */
/* time (ipb and the Q limbs per thread, cuda/main.cu:15-28).             */
/* bi_mul_set_tuning_* sets a tiling by hand (BI_EINVAL if it does not    */
/* fit a CTA); ipc = -1 picks a per-instance kernel (slices = 0: the warp */
/* kernel, full products of at most 32 limbs; 1: the thread kernel, full  */
/* products of at most 24 limbs, truncated ones of at most 32); ipc = 0   */
/* returns (m, full) to the library's own choice.                         */
bi_status bi_mul_autotune_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                              uint32_t m, uint64_t n, int full, int reps, int* chosen,
                              bi_stream stream);
bi_status bi_mul_autotune_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                              uint32_t m, uint64_t n, int full, int reps, int* chosen,
                              bi_stream stream);
bi_status bi_mul_set_tuning_u64(uint32_t m, int full, int ipc, int slices);
bi_status bi_mul_set_tuning_u32(uint32_t m, int full, int ipc, int slices);

/* ---------------------------------------------------------------------- */
/* Division with remainder: q_i = floor(u_i / v_i), r_i = u_i mod v_i.     */
/* u is [n][mu], v is [n][mv] with mv <= mu, q is [n][mu], r is [n][mv].   */
/* Replaces div_shinv (prototypes/div.c:427-467; quotient by a shifted     */
/* inverse refined with shorter iterates and divisor prefixes) and the     */
/* Futhark div / test_div (futhark/div.fut:150-167,                        */
/* futhark/test/gmp-validation-lib.fut:26-27), which require equal sizes;  */
/* here the divisor may be shorter.  status (may be NULL) is [n]:          */
/* 0 = ok, 1 = divisor zero (q_i and r_i are set to 0), 2 = internal      */
/* correction bound exceeded (never observed).  The reference divides by   */
/* zero (div.c:165-181); this entry reports it per instance instead.       */
/* q and r must not overlap u, v or each other.                            */
/* mu <= bi_max_limbs_div_* () (8192 64-bit limbs), mv <= 4096 64-bit    */
/* limbs.                                                                  */
/* ---------------------------------------------------------------------- */
uint32_t bi_max_limbs_div_u64(void);
uint32_t bi_max_limbs_div_u32(void);
bi_status bi_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r,
                     uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                     bi_stream stream);
bi_status bi_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r,
                     uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                     bi_stream stream);
/* The method depends on the divisor's size in 64-bit limbs and on n (the */
/* results do not: q and r are unique): schoolbook long division on one   */
/* thread per instance up to 16 limbs and on one warp or lane group (8 or */
/* 16 lanes, 1 to 32 limbs a lane) per instance up to 128 limbs, and up   */
/* to 1024 limbs once n exceeds a few instances per SM (otherwise the     */
/* shifted inverse on one CTA per instance); above 1024 limbs long        */
/* division 8 quotient limbs at a time on two or four warps.              */
/* The _shinv entries take the shifted inverse at every size (the         */
/* reference's algorithm; dividends up to 2048 64-bit limbs, else         */
/* BI_EUNSUPPORTED), the _long entries long division (divisors up to 4096 */
/* 64-bit limbs); same arguments and results.                             */
bi_status bi_div_shinv_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r,
                           uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                           bi_stream stream);
bi_status bi_div_shinv_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r,
                           uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                           bi_stream stream);
bi_status bi_div_long_u64(const uint64_t* u, const uint64_t* v, uint64_t* q, uint64_t* r,
                          uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                          bi_stream stream);
bi_status bi_div_long_u32(const uint32_t* u, const uint32_t* v, uint32_t* q, uint32_t* r,
                          uint8_t* status, uint32_t mu, uint32_t mv, uint64_t n,
                          bi_stream stream);

/* ---------------------------------------------------------------------- */
/* Host-pointer twins of the above (synchronous, pipelined; see top).     */
/* Mirror gpuAdd<Base,m,v>(n, h_as, h_bs, h_rs) (cuda/main.cu:108-110) and */
/* gpuMultiply<Base,m,v>(n, h_as, h_bs, h_rs) (cuda/main.cu:280-282).      */
/* ---------------------------------------------------------------------- */
bi_status bi_host_mul_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                          uint32_t m, uint64_t n);
bi_status bi_host_mul_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                          uint32_t m, uint64_t n);
bi_status bi_host_mulfull_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                              uint32_t m, uint64_t n);
bi_status bi_host_mulfull_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                              uint32_t m, uint64_t n);
/* Returns BI_EDIV0 (after computing every other instance) if any divisor  */
/* was zero; status may be NULL.                                           */
bi_status bi_host_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* q,
                          uint64_t* r, uint8_t* status, uint32_t mu, uint32_t mv,
                          uint64_t n);
bi_status bi_host_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* q,
                          uint32_t* r, uint8_t* status, uint32_t mu, uint32_t mv,
                          uint64_t n);
bi_status bi_host_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                          uint32_t m, uint64_t n);
bi_status bi_host_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                          uint32_t m, uint64_t n);
bi_status bi_host_sub_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                          uint8_t* sign, uint32_t m, uint64_t n);
bi_status bi_host_sub_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                          uint8_t* sign, uint32_t m, uint64_t n);

/* ---------------------------------------------------------------------- */
/* Fused chains: the reference's second benchmark type, consecutive       */
/* operations in one kernel with intermediates kept on chip               */
/* (thesis/sections/performance.tex:28-36).  p >= 1.                       */
/*  - add chain = baddKer1Bench<..., p> (cuda/ker-add.cu.h:88-112), the    */
/*    thesis's 10(u+v): r1 = a + b, then p-1 times r = r1 + r, i.e.        */
/*    r = p (a + b) mod B^m; sizes that are not a multiple of 64 bytes     */
/*    (or unaligned buffers) run as separate launches, r not aliasing a/b; */
/*  - mul chain = convMul*Bench<..., p> (cuda/ker-mul.cu.h:223-250,        */
/*    668-695): r1 = a b, then p-1 times r = r1 r, all truncated to m      */
/*    limbs, i.e. r = (a b)^p mod B^m.                                     */
/* ---------------------------------------------------------------------- */
bi_status bi_add_chain_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                           uint32_t m, uint64_t n, uint32_t p, bi_stream stream);
bi_status bi_add_chain_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                           uint32_t m, uint64_t n, uint32_t p, bi_stream stream);
bi_status bi_mul_chain_u64(const uint64_t* a, const uint64_t* b, uint64_t* r,
                           uint32_t m, uint64_t n, uint32_t p, bi_stream stream);
bi_status bi_mul_chain_u32(const uint32_t* a, const uint32_t* b, uint32_t* r,
                           uint32_t m, uint64_t n, uint32_t p, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* The division prototype's helper primitives as batched device ops       */
/* (prototypes/div.c:49-202; Futhark forms futhark/helper.fut:83-124,     */
/* futhark/div.fut:21-69), over [n][m] limbs:                              */
/*  bi_cmp:   out[i] = -1, 0, 1 as a_i <, ==, > b_i (lt, eq, :49-62);      */
/*  bi_findk: k[i] = index of a_i's top nonzero limb, 0 for zero (findk,   */
/*            :92-96; prec = k + 1), zero[i] = (a_i == 0) (ez, :64-69);    */
/*            either output may be NULL;                                   */
/*  bi_shift: shift by whole limbs (shift, :104-117): digits >= 0 gives    */
/*            r_i = a_i * B^digits mod B^m, digits < 0 r_i = a_i / B^-digits;*/
/*            r must not alias a;                                          */
/*  bi_muld:  r_i = a_i * d_i mod B^m with one limb d_i (multd, :197-217);  */
/*  bi_quod:  q_i = floor(a_i / d_i), rem_i = a_i mod d_i (rem may be NULL)*/
/*            with one limb d_i (quod, :165-181); d_i = 0 gives 0 and 0;   */
/*            q must not alias a.                                          */
/* ---------------------------------------------------------------------- */
bi_status bi_cmp_u64(const uint64_t* a, const uint64_t* b, int8_t* out,
                     uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_cmp_u32(const uint32_t* a, const uint32_t* b, int8_t* out,
                     uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_findk_u64(const uint64_t* a, uint32_t* k, uint8_t* zero,
                       uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_findk_u32(const uint32_t* a, uint32_t* k, uint8_t* zero,
                       uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_shift_u64(const uint64_t* a, uint64_t* r, int32_t digits,
                       uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_shift_u32(const uint32_t* a, uint32_t* r, int32_t digits,
                       uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_muld_u64(const uint64_t* a, const uint64_t* d, uint64_t* r,
                      uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_muld_u32(const uint32_t* a, const uint32_t* d, uint32_t* r,
                      uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_quod_u64(const uint64_t* a, const uint64_t* d, uint64_t* q,
                      uint64_t* rem, uint32_t m, uint64_t n, bi_stream stream);
bi_status bi_quod_u32(const uint32_t* a, const uint32_t* d, uint32_t* q,
                      uint32_t* rem, uint32_t m, uint64_t n, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* The Futhark library's shape-agnostic entries on one integer of m limbs */
/* (futhark/test/gmp-validation-lib.fut:13-27), host pointers:            */
/* test_add = (u + v) mod B^m, test_sub = |u - v|, test_mul = (u v) mod   */
/* B^m, test_div = floor(u / v) (v = 0: BI_EDIV0 and w = 0).              */
/* ---------------------------------------------------------------------- */
bi_status bi_test_add_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m);
bi_status bi_test_add_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m);
bi_status bi_test_sub_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m);
bi_status bi_test_sub_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m);
bi_status bi_test_mul_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m);
bi_status bi_test_mul_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m);
bi_status bi_test_div_u64(const uint64_t* u, const uint64_t* v, uint64_t* w, uint32_t m);
bi_status bi_test_div_u32(const uint32_t* u, const uint32_t* v, uint32_t* w, uint32_t m);

/* ---------------------------------------------------------------------- */
/* GMP word arrays.  The reference moves integers in and out of GMP with  */
/* mpz_import / mpz_export in order -1 (least significant word first),    */
/* native byte order (cuda/helpers.h:161-187, gmp-validation.c:30-52).    */
/* bi_limbs_from_words reads `count` words of `size` bytes (1, 2, 4 or 8) */
/* in that order into m 64-bit limbs (zero-extended; BI_EINVAL if the     */
/* value needs more than m limbs); bi_limbs_to_words writes the value of  */
/* m limbs as words of `size` bytes, least significant first, without    */
/* leading zero words (*count = words written, 0 for zero), as mpz_export */
/* does; `words` must hold ceil(m * 8 / size) words.  Host only.          */
/* ---------------------------------------------------------------------- */
bi_status bi_limbs_from_words(const void* words, size_t count, size_t size,
                              uint64_t* limbs, uint32_t m);
bi_status bi_limbs_to_words(const uint64_t* limbs, uint32_t m, size_t size,
                            void* words, size_t* count);

/* ---------------------------------------------------------------------- */
/* Uneven batches: instances of different operations and sizes in one      */
/* graph-captured launch.  The reference launches one template-specialised */
/* kernel per (operation, size) (cuda/main.cu:476-515); a plan instead     */
/* buckets the descriptors once and runs persistent add/sub, multiply and  */
/* divide kernels concurrently from one CUDA graph.  64-bit limbs only.    */
/* ---------------------------------------------------------------------- */
#define BI_OP_ADD      0u   /* r = (a + b) mod B^m                         */
#define BI_OP_SUB      1u   /* r = |a - b|, flags[flag] = (a < b)          */
#define BI_OP_MUL      2u   /* r = (a * b) mod B^m                         */
#define BI_OP_MULFULL  3u   /* r = a * b, 2m limbs                         */
#define BI_OP_DIV      4u   /* r = a / b (m limbs), r2 = a mod b (mb       */
                            /* limbs), flags[flag] = status as bi_div_u64  */

typedef struct bi_desc {
    uint32_t op;        /* BI_OP_* */
    uint32_t m;         /* elements of a (the dividend for BI_OP_DIV) */
    uint32_t mb;        /* elements of b for BI_OP_DIV (1 <= mb <= m); else ignored (= m) */
    uint32_t width;     /* element width: 0 or 64 = 64-bit limbs; 32 = 32-bit words */
    uint64_t a, b;      /* element offsets of the operands in the input arena */
    uint64_t r, r2;     /* element offsets of the results in the output arena */
    uint64_t flag;      /* byte offset of the sign / status in the flag arena */
} bi_desc;
/* With width = 32 the instance is the reference's U32bits layout: m, mb   */
/* and the offsets count 32-bit words of the same arenas (word k of an     */
/* arena of 64-bit limbs is the low half of limb k/2 for even k), so a    */
/* batch can mix 32-bit-word and 64-bit-limb instances.  Size limits are  */
/* the same in bits: twice as many words as limbs.                        */

typedef struct bi_plan bi_plan;

/* Build a plan from host descriptors (m <= 2048 for add, sub and the     */
/* multiplies; a division's dividend m <= 8192 and divisor mb <= 4096).    */
/* in_limbs, out_limbs: limbs of the input and output arenas the plan     */
/* will run on; nflags: bytes of its flag arena (0: no flag arena, and    */
/* bi_plan_execute then takes flags = NULL).  Every operand, result and    */
/* flag a descriptor names must lie inside its arena, else BI_EINVAL       */
/* before anything is allocated.  Allocates device work lists; the plan is */
/* bound to the current device.                                            */
bi_status bi_plan_create(bi_plan** plan, const bi_desc* descs, uint64_t count,
                         uint64_t in_limbs, uint64_t out_limbs, uint64_t nflags);
/* Run the plan: in/out are device arenas (16-byte aligned) of at least    */
/* the sizes the plan was built for, flags may be NULL.  The first call    */
/* (and any call with other arenas or tuning)                              */
/* captures the CUDA graph; later calls replay it on `stream`.  Calls on    */
/* one plan are serialised; its launches must not overlap on the device.   */
bi_status bi_plan_execute(bi_plan* plan, const uint64_t* in, uint64_t* out,
                          uint8_t* flags, bi_stream stream);
/* Time candidate configurations on this plan's data (each as a run of   */
/* the whole plan, its kernels sharing the GPU) and keep the fastest:      */
/* add/sub rows per step (2/4/8 x 16 bytes per lane) and limb width per    */
/* lane (8 or 16 bytes), multiply instances per CTA (default / 2 / 4),    */
/* and the word width of the arithmetic for full products of at most 32   */
/* limbs (32-bit words on the warp kernel, 64-bit limbs on the CTA        */
/* kernel).  chosen (may be NULL) receives {rows, limbs per lane, ipc     */
/* divisor}; bi_plan_get_tuning returns all four choices.                 */
bi_status bi_plan_autotune(bi_plan* plan, const uint64_t* in, uint64_t* out,
                           uint8_t* flags, int reps, int* chosen);
bi_status bi_plan_set_tuning(bi_plan* plan, int addsub_rows, int addsub_vec,
                             int mul_ipc_div);
/* Full products of at most 32 limbs computed on 32-bit words (bits = 32,   */
/* the warp kernel; the default) or 64-bit limbs (bits = 64, the CTA       */
/* kernel with the rest).                                                  */
bi_status bi_plan_set_mul_word_bits(bi_plan* plan, int bits);
/* tuning[0..3] = add/sub rows, limbs per lane, multiply ipc divisor,      */
/* word bits of the small full products.                                   */
bi_status bi_plan_get_tuning(bi_plan* plan, int* tuning);
/* stats[0..5] = add/sub instances, multiply instances, multiply items,    */
/* divisions, multiply and divide shared-memory bytes per CTA.             */
bi_status bi_plan_stats(const bi_plan* plan, uint64_t* stats);
bi_status bi_plan_destroy(bi_plan* plan);

/* ---------------------------------------------------------------------- */
/* Uneven batch that allocates nothing.  No counterpart in the reference.  */
/* For callers that cannot allocate device memory where they need a batch  */
/* run (an allocator that forbids cudaMalloc, a callback that must not     */
/* allocate): the scratch that bi_plan_create allocates -- a copy of the   */
/* descriptors, the work lists and the work counters -- lives instead in a */
/* fixed device array owned by the library (about 344 KB, held on every    */
/* GPU that loads the library until the process exits).  At most          */
/* bi_batch_noalloc_max_descs() descriptors (4096) per call; larger counts */
/* are rejected with BI_EINVAL, and so is any descriptor whose operands,   */
/* results or flag leave the arenas (in_limbs, out_limbs limbs; nflags     */
/* bytes, 0 when flags is NULL).  Same descriptors, arenas and results as  */
/* bi_plan_execute; descs is host memory.  Each call looks up the array's  */
/* device address on the current device, stages its lists from host       */
/* memory and returns when its work on `stream` has finished; a stream     */
/* that is being captured is refused with BI_EUNSUPPORTED before anything */
/* is enqueued.  Every call shares the one array: calls that overlap on    */
/* the GPU race, so issue them one after another.                          */
/* ---------------------------------------------------------------------- */
uint32_t bi_batch_noalloc_max_descs(void);
bi_status bi_batch_run_noalloc(const bi_desc* descs, uint64_t count,
                               const uint64_t* in, uint64_t in_limbs,
                               uint64_t* out, uint64_t out_limbs,
                               uint8_t* flags, uint64_t nflags, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* Serving loop: requests of any operation and size, submitted one at a    */
/* time, run by a persistent device-resident kernel with continuous        */
/* batching.  No counterpart in the reference (its benchmarks launch fixed */
/* batches, cuda/main.cu:476-515).  A request is a bi_desc over the        */
/* server's operand arena `in` (device, 16-byte aligned); the server fills */
/* in r, r2 (offsets of the results in its output arena, in the request's */
/* elements) and ignores flag.  A request's width says whether m, mb and  */
/* the offsets count 64-bit limbs or 32-bit words; m in 64-bit limbs <=   */
/* max_limbs for every op (the dividend for BI_OP_DIV, divisor 1 <= mb <= */
/* m).                                                                     */
/*                                                                         */
/* Admission: a request enters when one of ring_slots slots and room for   */
/* its results in the output arena (the HBM budget) are free; otherwise    */
/* bi_server_submit returns BI_EBUSY and the caller polls, releases and    */
/* retries.  Slots and arena space are reclaimed in submission order as    */
/* requests are released.  The loop's CTAs leave after idle_us without a   */
/* request and the next submit or poll relaunches it.  One client thread   */
/* per server.  Results stay valid in the arena until released.            */
/* ---------------------------------------------------------------------- */
typedef struct bi_server bi_server;

typedef struct bi_completion {
    uint64_t ticket;    /* request number returned by bi_server_submit */
    uint64_t r, r2;     /* limb offsets of the result(s) in the output arena */
    uint32_t status;    /* sub: 1 if a < b; div: as bi_div_u64; 255: lost */
    uint32_t op;
} bi_completion;

typedef struct bi_serve_report {
    double requests;      /* requests completed */
    double launches;      /* kernel launches: loop (re)starts, or one per request */
    double busy;          /* admissions deferred for want of a slot or arena room */
    double duration_s;    /* replay start to the last completion seen */
    double offered_rps;   /* requests / last arrival time */
    double achieved_rps;  /* requests / duration_s */
    double p50_us, p90_us, p99_us, p999_us, max_us, mean_us;  /* arrival -> completion seen */
} bi_serve_report;

/* out == NULL: the server allocates an arena of out_limbs limbs (0: an    */
/* eighth of the free HBM, at most 2^28 limbs).  ring_slots: power of two  */
/* (0: 65536); max_limbs (0: 512, at most 2048) sizes the shared memory;   */
/* ctas (0: as many as are resident at once); idle_us (0: 2000).           */
bi_status bi_server_create(bi_server** server, const uint64_t* in, uint64_t in_limbs,
                           uint64_t* out, uint64_t out_limbs, uint32_t ring_slots,
                           uint32_t max_limbs, uint32_t ctas, uint32_t idle_us);
bi_status bi_server_submit(bi_server* server, const bi_desc* request, uint64_t* ticket);
/* Collect up to max completions (in completion order) into out.           */
bi_status bi_server_poll(bi_server* server, bi_completion* out, uint32_t max, uint32_t* count);
/* Return a completed request's slot and arena space.                      */
bi_status bi_server_release(bi_server* server, uint64_t ticket);
/* info[0..9] = arena pointer, arena limbs, CTAs, shared bytes per CTA,    */
/* launches, deferred admissions, lost requests, ring slots, submitted,    */
/* completed.                                                              */
bi_status bi_server_info(const bi_server* server, uint64_t* info);
/* Failure injection on the host: publish one ring slot whose contents are */
/* never written, as if the host's write had been lost.  The CTA that     */
/* claims it waits (at most one second) for the slot's sequence number,   */
/* gives up and completes it with status 255; the other requests go on.   */
/* The ticket is released like any other.                                 */
bi_status bi_server_inject_dropped(bi_server* server, uint64_t* ticket);
/* Stops the loop and frees the server.  A running loop first finishes     */
/* every request already submitted; requests submitted after the loop     */
/* ended without a poll or submit to relaunch it are dropped.             */
bi_status bi_server_destroy(bi_server* server);

/* Open-loop replay on an idle server: request i arrives arrival_ns[i] ns  */
/* after the start (non-decreasing), is admitted when it can be, and is    */
/* released once its completion is seen; latency_ns[i] = completion seen - */
/* arrival.  done (may be NULL) receives each request's completion.        */
bi_status bi_server_replay(bi_server* server, const bi_desc* requests,
                           const uint64_t* arrival_ns, uint64_t n, uint64_t* latency_ns,
                           bi_completion* done, bi_serve_report* report);
/* The same stream with one library launch per request (bi_add_u64, ...,  */
/* bi_div_u64 with n = 1) round-robin over `streams` streams, each result  */
/* placed in `out` in arrival order; completion seen by event query.        */
bi_status bi_serve_replay_plain(const uint64_t* in, uint64_t* out, uint64_t out_limbs,
                                const bi_desc* requests, const uint64_t* arrival_ns,
                                uint64_t n, uint32_t streams, uint64_t* latency_ns,
                                bi_completion* done, bi_serve_report* report);

/* ---------------------------------------------------------------------- */
/* Synthetic inputs: dst[i] = splitmix64 output number offset+i+1 of the   */
/* stream `seed`.  No counterpart in the reference, whose benchmarks draw  */
/* unseeded rand() digits (cuda/helpers.h:96-111); this makes multi-GiB    */
/* benchmark inputs reproducible and cheap to create on the device.        */
/* ---------------------------------------------------------------------- */
bi_status bi_fill_splitmix64(uint64_t* dst, uint64_t count, uint64_t seed,
                             uint64_t offset, bi_stream stream);

/* ---------------------------------------------------------------------- */
/* Integer-pipe probe: rates[0..5] = 32x32-bit word products per second    */
/* the GPU sustains with (0) mad.lo.u32, (1) mad.hi.u32, (2) mad.wide.u32, */
/* (3) mad.lo.cc/madc.hi.cc carry-chain rows, (4) mul.lo/hi.u64, (5)       */
/* mad.wide.u32 accumulating 64-bit column sums.  The                      */
/* multiply roofline's denominator; no counterpart in the reference.       */
/* Synchronous on `stream`.                                                */
/* ---------------------------------------------------------------------- */
bi_status bi_probe_intpipe(double* rates, bi_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* BIGINT_GB300_H */
