/*
 * Minimal declarations of the public GMP mpz ABI, used only to compile the
 * reference's CPU prototype (prototypes/div.c) against the runtime-only
 * libgmp.so.10 present on this image (it ships no gmp.h).  Test
 * infrastructure: nothing in the library includes this file.
 */
#ifndef ORACLE_GMP_SHIM_H
#define ORACLE_GMP_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { int _mp_alloc; int _mp_size; void* _mp_d; } __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;

void  __gmpz_init(mpz_ptr);
void  __gmpz_clear(mpz_ptr);
void  __gmpz_import(mpz_ptr, size_t, int, size_t, int, size_t, const void*);
void* __gmpz_export(void*, size_t*, int, size_t, int, size_t, mpz_srcptr);
void  __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void  __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void  __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void  __gmpz_fdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
void  __gmpz_tdiv_qr(mpz_ptr, mpz_ptr, mpz_srcptr, mpz_srcptr);
void  __gmpz_abs(mpz_ptr, mpz_srcptr);

#define mpz_init    __gmpz_init
#define mpz_clear   __gmpz_clear
#define mpz_import  __gmpz_import
#define mpz_export  __gmpz_export
#define mpz_add     __gmpz_add
#define mpz_sub     __gmpz_sub
#define mpz_mul     __gmpz_mul
#define mpz_div     __gmpz_fdiv_q
#define mpz_fdiv_q  __gmpz_fdiv_q
#define mpz_tdiv_qr __gmpz_tdiv_qr
#define mpz_abs     __gmpz_abs
#ifdef __cplusplus
}
#endif
#endif
