/*
 * Test infrastructure only: declarations of the documented GMP mpz API used by
 * the reference sources, so they can be compiled and linked against the
 * runtime-only libgmp.so.10 (GMP 6.3.x ABI) that the build host ships without
 * headers.  Only names and signatures from the public GMP manual are declared.
 */
#pragma once
#include <stddef.h>
#include <stdio.h>

#define __GNU_MP_VERSION 6
#define __GNU_MP_VERSION_MINOR 3
#define __GNU_MP_VERSION_PATCHLEVEL 0

typedef unsigned long mp_limb_t;
typedef struct {
    int _mp_alloc;
    int _mp_size;
    mp_limb_t *_mp_d;
} __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;

#ifdef __cplusplus
extern "C" {
#endif
void __gmpz_init(mpz_ptr);
void __gmpz_inits(mpz_ptr, ...);
void __gmpz_clear(mpz_ptr);
void __gmpz_clears(mpz_ptr, ...);
void __gmpz_set(mpz_ptr, mpz_srcptr);
void __gmpz_set_ui(mpz_ptr, unsigned long);
unsigned long __gmpz_get_ui(mpz_srcptr);
double __gmpz_get_d_2exp(long *, mpz_srcptr);
void __gmpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_sub_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mod(mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long __gmpz_fdiv_ui(mpz_srcptr, unsigned long);
unsigned long __gmpz_fdiv_r_ui(mpz_ptr, mpz_srcptr, unsigned long);
unsigned long __gmpz_cdiv_ui(mpz_srcptr, unsigned long);
unsigned long __gmpz_tdiv_q_ui(mpz_ptr, mpz_srcptr, unsigned long);
unsigned long __gmpz_gcd_ui(mpz_ptr, mpz_srcptr, unsigned long);
int __gmpz_invert(mpz_ptr, mpz_srcptr, mpz_srcptr);
int __gmpz_cmp_ui(mpz_srcptr, unsigned long);
size_t __gmpz_sizeinbase(mpz_srcptr, int);
void __gmpz_primorial_ui(mpz_ptr, unsigned long);
void __gmpz_ui_pow_ui(mpz_ptr, unsigned long, unsigned long);
void __gmpz_nextprime(mpz_ptr, mpz_srcptr);
int __gmpz_prevprime(mpz_ptr, mpz_srcptr);
int __gmpz_probab_prime_p(mpz_srcptr, int);
#ifdef __cplusplus
}
#endif

#define mpz_init __gmpz_init
#define mpz_inits __gmpz_inits
#define mpz_clear __gmpz_clear
#define mpz_clears __gmpz_clears
#define mpz_set __gmpz_set
#define mpz_set_ui __gmpz_set_ui
#define mpz_get_ui __gmpz_get_ui
#define mpz_get_d_2exp __gmpz_get_d_2exp
#define mpz_add_ui __gmpz_add_ui
#define mpz_sub_ui __gmpz_sub_ui
#define mpz_sub __gmpz_sub
#define mpz_mul __gmpz_mul
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_mod __gmpz_mod
#define mpz_fdiv_ui __gmpz_fdiv_ui
#define mpz_fdiv_r_ui __gmpz_fdiv_r_ui
#define mpz_mod_ui __gmpz_fdiv_r_ui
#define mpz_cdiv_ui __gmpz_cdiv_ui
#define mpz_tdiv_q_ui __gmpz_tdiv_q_ui
#define mpz_gcd_ui __gmpz_gcd_ui
#define mpz_invert __gmpz_invert
#define mpz_cmp_ui __gmpz_cmp_ui
#define mpz_sizeinbase __gmpz_sizeinbase
#define mpz_primorial_ui __gmpz_primorial_ui
#define mpz_ui_pow_ui __gmpz_ui_pow_ui
#define mpz_nextprime __gmpz_nextprime
#define mpz_prevprime __gmpz_prevprime
#define mpz_probab_prime_p __gmpz_probab_prime_p
#define mpz_odd_p(z) ((z)->_mp_size != 0 && ((z)->_mp_d[0] & 1))
#define mpz_even_p(z) (!mpz_odd_p(z))
