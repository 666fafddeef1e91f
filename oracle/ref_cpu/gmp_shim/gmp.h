/*
 * The subset of GMP's C interface that the reference's host code calls,
 * declared for this project from GMP's documented API (GMP 6 manual, "Integer
 * Functions" and "Rational Number Functions") and its documented object
 * layouts, so that the reference's host sources compile in a container that
 * has the shared library libgmp.so.10 but not its development headers.
 * CHECKER INFRASTRUCTURE ONLY: used by oracle/ref_cpu/build_mock.py to build
 * the reference's host mock backend; nothing in the product includes it.
 * The library exports its functions as __gmpz_* / __gmpq_*; the documented
 * names are inline forwards to them.
 */
#ifndef RPG_GMP_SHIM_H
#define RPG_GMP_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t; /* 64-bit limbs on the LP64 hosts this project runs on */
typedef struct {
    int _mp_alloc;
    int _mp_size;
    mp_limb_t *_mp_d;
} __mpz_struct;
typedef struct {
    __mpz_struct _mp_num;
    __mpz_struct _mp_den;
} __mpq_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpq_struct mpq_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;
typedef __mpq_struct *mpq_ptr;
typedef const __mpq_struct *mpq_srcptr;

void __gmpz_init(mpz_ptr);
void __gmpz_init_set(mpz_ptr, mpz_srcptr);
void __gmpz_init_set_si(mpz_ptr, long);
int __gmpz_init_set_str(mpz_ptr, const char *, int);
void __gmpz_clear(mpz_ptr);
void __gmpz_set(mpz_ptr, mpz_srcptr);
void __gmpz_set_si(mpz_ptr, long);
int __gmpz_set_str(mpz_ptr, const char *, int);
void __gmpz_swap(mpz_ptr, mpz_ptr);
void __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul_si(mpz_ptr, mpz_srcptr, long);
void __gmpz_neg(mpz_ptr, mpz_srcptr);
int __gmpz_cmp(mpz_srcptr, mpz_srcptr);
int __gmpz_cmp_si(mpz_srcptr, long);
char *__gmpz_get_str(char *, int, mpz_srcptr);
void __gmpz_ui_pow_ui(mpz_ptr, unsigned long, unsigned long);
int __gmpz_perfect_square_p(mpz_srcptr);
void __gmpz_sqrt(mpz_ptr, mpz_srcptr);

void __gmpq_init(mpq_ptr);
void __gmpq_clear(mpq_ptr);
void __gmpq_set(mpq_ptr, mpq_srcptr);
void __gmpq_set_z(mpq_ptr, mpz_srcptr);
void __gmpq_set_si(mpq_ptr, long, unsigned long);
int __gmpq_set_str(mpq_ptr, const char *, int);
void __gmpq_swap(mpq_ptr, mpq_ptr);
void __gmpq_canonicalize(mpq_ptr);
void __gmpq_add(mpq_ptr, mpq_srcptr, mpq_srcptr);
void __gmpq_sub(mpq_ptr, mpq_srcptr, mpq_srcptr);
void __gmpq_mul(mpq_ptr, mpq_srcptr, mpq_srcptr);
void __gmpq_div(mpq_ptr, mpq_srcptr, mpq_srcptr);
int __gmpq_cmp(mpq_srcptr, mpq_srcptr);
int __gmpq_cmp_si(mpq_srcptr, long, unsigned long);

static inline void mpz_ui_pow_ui(mpz_ptr r, unsigned long b, unsigned long e) { __gmpz_ui_pow_ui(r, b, e); }
static inline void mpz_mul_si(mpz_ptr r, mpz_srcptr a, long b) { __gmpz_mul_si(r, a, b); }
static inline int mpz_perfect_square_p(mpz_srcptr a) { return __gmpz_perfect_square_p(a); }
static inline void mpz_sqrt(mpz_ptr r, mpz_srcptr a) { __gmpz_sqrt(r, a); }

#ifdef __cplusplus
}
#endif

#endif
