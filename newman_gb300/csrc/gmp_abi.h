// Declarations of the documented GMP floating-point (mpf) C API, for linking
// against the runtime library libgmp.so.10 (GMP 6.x) when the development
// headers are not installed.
//
// Only names, signatures and the public struct layout documented in the GMP
// manual ("Floating-point Functions", "Internals / Float Internals") appear
// here.  The layout is the LP64 one (x86_64 and aarch64 Linux): a limb is an
// unsigned long and an exponent is a long.
#pragma once

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;
typedef long mp_exp_t;
typedef unsigned long mp_bitcnt_t;

typedef struct {
  int _mp_prec;       // limbs of precision (not counting the extra one)
  int _mp_size;       // signed limb count of the mantissa
  mp_exp_t _mp_exp;   // exponent in limbs
  mp_limb_t* _mp_d;   // limb array, least significant first
} __mpf_struct;

typedef __mpf_struct mpf_t[1];
typedef __mpf_struct* mpf_ptr;
typedef const __mpf_struct* mpf_srcptr;

void __gmpf_init2(mpf_ptr, mp_bitcnt_t);
void __gmpf_clear(mpf_ptr);
void __gmpf_set(mpf_ptr, mpf_srcptr);
void __gmpf_set_d(mpf_ptr, double);
void __gmpf_set_si(mpf_ptr, long);
void __gmpf_set_ui(mpf_ptr, unsigned long);
int __gmpf_set_str(mpf_ptr, const char*, int);
void __gmpf_set_prec(mpf_ptr, mp_bitcnt_t);
mp_bitcnt_t __gmpf_get_prec(mpf_srcptr);
void __gmpf_set_default_prec(mp_bitcnt_t);
double __gmpf_get_d(mpf_srcptr);
double __gmpf_get_d_2exp(long*, mpf_srcptr);
char* __gmpf_get_str(char*, mp_exp_t*, int, size_t, mpf_srcptr);
void __gmpf_add(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_sub(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul_ui(mpf_ptr, mpf_srcptr, unsigned long);
void __gmpf_mul_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
void __gmpf_div_ui(mpf_ptr, mpf_srcptr, unsigned long);
void __gmpf_div_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
void __gmpf_div(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_neg(mpf_ptr, mpf_srcptr);
void __gmpf_abs(mpf_ptr, mpf_srcptr);
int __gmpf_cmp(mpf_srcptr, mpf_srcptr);
int __gmpf_cmp_d(mpf_srcptr, double);

#ifdef __cplusplus
}
#endif

#define mpf_init2 __gmpf_init2
#define mpf_clear __gmpf_clear
#define mpf_set __gmpf_set
#define mpf_set_d __gmpf_set_d
#define mpf_set_si __gmpf_set_si
#define mpf_set_ui __gmpf_set_ui
#define mpf_set_str __gmpf_set_str
#define mpf_set_prec __gmpf_set_prec
#define mpf_get_prec __gmpf_get_prec
#define mpf_set_default_prec __gmpf_set_default_prec
#define mpf_get_d __gmpf_get_d
#define mpf_get_d_2exp __gmpf_get_d_2exp
#define mpf_get_str __gmpf_get_str
#define mpf_add __gmpf_add
#define mpf_sub __gmpf_sub
#define mpf_mul __gmpf_mul
#define mpf_mul_ui __gmpf_mul_ui
#define mpf_mul_2exp __gmpf_mul_2exp
#define mpf_div_ui __gmpf_div_ui
#define mpf_div_2exp __gmpf_div_2exp
#define mpf_div __gmpf_div
#define mpf_neg __gmpf_neg
#define mpf_abs __gmpf_abs
#define mpf_cmp __gmpf_cmp
#define mpf_cmp_d __gmpf_cmp_d

// mpf_sgn is a macro in GMP's header; restated from the documented layout.
static inline int mpf_sgn_(mpf_srcptr f) { return f->_mp_size < 0 ? -1 : (f->_mp_size > 0); }
