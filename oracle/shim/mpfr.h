/*
 * Declaration shim for the documented MPFR 4.x C API.
 *
 * This image ships the MPFR/GMP runtime libraries (libmpfr.so.6,
 * libgmp.so.10) but not their development headers.  The reference renderer
 * (renderer.cpp, built with -DFRACTAL_HAVE_MPFR) only needs the public types
 * and the prototypes of the functions it calls; this file declares exactly
 * those, following the layout documented in the MPFR manual (section
 * "Nomenclature and Types" / "Internals": precision, sign, exponent, limb
 * pointer).  Every declared name is an exported symbol of libmpfr.so.6.
 *
 * Test infrastructure only: it exists so the reference can be compiled as
 * the oracle.  The product library declares the few MPFR entry points it
 * uses on its own and loads them with dlopen.
 */
#ifndef ORACLE_SHIM_MPFR_H
#define ORACLE_SHIM_MPFR_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;
typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;

typedef struct {
    mpfr_prec_t _mpfr_prec;
    mpfr_sign_t _mpfr_sign;
    mpfr_exp_t _mpfr_exp;
    mp_limb_t *_mpfr_d;
} __mpfr_struct;

typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct *mpfr_ptr;
typedef const __mpfr_struct *mpfr_srcptr;

typedef enum {
    MPFR_RNDN = 0,
    MPFR_RNDZ,
    MPFR_RNDU,
    MPFR_RNDD,
    MPFR_RNDA,
    MPFR_RNDF,
    MPFR_RNDNA = -1
} mpfr_rnd_t;

void mpfr_init2(mpfr_ptr, mpfr_prec_t);
void mpfr_clear(mpfr_ptr);
void mpfr_clears(mpfr_ptr, ...);
int mpfr_set_str(mpfr_ptr, const char *, int, mpfr_rnd_t);
int mpfr_set(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_set_d(mpfr_ptr, double, mpfr_rnd_t);
int mpfr_set_ui(mpfr_ptr, unsigned long, mpfr_rnd_t);
void mpfr_set_zero(mpfr_ptr, int);
int mpfr_mul(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_add(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sub(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_div(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sqrt(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_neg(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_abs(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_add_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_ui_sub(mpfr_ptr, unsigned long, mpfr_srcptr, mpfr_rnd_t);
int mpfr_div_2ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_mul_2si(mpfr_ptr, mpfr_srcptr, long, mpfr_rnd_t);
int mpfr_pow_si(mpfr_ptr, mpfr_srcptr, long, mpfr_rnd_t);
int mpfr_log(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_log10(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sgn(mpfr_srcptr);
int mpfr_number_p(mpfr_srcptr);
int mpfr_cmp(mpfr_srcptr, mpfr_srcptr);
int mpfr_cmp_ui(mpfr_srcptr, unsigned long);
int mpfr_cmp_d(mpfr_srcptr, double);
double mpfr_get_d(mpfr_srcptr, mpfr_rnd_t);
long double mpfr_get_ld(mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d_2exp(long *, mpfr_srcptr, mpfr_rnd_t);

#ifdef __cplusplus
}
#endif

#endif
