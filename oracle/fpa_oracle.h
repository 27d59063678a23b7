/*
 * fpa_oracle.h -- CPU oracle for the fpa add/sub/mul/div/sqrt path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the semantics of
 * cuBigFloat's warp kernels (fpa_warp_add_sub.h, fpa_warp_mul.h, fpa_warp_div.h,
 * fpa_warp_sqrt.h, fpa_internal.h) computed with exact integer arithmetic.  It is
 * used by the tests as the checker, by smoke() as the checker and by bench.py as
 * the timed CPU baseline.  The product library never links or calls it.
 *
 * Encoding (fpa_internal.h:1-17, tests.c:114-159):
 *   exp word 0..8  : classes (ZERO=2, NEG_TINY=3, POS_TINY=4, NEG_INF=5, POS_INF=6,
 *                    NAN=7, SNAN=8)
 *   exp word >= 9  : bit 0 = sign, bits 31..1 = BIAS + e, BIAS = 0x3FFFFFF3
 *   mantissa       : n little-endian 32-bit limbs, top bit of limb n-1 set;
 *                    value = (-1)^sign * M * 2^(e - 32n)
 * Special results leave the result limbs untouched, as the reference does.
 */
#ifndef FPA_ORACLE_H
#define FPA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_ADD = 0, ORACLE_SUB = 1, ORACLE_MUL = 2, ORACLE_DIV = 3, ORACLE_SQRT = 4 };

/* One operation on one instance.  n = limbs (precision/32), mode = fpa_rounding_mode.
 * b_exp/b_limbs are ignored for sqrt.  Returns 0, or -1 for a bad op/mode/n. */
int oracle_op(int op, uint32_t n, int mode,
              uint32_t *r_exp, uint32_t *r_limbs,
              uint32_t a_exp, const uint32_t *a_limbs,
              uint32_t b_exp, const uint32_t *b_limbs);

/* Elementwise over `count` instances stored contiguously (exps[i], limbs[i*n..i*n+n)),
 * split over `threads` pthreads (threads<=1: run on the calling thread). */
/* r = RND(a*b + c), one rounding, for `count` instances (no counterpart in the reference;
 * special values: the mul table's class of the exact product combined with c by the add
 * table).  Returns 0, or -1 for a bad mode/n. */
int oracle_fma_batch(uint32_t n, int mode, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                     const uint32_t *a_exps, const uint32_t *a_limbs, const uint32_t *b_exps,
                     const uint32_t *b_limbs, const uint32_t *c_exps, const uint32_t *c_limbs);

int oracle_batch(int op, uint32_t n, int mode, uint32_t count,
                 uint32_t *r_exps, uint32_t *r_limbs,
                 const uint32_t *a_exps, const uint32_t *a_limbs,
                 const uint32_t *b_exps, const uint32_t *b_limbs,
                 int threads);

/* Heterogeneous batch: instance i has its own op, limb count and mode; operand i
 * starts at limb offset a_off[i] / b_off[i] / r_off[i] of the flat limb arrays. */
int oracle_mixed(uint32_t count, const uint8_t *ops, const uint16_t *limbs_n, const uint8_t *modes,
                 uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *r_off,
                 const uint32_t *a_exps, const uint32_t *a_limbs, const uint64_t *a_off,
                 const uint32_t *b_exps, const uint32_t *b_limbs, const uint64_t *b_off,
                 int threads);

/* Conversions into the format (fpa_set_ui/si/float/double; floats and doubles given as
 * their IEEE bit patterns), precision change (fpa_set, nx -> nr limbs, rounded in `mode`),
 * sign, compare and negation, each over `count` instances.  Return 0, or -1 for bad sizes. */
int oracle_set_ui(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *vals);
int oracle_set_si(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const int64_t *vals);
int oracle_set_float(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *bits);
int oracle_set_double(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint64_t *bits);
int oracle_set_prec(uint32_t nr, uint32_t nx, int mode, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs,
                    const uint32_t *x_exps, const uint32_t *x_limbs);
int oracle_sgn(uint32_t count, int32_t *r, const uint32_t *x_exps);
int oracle_cmp(uint32_t n, uint32_t count, int32_t *r, const uint32_t *a_exps, const uint32_t *a_limbs,
               const uint32_t *b_exps, const uint32_t *b_limbs);
int oracle_neg(uint32_t n, uint32_t count, uint32_t *r_exps, uint32_t *r_limbs, const uint32_t *a_exps,
               const uint32_t *a_limbs);

#ifdef __cplusplus
}
#endif

#endif
